"""Mesh planner checks on the CPU (no GPU): the lane groups of the regular
assembly kernel.

The regular kernel gives each warp one trial face and its 32 lanes one group of
test faces, and every lane adds its 3 x 3 block into shared-memory rows of its
face's vertices without atomics.  That is race-free only if the faces of one
group share no vertex, i.e. their tile-local rows are pairwise distinct.  The
planner (boundary-lab_gb300/csrc/bem_plan.cpp) is compiled here with a small
driver (tests/plan_check.cpp) and its layout checked: every face in exactly one
slot, rows distinct within a group and inside the tile, and the groups packed
close to the lower bound max(ceil(faces / 32), largest vertex valence) per tile.
"""

import shutil
import subprocess
from collections import defaultdict
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "boundary-lab_gb300" / "csrc"
meshes = pkg_module("meshes")


@pytest.fixture(scope="module")
def plan_tool(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("plan") / "plan_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", f"-I{CSRC}", str(ROOT / "tests" / "plan_check.cpp"),
                    str(CSRC / "bem_plan.cpp"), "-o", str(exe)], check=True, capture_output=True)
    return exe


def run_plan(tool, tmp_path, mesh, tile_faces=512):
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        np.array([mesh.n_vertices, len(mesh.faces)], np.int32).tofile(f)
        np.ascontiguousarray(mesh.vertices, np.float64).tofile(f)
        np.ascontiguousarray(mesh.faces, np.int32).tofile(f)
    out = subprocess.run([str(tool), str(path), str(tile_faces)], check=True, capture_output=True, text=True).stdout
    tiles = []
    for line in out.splitlines():
        w = line.split()
        if w[0] in ("npairs", "pair", "fext", "scat"):
            continue
        if w[0] == "tile":
            tiles.append({"rows": int(w[3]), "groups": int(w[5]), "slots": defaultdict(list)})
        elif w[0] == "slot":
            g, face, *loc = map(int, w[1:])
            tiles[-1]["slots"][g].append((face, loc))
    return tiles


def make_mesh(name, faces):
    if name == "sphere":
        return meshes.sphere_with_cap(0.1, 3, 30.0)
    if name == "seeded":
        return meshes.seeded_piston_mesh(faces, 7)
    return meshes.box_with_piston((0.3, 0.2, 0.25), faces, 0.05, "+z")


@pytest.mark.parametrize("name,faces,tile_faces", [
    ("sphere", 1280, 512),
    ("seeded", 3000, 512),
    ("box", 5000, 512),
    ("box", 10000, 512),
    ("box", 10000, 256),
])
def test_lane_groups_are_vertex_disjoint_and_dense(plan_tool, tmp_path, name, faces, tile_faces):
    mesh = make_mesh(name, faces)
    tiles = run_plan(plan_tool, tmp_path, mesh, tile_faces)
    seen = np.zeros(len(mesh.faces), dtype=int)
    total_groups = minimum = 0
    for t in tiles:
        n_tile = 0
        valence = defaultdict(int)
        for g, members in t["slots"].items():
            assert 1 <= len(members) <= 32
            rows = [r for _, loc in members for r in loc]
            assert len(set(rows)) == len(rows), f"group {g} shares a vertex row"
            assert all(0 <= r < t["rows"] for r in rows)
            for face, loc in members:
                seen[face] += 1
                for r in loc:
                    valence[r] += 1
            n_tile += len(members)
        total_groups += t["groups"]
        # lower bound: 32 faces per group, and the faces around one vertex in distinct groups
        minimum += max(-(-n_tile // 32), max(valence.values()))
    assert np.all(seen == 1), "every face in exactly one lane slot"
    # 512-face tiles (the production size) pack to within a group or so of the
    # bound; small tiles leave the packer fewer groups to trade faces between
    slack = max(1, len(tiles) // 10) if tile_faces >= 512 else int(0.15 * minimum)
    assert total_groups <= minimum + slack, (total_groups, minimum)


def test_singular_scatter_plan_keeps_the_pair_order(plan_tool, tmp_path):
    """The singular scatter runs one thread per target entry of the extended rows,
    adding that entry's contributions in pair order.  On random float32 blocks its
    sums must equal, bit for bit, those of the sequential walk it replaced (one
    thread per trial face: its pairs in order, rows of test vertex a, columns b),
    and every block element must land exactly once."""
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 900, 0.05, "+z")
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        np.array([mesh.n_vertices, len(mesh.faces)], np.int32).tofile(f)
        np.ascontiguousarray(mesh.vertices, np.float64).tofile(f)
        np.ascontiguousarray(mesh.faces, np.int32).tofile(f)
    out = subprocess.run([str(plan_tool), str(path), "128"], check=True, capture_output=True, text=True).stdout
    pairs, fext, scat, n_ext = [], [], [], 0
    for line in out.splitlines():
        w = line.split()
        if w[0] == "npairs":
            n_ext = int(w[3])
        elif w[0] == "pair":
            pairs.append((int(w[1]), int(w[2])))
        elif w[0] == "fext":
            fext.append(tuple(map(int, w[1:])))
        elif w[0] == "scat":
            scat.append((int(w[1]), int(w[2]), [int(x) for x in w[3:]]))
    nf = len(mesh.faces)
    rng = np.random.default_rng(0)
    blocks = rng.normal(size=12 * len(pairs)).astype(np.float32)
    base = rng.normal(size=(3 * nf, n_ext)).astype(np.float32)
    walk = base.copy()
    for k, (g, f) in enumerate(pairs):  # pairs are sorted by trial face
        for a in range(3):
            for b in range(3):
                walk[3 * g + b, fext[f][a]] = np.float32(walk[3 * g + b, fext[f][a]] + blocks[12 * k + 3 * a + b])
    planned = base.copy()
    used = np.zeros(12 * len(pairs), int)
    for col, row, srcs in scat:
        v = planned[col, row]
        for s in srcs:
            v = np.float32(v + blocks[s])
            used[s] += 1
        planned[col, row] = v
    assert np.array_equal(walk.view(np.int32), planned.view(np.int32))
    assert len({(c, r) for c, r, _ in scat}) == len(scat)
    assert np.all(used.reshape(-1, 12)[:, :9] == 1) and np.all(used.reshape(-1, 12)[:, 9:] == 0)


def _mesh_file(tmp_path, mesh):
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        np.array([mesh.n_vertices, len(mesh.faces)], np.int32).tofile(f)
        np.ascontiguousarray(mesh.vertices, np.float64).tofile(f)
        np.ascontiguousarray(mesh.faces, np.int32).tofile(f)
    return path


def test_plan_does_not_depend_on_the_thread_count(plan_tool, tmp_path):
    """The planner cuts its loops (face geometry, pair enumeration, lane packing,
    field-major copies, scatter plan) into contiguous slices on worker threads and
    joins them in slice order: the whole printed plan is the same for 1, 3 and 8
    threads (BEM_PLAN_THREADS) on a mesh large enough to be planned in parallel."""
    import os

    path = _mesh_file(tmp_path, meshes.box_with_piston((0.3, 0.2, 0.25), 5000, 0.05, "+z"))
    outs = []
    for t in ("1", "3", "8"):
        env = {**os.environ, "BEM_PLAN_THREADS": t}
        outs.append(subprocess.run([str(plan_tool), str(path), "512"], check=True, capture_output=True, text=True,
                                   env=env).stdout)
    assert outs[0] == outs[1] == outs[2]


def test_pair_radius_and_duffy_points(plan_tool, tmp_path):
    """The planner's pair radius (the interval of the singular remainder's
    Chebyshev expansion) is the largest distance between a vertex of a pair's test
    face and one of its trial face, the trial face reflected for image pairs; the
    Duffy point count is the sum of the pairs' rule sizes.  Checked against numpy
    on a half model planned with symmetry x, whose image pairs carry reflected
    trial faces."""
    mesh = meshes.fundamental_domain(meshes.box_with_piston((0.3, 0.2, 0.25), 2000, 0.05, "+z"), "x")
    out = subprocess.run([str(plan_tool), str(_mesh_file(tmp_path, mesh)), "512", "1"], check=True,
                         capture_output=True, text=True).stdout
    radius = points = None
    pairs = []
    for line in out.splitlines():
        w = line.split()
        if w[0] == "radius":
            radius, points = float(w[1]), int(w[3])
        elif w[0] == "pair":
            pairs.append(tuple(map(int, w[1:5])))
    assert pairs and radius is not None
    p = np.array(pairs)
    assert np.any(p[:, 2] == 1), "the half model has image pairs"
    v = np.asarray(mesh.vertices, np.float64)
    fc = np.asarray(mesh.faces)
    sx = np.where(p[:, 2] & 1, -1.0, 1.0)
    sy = np.where(p[:, 2] & 2, -1.0, 1.0)
    best = 0.0
    for a in range(3):
        t = v[fc[p[:, 1], a]]
        for b in range(3):
            q = v[fc[p[:, 0], b]]
            d = np.stack([sx * q[:, 0] - t[:, 0], sy * q[:, 1] - t[:, 1], q[:, 2] - t[:, 2]], 1)
            best = max(best, float(np.max(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])))
    assert radius == pytest.approx(np.sqrt(best), rel=1e-15)
    assert points == int(p[:, 3].sum())
