"""Pins of the CPU oracle (runs without a GPU).

The reference engine is Julia and cannot run here, and it ships no numeric
golden vectors for this path.  The oracle is therefore pinned against what the
reference does provide: its literal rule constants and fixture meshes (read
from its files into tests/golden by tests/golden/make_golden.py), the
relations its own tests assert, and analytic solutions.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module, reference_checkout

meshes = pkg_module("meshes")
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def O():
    from oracle import oracle

    oracle.lib()
    return oracle


def test_triangle_rule_matches_reference_literals(O):
    g = json.loads((GOLDEN / "triangle_rule_order4.json").read_text())
    pts, w = O.triangle_rule(4)
    assert np.array_equal(pts, np.asarray(g["points"]))
    assert np.array_equal(w, g["weight_factor"] * np.asarray(g["weights"]))
    # the reference keeps asymmetric final digits (BeatEngineCore.jl:524, :528)
    assert pts[1, 0] != pts[1, 1]
    for order, n in ((1, 1), (2, 3), (3, 3)):
        p, ww = O.triangle_rule(order)
        assert len(ww) == n and abs(ww.sum() - 0.5) < 1e-15


@pytest.mark.parametrize("kind,count", [(1, 1536), (2, 1280), (3, 512)])
def test_duffy_rules_cover_the_pair_domain(O, kind, count):
    test, trial, w = O.duffy_rule(4, kind)
    assert len(w) == count
    # each rule integrates 1 over T x T (area 1/2 each): sum of weights = 1/4
    assert abs(w.sum() - 0.25) < 1e-13
    for pts in (test, trial):
        assert np.all(pts >= -1e-15) and np.all(pts.sum(axis=1) <= 1 + 1e-15)
    # and a smooth integrand: int_T int_T x1 y2 = (1/6)(1/6)
    assert abs(np.sum(w * test[:, 0] * trial[:, 1]) - 1 / 36) < 1e-12


def test_reference_fixture_mesh_counts():
    counts = json.loads((GOLDEN / "reference_mesh_counts.json").read_text())
    assert counts["sample.msh"] == {"nodes": 1390, "triangles": 2776}
    assert counts["sample_quarter.msh"] == {"nodes": 441, "triangles": 798}


def test_loader_on_reference_fixture_meshes():
    ref = reference_checkout()
    root = ref / "src/blab/solvers/julia_local/test_meshes" if ref is not None else None
    if root is None or not root.exists():
        pytest.skip("reference checkout not present")
    counts = json.loads((GOLDEN / "reference_mesh_counts.json").read_text())
    for name, c in counts.items():
        mesh = meshes.read_gmsh22(root / name, 0.001)
        assert mesh.n_faces == c["triangles"]


@pytest.fixture(scope="module")
def subset16():
    g = json.loads((GOLDEN / "sample_subset16.json").read_text())
    return meshes.BoundaryMesh(np.asarray(g["vertices_mm"]) * 0.001, np.asarray(g["faces"]), np.asarray(g["tags"]))


def test_reference_cpu_pipeline_relations(O, subset16):
    """runtests.jl:79-146 on the same 16 elements: finite non-zero operators, factorised solve ==
    direct solve (rtol 1e-4), matrix-free RHS == materialised RHS (rtol 2e-5, runtests.jl:329)."""
    k = 2 * np.pi * 1000.0 / 343.0
    ops = O.assemble(subset16, k, regular_order=2, singular_order=2)
    for a in (ops.single_layer, ops.double_layer, ops.adjoint_double_layer, ops.hypersingular):
        assert np.all(np.isfinite(a)) and np.sum(np.abs(a) ** 2) > 0
    M11, M10 = O.mass(subset16, regular_order=2)
    lhs, rhs_op = O.burton_miller_matrices(ops, M11, M10, k)
    q = np.zeros(subset16.n_faces, complex)
    q[0] = 1j
    eta = 1j / k
    mf = -(ops.single_layer @ q) - eta * (ops.adjoint_double_layer @ q) - 0.5 * eta * (M10 @ q)
    assert np.allclose(mf, rhs_op @ q, rtol=2e-5)
    p_direct = np.linalg.solve(lhs, rhs_op @ q)
    p_lu = O.solve(lhs, rhs_op @ q)
    assert np.allclose(p_lu, p_direct, rtol=1e-4, atol=1e-4)
    assert np.all(np.isfinite(O.field(subset16, p_lu, q, k, O_fib(8, 2.0), regular_order=2)))


def O_fib(n, r):
    request = pkg_module("request")
    return request.fibonacci_sphere(n, r)


@pytest.mark.parametrize("freq", [200.0, 1000.0])
def test_oracle_pulsating_sphere(O, freq):
    """Uniform normal velocity on a sphere: p(a) = i rho omega a / (ika - 1).  Faceting limits
    agreement to ~0.5% on 1280 faces; this is a sanity check, not a parity pin."""
    v, f = meshes.icosphere(0.1, 3)
    mesh = meshes.BoundaryMesh(v, f, np.full(len(f), 2))
    rho, c, a = 1.205, 343.0, 0.1
    omega = 2 * np.pi * freq
    k = omega / c
    q = O.neumann_data(mesh, np.arange(len(f)), 1.0, rho, omega)
    sol = O.solve_frequency(mesh, k, q, np.array([[0, 0, 2.0]]))
    exact = 1j * rho * omega * a / (1j * k * a - 1)
    assert abs(sol.pressure[:, 0].mean() - exact) / abs(exact) < 5e-3
    A = 1j * rho * omega * a * a * np.exp(-1j * k * a) / (1j * k * a - 1)
    far = A * np.exp(1j * k * 2.0) / 2.0
    assert abs(sol.field[0, 0] - far) / abs(far) < 2e-2


def test_fp32_restatement_tracks_fp64(O):
    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)
    k = 2 * np.pi * 1500 / 343.0
    omega = k * 343.0
    q = O.neumann_data(mesh, np.nonzero(mesh.tags == 2)[0], 1.0, 1.205, omega)
    pts = np.array([[0, 0, 2.0], [2.0, 0, 0]])
    a = O.solve_frequency(mesh, k, q, pts)
    b = O.solve_frequency(mesh, k, q.astype(np.complex64), pts, precision="f32")
    assert np.linalg.norm(b.field - a.field) / np.linalg.norm(a.field) < 1e-4


def test_singular_pairs_are_the_vertex_sharing_pairs(O):
    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)
    f = mesh.faces
    expected = sum(1 for i in range(len(f)) for j in range(len(f)) if set(f[i]) & set(f[j]))
    assert O.singular_pair_count(mesh, 4) == expected
    assert O.color_count(mesh) >= 7  # valence-6 vertices need at least 7 colours


@pytest.mark.parametrize("name", ["sample_half", "sample_quarter", "sample_detailed"])
def test_fixture_meshes_match_the_reference_files(name):
    """The committed .npz fixtures hold the reference's test meshes: their counts are the
    counts read from the .msh files, and where the checkout is present the fixture equals
    what the loader (read_gmsh22, BeatEngineCore.jl:193-234) reads from the file."""
    z = np.load(GOLDEN / f"{name}.npz")
    counts = json.loads((GOLDEN / "reference_mesh_counts.json").read_text())[f"{name}.msh"]
    assert z["nodes_mm"].shape == (counts["nodes"], 3)
    assert z["faces"].shape == (counts["triangles"], 3)
    assert z["faces"].min() >= 0 and z["faces"].max() < counts["nodes"]
    ref = reference_checkout()
    path = None if ref is None else ref / "src/blab/solvers/julia_local/test_meshes" / f"{name}.msh"
    if path is None or not path.exists():
        pytest.skip("reference checkout not present")
    mesh = meshes.read_gmsh22(path, 1.0)
    assert np.array_equal(mesh.vertices, z["nodes_mm"])
    assert np.array_equal(mesh.faces, z["faces"]) and np.array_equal(mesh.tags, z["tags"])
