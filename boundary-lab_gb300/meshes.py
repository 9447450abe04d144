"""Boundary meshes: Gmsh 2.2 I/O, geometry, and seeded synthetic generators.

The loader follows the reference's ``load_gmsh22_with_tags``
(src/blab/solvers/julia_local/src/BeatEngineCore.jl:193-234): only element
type 2 (3-node triangle) is read, element lines with fewer than 8 tokens are
skipped, the physical tag is the 4th token, the three nodes are the last three
tokens, and node coordinates are multiplied by ``scale``.  Geometry (normals,
areas, centroids) follows ``BoundaryMesh`` (BeatEngineCore.jl:236-256), and
multi-mesh combination follows ``load_combined_mesh`` (solver.jl:252-269):
meshes are appended without welding, each translated by its own offset.

The generators produce closed, outward-wound surfaces used as synthetic
workloads: an icosphere, a cube-sphere, a rectangular box with a circular
piston on one face, and an exponential horn mounted in a box.  All are
deterministic for a given set of arguments (and seed, where one is taken).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path
from typing import Sequence

import numpy as np

RADIATOR_TAG = 2
WALL_TAG = 1


@dataclass
class BoundaryMesh:
    """Triangulated boundary: vertices (N_p, 3) float64, faces (N_f, 3) int32 0-based."""

    vertices: np.ndarray
    faces: np.ndarray
    tags: np.ndarray
    element_mesh_ids: np.ndarray | None = None
    normals: np.ndarray = field(init=False)
    areas: np.ndarray = field(init=False)
    centroids: np.ndarray = field(init=False)

    def __post_init__(self) -> None:
        self.vertices = np.ascontiguousarray(self.vertices, dtype=np.float64)
        self.faces = np.ascontiguousarray(self.faces, dtype=np.int32)
        self.tags = np.ascontiguousarray(self.tags, dtype=np.int32)
        if self.element_mesh_ids is None:
            self.element_mesh_ids = np.ones(len(self.faces), dtype=np.int32)
        else:
            self.element_mesh_ids = np.ascontiguousarray(self.element_mesh_ids, dtype=np.int32)
        if self.faces.ndim != 2 or (self.faces.size and self.faces.shape[1] != 3):
            raise ValueError("faces must have shape (N_f, 3)")
        if self.faces.size and (self.faces.min() < 0 or self.faces.max() >= len(self.vertices)):
            raise ValueError("face index out of range")
        v = self.vertices[self.faces]
        cross = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
        norm = np.linalg.norm(cross, axis=1)
        if np.any(norm == 0.0):
            raise ValueError("degenerate (zero-area) triangle in mesh")
        self.areas = norm / 2.0
        self.normals = cross / norm[:, None]
        self.centroids = v.sum(axis=1) / 3.0

    @property
    def n_faces(self) -> int:
        return int(self.faces.shape[0])

    @property
    def n_vertices(self) -> int:
        return int(self.vertices.shape[0])

    def signed_volume(self) -> float:
        v = self.vertices[self.faces]
        return float(np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])).sum() / 6.0)


# ---------------------------------------------------------------------------
# Gmsh 2.2 ASCII
# ---------------------------------------------------------------------------


def write_gmsh22(path: str | Path, vertices: np.ndarray, faces: np.ndarray, tags: np.ndarray) -> None:
    """Write a Gmsh 2.2 ASCII mesh with 3-node triangles carrying (physical, elementary) tags."""
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(len(vertices))]
    lines.extend(
        f"{i + 1} {x:.17g} {y:.17g} {z:.17g}" for i, (x, y, z) in enumerate(np.asarray(vertices, float))
    )
    lines.extend(["$EndNodes", "$Elements", str(len(faces))])
    for i, (face, tag) in enumerate(zip(np.asarray(faces), np.asarray(tags))):
        a, b, c = (int(n) + 1 for n in face)
        lines.append(f"{i + 1} 2 2 {int(tag)} {int(tag)} {a} {b} {c}")
    lines.append("$EndElements")
    Path(path).write_text("\n".join(lines) + "\n", encoding="utf-8")


def read_gmsh22(path: str | Path, scale: float = 1.0) -> BoundaryMesh:
    """Read triangles and physical tags from a Gmsh 2.2 ASCII file (BeatEngineCore.jl:193-234)."""
    lines = Path(path).read_text(encoding="utf-8", errors="replace").splitlines()
    try:
        node_start = lines.index("$Nodes")
        node_end = lines.index("$EndNodes")
        elem_start = lines.index("$Elements")
        elem_end = lines.index("$EndElements")
    except ValueError as exc:
        raise ValueError("Only Gmsh 2.2 ASCII meshes with Nodes and Elements sections are supported.") from exc

    node_index: dict[int, int] = {}
    coords: list[tuple[float, float, float]] = []
    for line in lines[node_start + 2 : node_end]:
        parts = line.split()
        if len(parts) < 4:
            continue
        coords.append((float(parts[1]) * scale, float(parts[2]) * scale, float(parts[3]) * scale))
        node_index[int(parts[0])] = len(coords) - 1

    faces: list[tuple[int, int, int]] = []
    tags: list[int] = []
    for line in lines[elem_start + 2 : elem_end]:
        parts = line.split()
        if len(parts) < 8 or int(parts[1]) != 2:
            continue
        n1 = node_index.get(int(parts[-3]), -1)
        n2 = node_index.get(int(parts[-2]), -1)
        n3 = node_index.get(int(parts[-1]), -1)
        if n1 < 0 or n2 < 0 or n3 < 0:
            continue
        faces.append((n1, n2, n3))
        tags.append(int(parts[3]))

    return BoundaryMesh(
        np.asarray(coords, dtype=np.float64).reshape(-1, 3),
        np.asarray(faces, dtype=np.int32).reshape(-1, 3),
        np.asarray(tags, dtype=np.int32),
    )


def combine_meshes(meshes: Sequence[BoundaryMesh], translations: Sequence[Sequence[float]] | None = None) -> BoundaryMesh:
    """Append meshes without welding (solver.jl:252-269); element_mesh_ids are 1-based mesh ids."""
    if not meshes:
        raise ValueError("at least one mesh is required")
    translations = translations or [(0.0, 0.0, 0.0)] * len(meshes)
    vertices, faces, tags, ids = [], [], [], []
    offset = 0
    for mesh_id, (mesh, t) in enumerate(zip(meshes, translations), start=1):
        vertices.append(mesh.vertices + np.asarray(t, dtype=np.float64)[None, :])
        faces.append(mesh.faces + offset)
        tags.append(mesh.tags)
        ids.append(np.full(mesh.n_faces, mesh_id, dtype=np.int32))
        offset += mesh.n_vertices
    return BoundaryMesh(np.concatenate(vertices), np.concatenate(faces), np.concatenate(tags), np.concatenate(ids))


# ---------------------------------------------------------------------------
# Generators
# ---------------------------------------------------------------------------


def _orient_outward(vertices: np.ndarray, faces: np.ndarray, center: np.ndarray) -> np.ndarray:
    v = vertices[faces]
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    flip = np.einsum("ij,ij->i", n, v.mean(axis=1) - center) < 0
    faces = faces.copy()
    faces[flip] = faces[flip][:, [0, 2, 1]]
    return faces


def icosphere(radius: float = 0.1, subdivisions: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Icosahedron refined ``subdivisions`` times (20 * 4**s faces), vertices projected to the sphere."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [
        (-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
        (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
        (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1),
    ]
    faces = [
        (0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
        (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
        (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
        (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1),
    ]
    pts = [np.asarray(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def midpoint(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = pts[a] + pts[b]
                pts.append(m / np.linalg.norm(m))
                cache[key] = len(pts) - 1
            return cache[key]

        new_faces = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            new_faces.extend([(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)])
        faces = new_faces
    vertices = np.asarray(pts) * radius
    f = _orient_outward(vertices, np.asarray(faces, dtype=np.int32), np.zeros(3))
    return vertices, f


def cube_sphere(radius: float, n: int) -> tuple[np.ndarray, np.ndarray]:
    """Sphere from a cube with n x n quads per side (12 n^2 faces), projected radially."""
    vertices, faces = _structured_box_surface(np.array([2.0, 2.0, 2.0]), (n, n, n))
    vertices = vertices - 1.0
    vertices = vertices / np.linalg.norm(vertices, axis=1, keepdims=True) * radius
    return vertices, _orient_outward(vertices, faces, np.zeros(3))


def _structured_box_surface(dims: np.ndarray, counts: tuple[int, int, int]) -> tuple[np.ndarray, np.ndarray]:
    """Conforming structured triangulation of the surface of [0,dx]x[0,dy]x[0,dz]."""
    nx, ny, nz = counts
    n = (nx, ny, nz)
    index: dict[tuple[int, int, int], int] = {}
    coords: list[tuple[float, float, float]] = []

    def vid(i: int, j: int, k: int) -> int:
        key = (i, j, k)
        if key not in index:
            index[key] = len(coords)
            coords.append((dims[0] * i / nx, dims[1] * j / ny, dims[2] * k / nz))
        return index[key]

    faces: list[tuple[int, int, int]] = []
    for axis in range(3):
        u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
        for side in (0, n[axis]):
            for a in range(n[u_ax]):
                for b in range(n[v_ax]):
                    def p(da: int, db: int) -> int:
                        ijk = [0, 0, 0]
                        ijk[axis] = side
                        ijk[u_ax] = a + da
                        ijk[v_ax] = b + db
                        return vid(*ijk)

                    p00, p10, p11, p01 = p(0, 0), p(1, 0), p(1, 1), p(0, 1)
                    if (a + b) % 2 == 0:
                        tris = [(p00, p10, p11), (p00, p11, p01)]
                    else:
                        tris = [(p00, p10, p01), (p10, p11, p01)]
                    if side == 0:
                        tris = [(t[0], t[2], t[1]) for t in tris]
                    faces.extend(tris)
    return np.asarray(coords, dtype=np.float64), np.asarray(faces, dtype=np.int32)


def box_counts_for_target(dims: Sequence[float], target_faces: int) -> tuple[int, int, int]:
    """Grid counts (nx, ny, nz) whose box surface has ~target_faces triangles of near-uniform size."""
    dx, dy, dz = dims
    area = 2.0 * (dx * dy + dx * dz + dy * dz)
    h0 = math.sqrt(2.0 * area / target_faces)
    best = None
    for scale in np.linspace(0.85, 1.15, 121):
        h = h0 * scale
        c = tuple(max(1, int(round(d / h))) for d in dims)
        nf = 4 * (c[0] * c[1] + c[0] * c[2] + c[1] * c[2])
        aspect = max(d / k for d, k in zip(dims, c)) / min(d / k for d, k in zip(dims, c))
        score = (abs(nf - target_faces), aspect)
        if best is None or score < best[0]:
            best = (score, c)
    return best[1]


def box_with_piston(
    dims: Sequence[float] = (0.3, 0.2, 0.25),
    target_faces: int = 10000,
    piston_radius: float = 0.05,
    piston_face: str = "+z",
    piston_center_uv: Sequence[float] = (0.0, 0.0),
) -> BoundaryMesh:
    """Closed box centred at the origin; faces of ``piston_face`` within ``piston_radius`` of the
    piston centre (offset ``piston_center_uv`` from the face centre, in the face's two in-plane
    axes) are tagged RADIATOR_TAG, all others WALL_TAG."""
    dims_arr = np.asarray(dims, dtype=np.float64)
    counts = box_counts_for_target(dims, target_faces)
    vertices, faces = _structured_box_surface(dims_arr, counts)
    vertices = vertices - dims_arr / 2.0
    faces = _orient_outward(vertices, faces, np.zeros(3))
    axis = "xyz".index(piston_face[1])
    sign = 1.0 if piston_face[0] == "+" else -1.0
    u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
    centre = np.zeros(3)
    centre[axis] = sign * dims_arr[axis] / 2.0
    centre[u_ax] = piston_center_uv[0]
    centre[v_ax] = piston_center_uv[1]
    cent = vertices[faces].mean(axis=1)
    on_face = np.abs(cent[:, axis] - centre[axis]) < 1e-9
    dist = np.hypot(cent[:, u_ax] - centre[u_ax], cent[:, v_ax] - centre[v_ax])
    tags = np.where(on_face & (dist < piston_radius), RADIATOR_TAG, WALL_TAG).astype(np.int32)
    return BoundaryMesh(vertices, faces, tags)


def sphere_with_cap(radius: float = 0.1, subdivisions: int = 3, cap_half_angle_deg: float = 30.0) -> BoundaryMesh:
    """Icosphere whose faces with centroid polar angle (from +z) below the cap angle are radiators."""
    vertices, faces = icosphere(radius, subdivisions)
    cent = vertices[faces].mean(axis=1)
    polar = np.degrees(np.arccos(np.clip(cent[:, 2] / np.linalg.norm(cent, axis=1), -1.0, 1.0)))
    tags = np.where(polar < cap_half_angle_deg, RADIATOR_TAG, WALL_TAG).astype(np.int32)
    return BoundaryMesh(vertices, faces, tags)


def seeded_piston_mesh(target_faces: int, seed: int, piston_radius: float = 0.03) -> BoundaryMesh:
    """Serving-stream geometry: a box (dims drawn from the seed) or a cube-sphere with a piston
    at a seeded position.  Deterministic in (target_faces, seed)."""
    rng = np.random.default_rng(seed)
    if rng.random() < 0.5:
        dims = (0.3, 0.2, 0.25)
        face = ["+x", "-x", "+y", "-y", "+z", "-z"][int(rng.integers(6))]
        axis = "xyz".index(face[1])
        u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
        half_u = dims[u_ax] / 2 - piston_radius * 1.1
        half_v = dims[v_ax] / 2 - piston_radius * 1.1
        uv = (rng.uniform(-half_u, half_u), rng.uniform(-half_v, half_v))
        return box_with_piston(dims, target_faces, piston_radius, face, uv)
    n = max(2, int(round(math.sqrt(target_faces / 12.0))))
    radius = 0.12
    vertices, faces = cube_sphere(radius, n)
    direction = rng.normal(size=3)
    direction /= np.linalg.norm(direction)
    cent = vertices[faces].mean(axis=1)
    cosang = cent @ direction / np.linalg.norm(cent, axis=1)
    half_angle = piston_radius / radius
    tags = np.where(cosang > math.cos(half_angle), RADIATOR_TAG, WALL_TAG).astype(np.int32)
    if not np.any(tags == RADIATOR_TAG):
        tags[int(np.argmax(cosang))] = RADIATOR_TAG
    return BoundaryMesh(vertices, faces, tags)


def horn_in_box(
    box_dims: Sequence[float] = (0.5, 0.4, 0.4),
    throat_radius: float = 0.025,
    mouth_radius: float = 0.15,
    length: float = 0.2,
    target_faces: int = 20000,
) -> BoundaryMesh:
    """Axisymmetric exponential horn (radius r(z) = r_t exp(m z), mouth flush with the +z face)
    mounted in a closed box centred at the origin.  The throat disc is tagged RADIATOR_TAG.

    Surface pieces, all sharing vertices along their seams: the box's five plain faces, the front
    face with a circular hole (a polar-to-square ring), the horn wall, and the throat disc."""
    bx, by, bz = box_dims
    z_front = bz / 2.0
    z_throat = z_front - length
    # ring count around the axis, shared by the front-face hole, the horn wall and the disc
    h = math.sqrt(2.0 * (2 * (bx * by + bx * bz + by * bz)) / target_faces)
    n_theta = max(16, 4 * int(round(2 * math.pi * mouth_radius / h / 4)))
    m = math.log(mouth_radius / throat_radius) / length

    coords: list[np.ndarray] = []
    faces: list[tuple[int, int, int]] = []
    tags: list[int] = []

    def add(p: np.ndarray) -> int:
        coords.append(np.asarray(p, dtype=np.float64))
        return len(coords) - 1

    # ---- horn wall: rings from throat (s=0) to mouth (s=length)
    n_len = max(4, int(round(length / h)))
    rings: list[list[int]] = []
    for i in range(n_len + 1):
        s = length * i / n_len
        r = throat_radius * math.exp(m * s)
        z = z_throat + s
        rings.append([add((r * math.cos(2 * math.pi * j / n_theta), r * math.sin(2 * math.pi * j / n_theta), z)) for j in range(n_theta)])
    for i in range(n_len):
        for j in range(n_theta):
            a, b = rings[i][j], rings[i][(j + 1) % n_theta]
            c, d = rings[i + 1][(j + 1) % n_theta], rings[i + 1][j]
            faces.extend([(a, c, b), (a, d, c)])
            tags.extend([WALL_TAG, WALL_TAG])
    # ---- throat disc: concentric rings down to the centre
    n_disc = max(2, int(round(throat_radius / h)) + 1)
    disc_rings = [rings[0]]
    for i in range(1, n_disc):
        r = throat_radius * (1 - i / n_disc)
        disc_rings.append([add((r * math.cos(2 * math.pi * j / n_theta), r * math.sin(2 * math.pi * j / n_theta), z_throat)) for j in range(n_theta)])
    centre = add((0.0, 0.0, z_throat))
    for i in range(n_disc - 1):
        for j in range(n_theta):
            a, b = disc_rings[i][j], disc_rings[i][(j + 1) % n_theta]
            c, d = disc_rings[i + 1][(j + 1) % n_theta], disc_rings[i + 1][j]
            faces.extend([(a, b, c), (a, c, d)])
            tags.extend([RADIATOR_TAG, RADIATOR_TAG])
    last = disc_rings[-1]
    for j in range(n_theta):
        faces.append((last[j], last[(j + 1) % n_theta], centre))
        tags.append(RADIATOR_TAG)

    # ---- box: structured grid on the five plain faces plus a front face with a hole
    counts = box_counts_for_target(box_dims, int(target_faces * 0.8))
    nx, ny, nz = counts
    grid: dict[tuple[int, int, int], int] = {}
    dims = np.asarray(box_dims, dtype=np.float64)

    def gid(i: int, j: int, k: int) -> int:
        key = (i, j, k)
        if key not in grid:
            grid[key] = add(np.array([i / nx, j / ny, k / nz]) * dims - dims / 2.0)
        return grid[key]

    n = (nx, ny, nz)
    for axis in range(3):
        u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
        for side in (0, n[axis]):
            if axis == 2 and side == nz:
                continue  # front face handled below
            for a in range(n[u_ax]):
                for b in range(n[v_ax]):
                    def p(da: int, db: int) -> int:
                        ijk = [0, 0, 0]
                        ijk[axis] = side
                        ijk[u_ax] = a + da
                        ijk[v_ax] = b + db
                        return gid(*ijk)

                    p00, p10, p11, p01 = p(0, 0), p(1, 0), p(1, 1), p(0, 1)
                    tris = [(p00, p10, p11), (p00, p11, p01)]
                    if side == 0:
                        tris = [(t[0], t[2], t[1]) for t in tris]
                    faces.extend(tris)
                    tags.extend([WALL_TAG, WALL_TAG])
    # front face boundary loop (counter-clockwise seen from +z), resampled to n_theta points
    boundary: list[int] = []
    for i in range(nx):
        boundary.append(gid(i, 0, nz))
    for j in range(ny):
        boundary.append(gid(nx, j, nz))
    for i in range(nx, 0, -1):
        boundary.append(gid(i, ny, nz))
    for j in range(ny, 0, -1):
        boundary.append(gid(0, j, nz))
    bpts = np.array([coords[b] for b in boundary])
    bang = np.arctan2(bpts[:, 1], bpts[:, 0])
    order = np.argsort(bang)
    boundary = [boundary[o] for o in order]
    bang = bang[order]
    # ring layers between the square boundary (t=1) and the mouth circle (t=0)
    n_layers = max(2, int(round((min(bx, by) / 2 - mouth_radius) / h)))
    mouth = rings[-1]
    layers: list[list[int]] = [mouth]
    for L in range(1, n_layers):
        t = L / n_layers
        layer = []
        for j in range(n_theta):
            ang = 2 * math.pi * j / n_theta
            d = np.array([math.cos(ang), math.sin(ang)])
            s = min(bx / 2 / max(abs(d[0]), 1e-12), by / 2 / max(abs(d[1]), 1e-12))
            rad = (1 - t) * mouth_radius + t * s
            layer.append(add((rad * d[0], rad * d[1], z_front)))
        layers.append(layer)
    for L in range(n_layers - 1):
        inner, outer = layers[L], layers[L + 1]
        for j in range(n_theta):
            a, b = inner[j], inner[(j + 1) % n_theta]
            c, d = outer[(j + 1) % n_theta], outer[j]
            faces.extend([(a, b, c), (a, c, d)])
            tags.extend([WALL_TAG, WALL_TAG])
    # stitch the outermost ring layer to the square boundary by angular sweep
    outer = layers[-1]
    oang = np.array([2 * math.pi * j / n_theta for j in range(n_theta)])
    oang = np.where(oang > math.pi, oang - 2 * math.pi, oang)
    oorder = np.argsort(oang)
    outer_sorted = [outer[o] for o in oorder]
    oang = oang[oorder]
    i = j = 0
    nb, no = len(boundary), len(outer_sorted)
    while i < nb or j < no:
        bi, bj = boundary[i % nb], outer_sorted[j % no]
        next_b = bang[(i + 1) % nb] + (2 * math.pi if i + 1 >= nb else 0.0)
        next_o = oang[(j + 1) % no] + (2 * math.pi if j + 1 >= no else 0.0)
        if j >= no or (i < nb and next_b <= next_o):
            faces.append((bj, bi, boundary[(i + 1) % nb]))
            i += 1
        else:
            faces.append((bj, bi, outer_sorted[(j + 1) % no]))
            j += 1
        tags.append(WALL_TAG)
    vertices = np.asarray(coords)
    f = np.asarray(faces, dtype=np.int32)
    # orient: front-face pieces must face +z; the horn wall faces the horn axis; others outward
    v = vertices[f]
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    cent = v.mean(axis=1)
    want = np.zeros_like(nrm)
    on_front = np.abs(cent[:, 2] - z_front) < 1e-9
    on_box = (np.abs(np.abs(cent[:, 0]) - bx / 2) < 1e-9) | (np.abs(np.abs(cent[:, 1]) - by / 2) < 1e-9) | (np.abs(cent[:, 2] + bz / 2) < 1e-9)
    want[on_box] = cent[on_box]
    want[on_front] = np.array([0.0, 0.0, 1.0])
    horn = ~(on_front | on_box)
    # inside the horn (wall and throat disc) the exterior region is the horn's air: normals point
    # toward the axis / toward +z at the throat
    radial = cent[horn].copy()
    radial[:, 2] = 0.0
    want[horn] = -radial
    disc = horn & (np.abs(cent[:, 2] - z_throat) < 1e-9)
    want[disc] = np.array([0.0, 0.0, 1.0])
    flip = np.einsum("ij,ij->i", nrm, want) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return BoundaryMesh(vertices, f, np.asarray(tags, dtype=np.int32))


# ---------------------------------------------------------------------------
# Symmetry (BeatEngineCore.jl:357-439)
# ---------------------------------------------------------------------------

SYMMETRY_AXES = {"off": (), "x": (0,), "xy": (0, 1)}


def symmetry_plane_tolerance(vertices: np.ndarray) -> float:
    """max(1e-9, 1e-6 x bounding-box diagonal) (symmetry_plane_tolerance)."""
    v = np.asarray(vertices, dtype=np.float64)
    if len(v) == 0:
        return 1e-9
    return max(1e-9, float(np.linalg.norm(v.max(axis=0) - v.min(axis=0))) * 1e-6)


def snap_symmetry_planes(mesh: BoundaryMesh, mode: str) -> BoundaryMesh:
    """Vertices within the plane tolerance of an active symmetry plane moved onto it
    (snap_symmetry_planes); the same mesh object when nothing moves."""
    axes = SYMMETRY_AXES[mode]
    if not axes:
        return mesh
    tol = symmetry_plane_tolerance(mesh.vertices)
    v = mesh.vertices.copy()
    for a in axes:
        v[np.abs(v[:, a]) <= tol, a] = 0.0
    if np.array_equal(v, mesh.vertices):
        return mesh
    return BoundaryMesh(v, mesh.faces, mesh.tags, mesh.element_mesh_ids)


def validate_symmetry_fundamental_domain(mesh: BoundaryMesh, mode: str) -> None:
    """Raise when a vertex lies on the negative side of an active plane
    (validate_symmetry_fundamental_domain!; same message)."""
    tol = symmetry_plane_tolerance(mesh.vertices)
    for a in SYMMETRY_AXES[mode]:
        bad = np.nonzero(mesh.vertices[:, a] < -tol)[0]
        if len(bad):
            name = "XY" if mode == "xy" else "X"
            axis = "X" if a == 0 else "Y"
            raise ValueError(f"Mesh is not in the positive {axis} fundamental domain for {name} symmetry. "
                             f"Vertex {int(bad[0]) + 1} has {axis.lower()}={mesh.vertices[bad[0], a]} m.")


def p1_symmetry_orbit_weights(mesh: BoundaryMesh, mode: str) -> np.ndarray:
    """2 per active symmetry plane the vertex lies on (p1_symmetry_orbit_weights)."""
    tol = symmetry_plane_tolerance(mesh.vertices)
    w = np.ones(mesh.n_vertices)
    for a in SYMMETRY_AXES[mode]:
        w[np.abs(mesh.vertices[:, a]) <= tol] *= 2.0
    return w


def fundamental_domain(mesh: BoundaryMesh, mode: str) -> BoundaryMesh:
    """The faces of a mesh whose centroids lie in the positive domain of the active
    planes, with unused vertices dropped (for building symmetric test models)."""
    keep = np.ones(mesh.n_faces, dtype=bool)
    for a in SYMMETRY_AXES[mode]:
        keep &= mesh.centroids[:, a] > 0.0
    faces = mesh.faces[keep]
    used = np.unique(faces)
    remap = -np.ones(mesh.n_vertices, dtype=np.int64)
    remap[used] = np.arange(len(used))
    part = snap_symmetry_planes(BoundaryMesh(mesh.vertices[used], remap[faces].astype(np.int32), mesh.tags[keep]), mode)
    validate_symmetry_fundamental_domain(part, mode)  # faces must not straddle a plane
    return part


def mirror_to_full(mesh: BoundaryMesh, mode: str) -> tuple[BoundaryMesh, np.ndarray]:
    """The full model of a fundamental-domain mesh: the mesh plus its reflections
    (faces reversed so normals stay outward), vertices on the planes shared.
    Returns (full mesh, index of each fundamental-domain vertex in the full mesh)."""
    mesh = snap_symmetry_planes(mesh, mode)
    verts = [mesh.vertices]
    faces = [mesh.faces]
    tags = [mesh.tags]
    index = np.arange(mesh.n_vertices)
    for signs in {"x": [(-1, 1)], "xy": [(-1, 1), (1, -1), (-1, -1)]}.get(mode, []):
        s = np.array([signs[0], signs[1], 1.0])
        base = sum(len(v) for v in verts)
        ids = np.empty(mesh.n_vertices, dtype=np.int64)
        new = []
        for i, p in enumerate(mesh.vertices):
            q = p * s
            if np.array_equal(q, p):
                ids[i] = i  # on every reflecting plane: shared with the original
            else:
                ids[i] = base + len(new)
                new.append(q)
        # vertices on one plane only: shared with the image across that plane
        if len(new):
            verts.append(np.array(new))
        f = ids[mesh.faces]
        faces.append(f[:, [0, 2, 1]] if signs[0] * signs[1] < 0 else f)
        tags.append(mesh.tags)
    full_v = np.concatenate(verts)
    full_f = np.concatenate(faces).astype(np.int64)
    # weld coincident vertices (a vertex on the x plane reflected in y lands on its y-image, etc.)
    key = {}
    remap = np.empty(len(full_v), dtype=np.int64)
    out_v = []
    for i, p in enumerate(full_v):
        k = tuple(np.round(p, 12))
        if k not in key:
            key[k] = len(out_v)
            out_v.append(p)
        remap[i] = key[k]
    full = BoundaryMesh(np.array(out_v), remap[full_f].astype(np.int32), np.concatenate(tags))
    return full, remap[index]


def config_mesh(name: str) -> BoundaryMesh:
    """The synthetic meshes of the benchmark workloads, by name."""
    if name == "sphere1280":
        return sphere_with_cap(0.1, 3, 30.0)
    if name == "box5k":
        return box_with_piston((0.3, 0.2, 0.25), 5000, 0.05, "+z")
    if name == "box10k":
        return box_with_piston((0.3, 0.2, 0.25), 10000, 0.05, "+z")
    if name == "horn20k":
        return horn_in_box(target_faces=22300)  # 20,032 triangles (10,018 dofs)
    raise ValueError(f"unknown synthetic mesh {name!r}")
