"""GPU parity: the CUDA path (through the C ABI) against the FP64 CPU oracle.

Tolerances (relative, Frobenius / 2-norm unless stated):
  FP64 form  : operators 1e-11, solutions and fields 1e-9 (rounding-order only)
  mixed form : operators 2e-6 (compensated FP32 entries), solutions and fields 1e-5
               (the required bound on far-field pressure vs the FP64 oracle)
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu

meshes = pkg_module("meshes")


def _oracle():
    from oracle import oracle

    return oracle


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def sphere320():
    return meshes.sphere_with_cap(0.1, 2, 30.0)


@pytest.fixture(scope="module")
def box_small():
    return meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")


@pytest.mark.parametrize("freq", [100.0, 1000.0, 4000.0])
def test_bm_lhs_fp64_matches_oracle(gpu_ctx, native, sphere320, freq):
    O = _oracle()
    k = 2 * np.pi * freq / 343.0
    m = gpu_ctx.upload_mesh(sphere320.vertices, sphere320.faces)
    try:
        A = m.assemble_lhs(k, precision=native.BEM_PRECISION_FP64)
    finally:
        m.release()
    ops = O.assemble(sphere320, k)
    M11, M10 = O.mass(sphere320)
    lhs, _ = O.burton_miller_matrices(ops, M11, M10, k)
    assert rel(A, lhs) < 1e-11
    assert np.max(np.abs(A - lhs)) < 1e-10 * np.max(np.abs(lhs))


@pytest.mark.parametrize("which", ["D", "H", "M"])
def test_single_operators_fp64(gpu_ctx, native, box_small, which):
    O = _oracle()
    k = 2 * np.pi * 2500.0 / 343.0
    coeffs = {"D": (1.0, 0.0, 0.0), "H": (0.0, 1.0, 0.0), "M": (0.0, 0.0, 1.0)}[which]
    m = gpu_ctx.upload_mesh(box_small.vertices, box_small.faces)
    try:
        A = m.assemble_lhs(k, coeffs=coeffs, precision=native.BEM_PRECISION_FP64)
    finally:
        m.release()
    ops = O.assemble(box_small, k)
    M11, _ = O.mass(box_small)
    ref = {"D": ops.double_layer, "H": ops.hypersingular, "M": M11.astype(complex)}[which]
    assert rel(A, ref) < 1e-11


@pytest.mark.parametrize("which", ["D", "H", "DH"])
def test_single_operators_mixed(gpu_ctx, native, box_small, which):
    """Mixed form with one operator at a time: D alone (cH = 0), H alone (cD = 0:
    the regular kernel without the double-layer term), and a complex cD."""
    O = _oracle()
    k = 2 * np.pi * 4000.0 / 343.0
    coeffs = {"D": (1.0, 0.0, 0.0), "H": (0.0, 1.0, 0.0), "DH": (0.3 - 0.7j, 0.2 + 0.4j, 0.0)}[which]
    m = gpu_ctx.upload_mesh(box_small.vertices, box_small.faces)
    try:
        A = m.assemble_lhs(k, coeffs=coeffs, precision=native.BEM_PRECISION_MIXED)
    finally:
        m.release()
    ops = O.assemble(box_small, k)
    ref = coeffs[0] * ops.double_layer + coeffs[1] * ops.hypersingular
    assert rel(A, ref) < 2e-6


def test_bm_lhs_mixed_matches_oracle(gpu_ctx, native, box_small):
    O = _oracle()
    freq = 6000.0
    k = 2 * np.pi * freq / 343.0
    m = gpu_ctx.upload_mesh(box_small.vertices, box_small.faces)
    try:
        A = m.assemble_lhs(k, precision=native.BEM_PRECISION_MIXED)
    finally:
        m.release()
    ops = O.assemble(box_small, k)
    M11, M10 = O.mass(box_small)
    lhs, _ = O.burton_miller_matrices(ops, M11, M10, k)
    assert rel(A, lhs) < 2e-6


@pytest.mark.parametrize("freq", [2000.0, 12000.0])
def test_singular_remainder_both_paths(gpu_ctx, native, box_small, freq):
    """The mixed form integrates the singular remainder through the mesh's Chebyshev
    moments in calls of at least 12 frequencies, for every frequency whose expansion on the
    pair radius R (0.104 m on this coarse box) converges, and point by point on the Duffy
    rules otherwise.  The operator inspection entry points assemble as such a sweep does:
    2 kHz (kR = 3.8) through the moments, 12 kHz (kR = 22.8) point by point.  Both must give
    the full BM operator and the right-hand-side operator to 2e-6."""
    O = _oracle()
    k = 2 * np.pi * freq / 343.0
    rng = np.random.default_rng(11)
    q = rng.normal(size=(box_small.n_faces, 1)) + 1j * rng.normal(size=(box_small.n_faces, 1))
    m = gpu_ctx.upload_mesh(box_small.vertices, box_small.faces)
    try:
        m.set_excitation((box_small.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :])
        m.set_observation_points(np.array([[0.0, 0.0, 2.0]]))
        freqs = np.concatenate([np.geomspace(300.0, 2500.0, 11), [12000.0]])
        _, _, st = m.solve(freqs, precision=native.BEM_PRECISION_MIXED)
        assert st["singular_cheb_freqs"] == 11  # all but 12 kHz
        A = m.assemble_lhs(k, precision=native.BEM_PRECISION_MIXED)
        Sq = m.apply_rhs_operator(k, q, coeffs=(1.0, 0.0, 0.0), precision=native.BEM_PRECISION_MIXED)
        Kq = m.apply_rhs_operator(k, q, coeffs=(0.0, 1.0, 0.0), precision=native.BEM_PRECISION_MIXED)
    finally:
        m.release()
    ops = O.assemble(box_small, k)
    M11, M10 = O.mass(box_small)
    lhs, _ = O.burton_miller_matrices(ops, M11, M10, k)
    assert rel(A, lhs) < 2e-6
    assert rel(Sq, ops.single_layer @ q) < 2e-6
    assert rel(Kq, ops.adjoint_double_layer @ q) < 2e-6


def test_short_calls_run_point_by_point(gpu_ctx, native, sphere320):
    """A call of fewer than 12 frequencies integrates point by point, also on a mesh whose
    moments an earlier, longer call formed, so its results depend on its own inputs only."""
    m = gpu_ctx.upload_mesh(sphere320.vertices, sphere320.faces)
    try:
        m.set_excitation((sphere320.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :])
        m.set_observation_points(np.array([[0.0, 0.0, 2.0]]))
        short = np.geomspace(300.0, 900.0, 8)
        p1, u1, st = m.solve(short, precision=native.BEM_PRECISION_MIXED)
        assert st["singular_cheb_freqs"] == 0
        _, _, st = m.solve(np.geomspace(1000.0, 2500.0, 12), precision=native.BEM_PRECISION_MIXED)
        assert st["singular_cheb_freqs"] == 12
        p2, u2, st = m.solve(short, precision=native.BEM_PRECISION_MIXED)
        assert st["singular_cheb_freqs"] == 0
        assert np.array_equal(p1, p2) and np.array_equal(u1, u2)
    finally:
        m.release()


@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-6)])
def test_rhs_operator_matches_oracle(gpu_ctx, native, box_small, precision, tol):
    O = _oracle()
    k = 2 * np.pi * 1500.0 / 343.0
    rng = np.random.default_rng(7)
    q = rng.normal(size=(box_small.n_faces, 2)) + 1j * rng.normal(size=(box_small.n_faces, 2))
    ops = O.assemble(box_small, k)
    M11, M10 = O.mass(box_small)
    _, rhs_op = O.burton_miller_matrices(ops, M11, M10, k)
    m = gpu_ctx.upload_mesh(box_small.vertices, box_small.faces)
    try:
        bm = m.apply_rhs_operator(k, q, precision=precision)
        s_only = m.apply_rhs_operator(k, q[:, 0], coeffs=(1.0, 0.0, 0.0), precision=precision)
        k_only = m.apply_rhs_operator(k, q[:, 0], coeffs=(0.0, 1.0, 0.0), precision=precision)
    finally:
        m.release()
    assert rel(bm, rhs_op @ q) < tol
    assert rel(s_only, ops.single_layer @ q[:, 0]) < tol
    assert rel(k_only, ops.adjoint_double_layer @ q[:, 0]) < tol


def _solve_both(gpu_ctx, native, mesh, freqs, precision, drives=None, points=None):
    O = _oracle()
    if drives is None:
        drives = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    if points is None:
        points = np.array([[0, 0, 2.0], [2.0, 0, 0], [0, 1.2, 1.6], [0, 0, -2.0], [1.0, 1.0, 1.0]])
    c, rho = 343.0, 1.205
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(points)
        p, u, stats = m.solve(freqs, precision=precision, sound_speed=c, rho=rho)
    finally:
        m.release()
    refs = []
    for f in freqs:
        omega = 2 * np.pi * f
        q = (drives * (1j * rho * omega)).T
        refs.append(O.solve_frequency(mesh, omega / c, q, points))
    return p, u, stats, refs


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_full_solve_matches_oracle(gpu_ctx, native, sphere320, precision, tol):
    freqs = [150.0, 1200.0, 3000.0]
    p, u, stats, refs = _solve_both(gpu_ctx, native, sphere320, freqs, precision)
    for i, ref in enumerate(refs):
        assert rel(p[i, 0], ref.pressure[:, 0]) < tol
        assert rel(u[i, 0], ref.field[:, 0]) < tol
    if precision == 1:
        assert stats["max_rel_residual"] <= 1e-10


def test_two_excitations_and_batching(gpu_ctx, native, box_small):
    rng = np.random.default_rng(3)
    drives = np.zeros((2, box_small.n_faces), np.complex128)
    drives[0, box_small.tags == meshes.RADIATOR_TAG] = 1.0
    drives[1, rng.choice(box_small.n_faces, 20, replace=False)] = 0.5 - 0.25j
    freqs = [300.0, 2000.0, 5000.0]
    p, u, _, refs = _solve_both(gpu_ctx, native, box_small, freqs, 1, drives=drives)
    for i, ref in enumerate(refs):
        for c in range(2):
            assert rel(p[i, c], ref.pressure[:, c]) < 1e-5
            assert rel(u[i, c], ref.field[:, c]) < 1e-5


def test_batch_equals_single(gpu_ctx, native, sphere320):
    drives = (sphere320.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    pts = np.array([[0, 0, 2.0], [0, 2.0, 0]])
    m = gpu_ctx.upload_mesh(sphere320.vertices, sphere320.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(pts)
        freqs = [200.0, 700.0, 1900.0, 2600.0]
        pb, ub, _ = m.solve(freqs, batch=4)
        for i, f in enumerate(freqs):
            ps, us, _ = m.solve([f], batch=1)
            assert rel(ps[0], pb[i]) < 1e-12
            assert rel(us[0], ub[i]) < 1e-12
    finally:
        m.release()


def test_auto_batch(gpu_ctx, native, sphere320):
    """bem_auto_batch: the largest batch is within [1, 32]; a sweep is split into equal
    batches of at most that; batch = 0 solves exactly like the batch it reports."""
    drives = (sphere320.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    m = gpu_ctx.upload_mesh(sphere320.vertices, sphere320.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(np.array([[0, 0, 2.0]]))
        bmax = m.auto_batch(0)
        assert 1 <= bmax <= 32
        for n in (1, 7, 40, 64):
            nb = -(-n // bmax)
            assert m.auto_batch(n) == -(-n // nb)
        freqs = np.linspace(300.0, 3000.0, 7)
        pa, ua, _ = m.solve(freqs, batch=0)
        pe, ue, _ = m.solve(freqs, batch=m.auto_batch(len(freqs)))
        assert rel(pa, pe) == 0.0 and rel(ua, ue) == 0.0
    finally:
        m.release()


def test_isolated_vertex_gets_zero_pressure(gpu_ctx, native, sphere320):
    v = np.vstack([sphere320.vertices, [[5.0, 5.0, 5.0]]])
    mesh = meshes.BoundaryMesh(v, sphere320.faces, sphere320.tags)
    drives = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(np.array([[0, 0, 2.0]]))
        p, u, _ = m.solve([800.0])
    finally:
        m.release()
    assert p[0, 0, -1] == 0
    assert np.all(np.isfinite(p)) and np.all(np.isfinite(u))


def test_single_triangle(gpu_ctx, native):
    O = _oracle()
    v = np.array([[0.0, 0.0, 0.0], [0.02, 0.0, 0.0], [0.0, 0.02, 0.0]])
    f = np.array([[0, 1, 2]])
    mesh = meshes.BoundaryMesh(v, f, np.array([2]))
    k = 2 * np.pi * 1000 / 343.0
    m = gpu_ctx.upload_mesh(v, f)
    try:
        A = m.assemble_lhs(k, precision=0)
    finally:
        m.release()
    ops = O.assemble(mesh, k)
    M11, M10 = O.mass(mesh)
    lhs, _ = O.burton_miller_matrices(ops, M11, M10, k)
    assert rel(A, lhs) < 1e-11


def test_invalid_inputs_raise(gpu_ctx, native):
    with pytest.raises(native.BemError):
        gpu_ctx.upload_mesh(np.zeros((3, 3)), np.array([[0, 1, 2]]))  # zero-area triangle
    with pytest.raises(native.BemError):
        gpu_ctx.upload_mesh(np.eye(3), np.array([[0, 1, 5]]))  # index out of range
    m = gpu_ctx.upload_mesh(np.eye(3), np.array([[0, 1, 2]]))
    try:
        with pytest.raises(native.BemError):
            m.solve([100.0])  # no excitation yet
        m.set_excitation(np.ones((1, 1)))
        m.set_observation_points(np.array([[0, 0, 3.0]]))
        with pytest.raises(native.BemError):
            m.solve([-5.0])
    finally:
        m.release()
