"""The allocation-free field entry point (bem_evaluate_field_noalloc).

Some callers cannot allocate device memory where they need a field: a real-time
audio callback (an allocation can block for an unbounded time there) or a host
framework that owns all device memory through its own pool.  They hand in their
own device buffers and the library uses a fixed scratch array of its own.  Here
the buffers are made with torch (the test may allocate; the entry point must
not), and the field is checked, twice in a row, in both precision forms:

* against the field bem_solve_frequencies returns for the same pressure (the
  existing entry point), on a 320-face sphere;
* against the oracle's field of seeded boundary traces;
* near the 16,384-face limit, against bem_evaluate_field and the oracle;
* that the device's free memory is the same before and after a call;
* that a zero-area triangle and an out-of-range vertex index are reported, and
  that a mesh above the limit is rejected.

This file is named to run last: it shares the library's fixed scratch array,
so running it after every other test also checks that earlier work leaves
nothing behind that it depends on.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu

meshes = pkg_module("meshes")
C, RHO = 343.0, 1.205


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _to_dev(torch, a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a if dtype is None else a.astype(dtype))).to("cuda:0")


def _fib(n, r):
    return pkg_module("request").fibonacci_sphere(n, r)


def _noalloc(native, torch, mesh, k, p, q, points, precision, calls=2):
    d_v = _to_dev(torch, mesh.vertices, np.float64)
    d_f = _to_dev(torch, mesh.faces, np.int32)
    d_p = _to_dev(torch, p, np.complex128)
    d_q = _to_dev(torch, q, np.complex128)
    d_x = _to_dev(torch, points, np.float64)
    outs = []
    for _ in range(calls):
        d_out = torch.full((len(points),), complex("nan+nanj"), dtype=torch.complex128, device="cuda:0")
        torch.cuda.synchronize()
        native.evaluate_field_noalloc(d_v.data_ptr(), mesh.n_vertices, d_f.data_ptr(), mesh.n_faces, k,
                                      d_p.data_ptr(), d_q.data_ptr(), d_x.data_ptr(), len(points), d_out.data_ptr(),
                                      precision=precision)
        outs.append(d_out.cpu().numpy())
    return outs


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_noalloc_field_matches_solve(native, precision, tol):
    import torch

    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    points = np.array([[0, 0, 2.0], [2.0, 0, 0], [0, 1.2, 1.6], [0, 0, -2.0], [1.0, 1.0, 1.0]])
    freq = 1500.0
    ctx = native.Context(0)
    try:
        m = ctx.upload_mesh(mesh.vertices, mesh.faces)
        m.set_excitation(drive)
        m.set_observation_points(points)
        p, u, _ = m.solve([freq], precision=precision, sound_speed=C, rho=RHO)
        m.release()
    finally:
        ctx.close()
    omega = 2 * np.pi * freq
    q = drive[0] * (1j * RHO * omega)
    for out in _noalloc(native, torch, mesh, omega / C, p[0, 0], q, points, precision):
        assert np.all(np.isfinite(out))
        assert _rel(out, u[0, 0]) < tol


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_noalloc_field_matches_oracle(native, precision, tol):
    import torch
    from oracle import oracle

    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    rng = np.random.default_rng(21)
    p = rng.normal(size=mesh.n_vertices) + 1j * rng.normal(size=mesh.n_vertices)
    q = rng.normal(size=mesh.n_faces) + 1j * rng.normal(size=mesh.n_faces)
    points = _fib(64, 1.5)
    k = 2 * np.pi * 2200.0 / C
    ref = oracle.field(mesh, p, q, k, points)
    for out in _noalloc(native, torch, mesh, k, p, q, points, precision):
        assert _rel(out, ref) < tol


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_noalloc_near_the_face_limit(native, gpu_ctx, precision, tol):
    """16,232 faces (limit 16,384): the same field as bem_evaluate_field on the uploaded
    mesh and as the oracle."""
    import torch
    from oracle import oracle

    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 16300, 0.05, "+z")
    assert 16000 < mesh.n_faces <= 16384
    rng = np.random.default_rng(22)
    p = rng.normal(size=mesh.n_vertices) + 1j * rng.normal(size=mesh.n_vertices)
    q = rng.normal(size=mesh.n_faces) + 1j * rng.normal(size=mesh.n_faces)
    points = _fib(48, 2.0)
    k = 2 * np.pi * 5000.0 / C
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        via_mesh = m.evaluate_field(k, p, q, points, precision=precision)
    finally:
        m.release()
    ref = oracle.field(mesh, p, q, k, points)
    assert _rel(via_mesh, ref) < tol
    for out in _noalloc(native, torch, mesh, k, p, q, points, precision):
        assert _rel(out, via_mesh) < tol
        assert _rel(out, ref) < tol


def test_noalloc_call_allocates_no_device_memory(native):
    """After a first call (lazy kernel loading, scratch address lookup), a second call
    leaves the device's free memory exactly as it was."""
    import torch

    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)
    rng = np.random.default_rng(3)
    p = rng.normal(size=mesh.n_vertices) + 1j * rng.normal(size=mesh.n_vertices)
    q = rng.normal(size=mesh.n_faces) + 1j * rng.normal(size=mesh.n_faces)
    points = _fib(32, 2.0)
    bufs = [_to_dev(torch, a, t) for a, t in ((mesh.vertices, np.float64), (mesh.faces, np.int32),
                                             (p, np.complex128), (q, np.complex128), (points, np.float64))]
    out = torch.zeros(len(points), dtype=torch.complex128, device="cuda:0")
    args = (bufs[0].data_ptr(), mesh.n_vertices, bufs[1].data_ptr(), mesh.n_faces, 2 * np.pi * 900.0 / C,
            bufs[2].data_ptr(), bufs[3].data_ptr(), bufs[4].data_ptr(), len(points), out.data_ptr())
    for precision in (0, 1):
        native.evaluate_field_noalloc(*args, precision=precision)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info(0)
    for precision in (0, 1):
        native.evaluate_field_noalloc(*args, precision=precision)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info(0)
    assert free_after == free_before


def test_noalloc_reports_bad_meshes(native):
    import torch

    dev = torch.device("cuda:0")
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    with pytest.raises(native.BemError, match="exceeds"):
        native.evaluate_field_noalloc(buf.data_ptr(), 3, buf.data_ptr(), 20000, 1.0, buf.data_ptr(), buf.data_ptr(),
                                      buf.data_ptr(), 1, buf.data_ptr())
    # a zero-area triangle (collinear vertices) with valid indices
    v = np.array([[0.0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0.2, 0, 0]])
    f = np.array([[0, 1, 2], [0, 1, 3]], np.int32)
    pts = np.array([[0.0, 0.0, 1.0]])
    d_v, d_f, d_x = _to_dev(torch, v), _to_dev(torch, f), _to_dev(torch, pts)
    d_p = torch.ones(4, dtype=torch.complex128, device=dev)
    d_q = torch.ones(2, dtype=torch.complex128, device=dev)
    d_out = torch.zeros(1, dtype=torch.complex128, device=dev)
    for precision in (0, 1):
        with pytest.raises(native.BemError, match="degenerate"):
            native.evaluate_field_noalloc(d_v.data_ptr(), 4, d_f.data_ptr(), 2, 10.0, d_p.data_ptr(), d_q.data_ptr(),
                                          d_x.data_ptr(), 1, d_out.data_ptr(), precision=precision)
    # a face index past the vertex count: the kernels skip the reads and report it
    f_bad = _to_dev(torch, np.array([[0, 1, 2], [0, 1, 7]], np.int32))
    with pytest.raises(native.BemError, match="out of range"):
        native.evaluate_field_noalloc(d_v.data_ptr(), 4, f_bad.data_ptr(), 2, 10.0, d_p.data_ptr(), d_q.data_ptr(),
                                      d_x.data_ptr(), 1, d_out.data_ptr())
