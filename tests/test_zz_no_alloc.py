"""The allocation-free field entry point (bem_evaluate_field_noalloc).

Callers that cannot allocate device memory where they need a field (a real-time
audio callback, a host framework that owns all device memory, code running
while a CUDA graph is being recorded) get this entry point: they hand in their
own device buffers and the library uses a fixed scratch array of its own.  Here
the buffers are made with torch (the test may allocate; the entry point must
not), and the field is checked against the one bem_solve_frequencies returns
for the same pressure, twice in a row, in both precision forms.

This file is named to run last: it shares the library's fixed scratch array,
so running it after every other test also checks that earlier work leaves
nothing behind that it depends on.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu

meshes = pkg_module("meshes")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_noalloc_field_matches_solve(native, precision, tol):
    import torch

    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    points = np.array([[0, 0, 2.0], [2.0, 0, 0], [0, 1.2, 1.6], [0, 0, -2.0], [1.0, 1.0, 1.0]])
    freq, c, rho = 1500.0, 343.0, 1.205
    ctx = native.Context(0)
    try:
        m = ctx.upload_mesh(mesh.vertices, mesh.faces)
        m.set_excitation(drive)
        m.set_observation_points(points)
        p, u, _ = m.solve([freq], precision=precision, sound_speed=c, rho=rho)
        m.release()
    finally:
        ctx.close()
    omega = 2 * np.pi * freq
    q = drive[0] * (1j * rho * omega)
    dev = torch.device("cuda:0")
    d_v = torch.from_numpy(np.ascontiguousarray(mesh.vertices)).to(dev)
    d_f = torch.from_numpy(np.ascontiguousarray(mesh.faces, dtype=np.int32)).to(dev)
    d_p = torch.from_numpy(np.ascontiguousarray(p[0, 0])).to(dev)
    d_q = torch.from_numpy(np.ascontiguousarray(q)).to(dev)
    d_x = torch.from_numpy(points).to(dev)
    torch.cuda.synchronize()
    for _ in range(2):
        d_out = torch.full((len(points),), complex("nan+nanj"), dtype=torch.complex128, device=dev)
        torch.cuda.synchronize()
        native.evaluate_field_noalloc(d_v.data_ptr(), mesh.n_vertices, d_f.data_ptr(), mesh.n_faces, omega / c,
                                      d_p.data_ptr(), d_q.data_ptr(), d_x.data_ptr(), len(points), d_out.data_ptr(),
                                      precision=precision)
        out = d_out.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert _rel(out, u[0, 0]) < tol


def test_noalloc_rejects_oversize(native):
    import torch

    dev = torch.device("cuda:0")
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    with pytest.raises(native.BemError, match="exceeds"):
        native.evaluate_field_noalloc(buf.data_ptr(), 3, buf.data_ptr(), 20000, 1.0, buf.data_ptr(), buf.data_ptr(),
                                      buf.data_ptr(), 1, buf.data_ptr())
