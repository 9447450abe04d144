"""Far field of several frequencies per CTA against one frequency per call.

The mixed form's field kernel evaluates up to four frequencies per CTA (NFQ x
excitations <= 4), sharing each (point, source) geometry, when the grid of point blocks
times frequency groups still gives every SM a CTA: with 2,000 points (63 blocks of 32) a
sweep of 11 frequencies takes four per CTA with one excitation and two with two.  A call
of one frequency evaluates one per CTA.  Every frequency's field must agree to the
refinement tolerance (1e-9: the batched and the single LU round differently).  Sweeps of
fewer than 12 frequencies keep the singular remainder point by point in both calls.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")
request = pkg_module("request")
C, RHO = 343.0, 1.205


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("nc", [1, 2])
def test_grouped_field_matches_single_frequency(gpu_ctx, native, nc):
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    d = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)
    drives = np.stack([d, (0.3 + 0.6j) * d * np.linspace(0.5, 1.5, mesh.n_faces)])[:nc]
    pts = request.fibonacci_sphere(2000, 2.0)
    freqs = np.geomspace(250.0, 4000.0, 11)
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(pts)
        _, u, st = m.solve(freqs, precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO, batch=11)
        assert st["batches"] == 1 and st["singular_cheb_freqs"] == 0
        for i, f in enumerate(freqs):
            _, u1, _ = m.solve([f], precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO)
            assert rel(u[i], u1[0]) < 1e-9, (f, rel(u[i], u1[0]))
    finally:
        m.release()
