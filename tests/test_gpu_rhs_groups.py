"""Right-hand sides of several frequencies in one launch against one frequency per call.

The mixed form integrates the right-hand sides of up to four frequencies (one
excitation) or two (two excitations) in one launch, sharing the frequency-independent
geometry of every quadrature pair; each frequency's arithmetic is that of the
one-frequency kernel.  A sweep solved in one call (frequency groups of 4 + 3 and 2 + 2 + 2 +
1) must match every frequency solved alone to the refinement tolerance: 1e-9, since the
batched and the single LU round differently and refinement stops at a 1e-10 residual.  The
symmetric (half-model) case runs the symmetry images through the same kernel.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")
C, RHO = 343.0, 1.205
PTS = np.array([[0.0, 0.0, 2.0], [1.5, 0.3, 1.2], [-0.8, 1.1, -1.4], [2.0, 0.0, 0.0]])


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("nc", [1, 2])
def test_grouped_rhs_matches_single_frequency(gpu_ctx, native, nc):
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 900, 0.05, "+z")
    d = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)
    drives = np.stack([d, (0.5 - 0.25j) * d * np.linspace(0.5, 1.5, mesh.n_faces)])[:nc]
    freqs = np.geomspace(250.0, 3800.0, 7)
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drives)
        m.set_observation_points(PTS)
        p, u, _ = m.solve(freqs, precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO)
        for i, f in enumerate(freqs):
            p1, u1, _ = m.solve([f], precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO)
            assert rel(p[i], p1[0]) < 1e-9, (f, rel(p[i], p1[0]))
            assert rel(u[i], u1[0]) < 1e-9, (f, rel(u[i], u1[0]))
    finally:
        m.release()


def test_grouped_rhs_half_model_matches_single_frequency(gpu_ctx, native):
    half = meshes.fundamental_domain(meshes.box_with_piston((0.3, 0.2, 0.25), 900, 0.05, "+z"), "x")
    d = (half.tags == meshes.RADIATOR_TAG).astype(np.complex128)
    freqs = np.geomspace(300.0, 3000.0, 4)
    m = gpu_ctx.upload_mesh(half.vertices, half.faces, symmetry="x")
    try:
        m.set_excitation(d[None, :])
        m.set_observation_points(PTS)
        p, u, _ = m.solve(freqs, precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO)
        for i, f in enumerate(freqs):
            p1, u1, _ = m.solve([f], precision=native.BEM_PRECISION_MIXED, sound_speed=C, rho=RHO)
            assert rel(p[i], p1[0]) < 1e-9, f
            assert rel(u[i], u1[0]) < 1e-9, f
    finally:
        m.release()
