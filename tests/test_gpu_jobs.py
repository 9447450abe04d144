"""Several meshes in shared launches (bem_solve_jobs) against each mesh solved alone.

Three meshes of different sizes (their matrices padded to the largest with an
identity block) and different frequency counts, cut into batches that mix them.
Each job's pressure and field must equal its own bem_solve_frequencies results:
FP64 form to 1e-12 (only the rounding of sums can differ), mixed form to 1e-8
(a batch refines until every system in it reaches the 1e-10 residual, so a job
may take one more refinement step than alone), and the mixed form stays within
1e-5 of the FP64 oracle.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")
C, RHO = 343.0, 1.205
PTS = np.array([[0.0, 0.0, 2.0], [1.5, 0.3, 1.2], [-0.8, 1.1, -1.4], [2.0, 0.0, 0.0], [0.2, -1.9, 0.4]])


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _meshes():
    return [meshes.sphere_with_cap(0.1, 2, 30.0),                      # 320 faces
            meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z"),  # ~600 faces
            meshes.box_with_piston((0.2, 0.2, 0.2), 420, 0.04, "+z")]


FREQS = [np.array([300.0, 1700.0, 2900.0]), np.geomspace(200.0, 4000.0, 5), np.array([800.0, 2500.0])]


def _upload(ctx, mesh):
    m = ctx.upload_mesh(mesh.vertices, mesh.faces)
    m.set_excitation((mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :])
    m.set_observation_points(PTS)
    return m


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("mixed", 1e-8)])
@pytest.mark.parametrize("batch", [0, 4])
def test_jobs_match_each_mesh_alone(gpu_ctx, native, form, tol, batch):
    precision = native.BEM_PRECISION_FP64 if form == "fp64" else native.BEM_PRECISION_MIXED
    ms = [_upload(gpu_ctx, mesh) for mesh in _meshes()]
    try:
        assert len({m.n_vertices for m in ms}) == 3  # padding to the largest is exercised
        outs, stats = gpu_ctx.solve_jobs(list(zip(ms, FREQS)), precision=precision, sound_speed=C, rho=RHO,
                                         batch=batch)
        if batch == 4:
            assert stats["batches"] == 3  # 10 frequencies in batches of 4, two of them mixing meshes
        for m, f, (p, u) in zip(ms, FREQS, outs):
            p1, u1, _ = m.solve(f, precision=precision, sound_speed=C, rho=RHO)
            assert p.shape == p1.shape and u.shape == u1.shape
            assert rel(p, p1) < tol
            assert rel(u, u1) < tol
    finally:
        for m in ms:
            m.release()


def test_jobs_mixed_form_matches_oracle(gpu_ctx, native):
    from oracle import oracle

    ms_host = _meshes()
    ms = [_upload(gpu_ctx, mesh) for mesh in ms_host]
    try:
        outs, _ = gpu_ctx.solve_jobs(list(zip(ms, FREQS)), precision=native.BEM_PRECISION_MIXED, sound_speed=C,
                                     rho=RHO, batch=4)
    finally:
        for m in ms:
            m.release()
    for mesh, f, (p, u) in zip(ms_host, FREQS, outs):
        drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)
        for i, fz in enumerate(f):
            w = 2 * np.pi * fz
            ref = oracle.solve_frequency(mesh, w / C, drive * (1j * RHO * w), PTS)
            assert rel(p[i, 0], ref.pressure[:, 0]) < 1e-5
            assert rel(u[i, 0], ref.field[:, 0]) < 1e-5


def test_jobs_reject_mixed_excitation_counts(gpu_ctx, native):
    a, b = _meshes()[:2]
    ma = _upload(gpu_ctx, a)
    mb = gpu_ctx.upload_mesh(b.vertices, b.faces)
    try:
        d = (b.tags == meshes.RADIATOR_TAG).astype(np.complex128)
        mb.set_excitation(np.stack([d, 0.5 * d]))
        mb.set_observation_points(PTS)
        with pytest.raises(native.BemError, match="same number of excitations"):
            gpu_ctx.solve_jobs([(ma, [500.0]), (mb, [600.0])])
    finally:
        ma.release()
        mb.release()
