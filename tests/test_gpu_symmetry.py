"""Symmetric models on the GPU against the symmetric CPU oracle (same
formulation: image pairs, image singular blocks, orbit row weights, field
images), and against the mirrored full model (physics)."""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")

PTS = np.array([[0.4, 0.3, 1.5], [1.2, -0.8, 0.2], [-0.6, 0.5, -1.1], [0.0, 0.0, 2.0], [0.3, 0.0, 0.9]])


def _part(mode, target=600):
    return meshes.fundamental_domain(meshes.box_with_piston((0.3, 0.2, 0.25), target, 0.05, "+z"), mode)


def _solve_gpu(gpu_ctx, native, mesh, freqs, precision, symmetry):
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces, symmetry=symmetry)
    try:
        m.set_excitation(drive)
        m.set_observation_points(PTS)
        p, u, st = m.solve(freqs, precision=precision, sound_speed=343.0, rho=1.205)
    finally:
        m.release()
    return p, u, st


@pytest.mark.parametrize("mode", ["x", "xy"])
@pytest.mark.parametrize("form,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_symmetric_solve_matches_oracle(gpu_ctx, native, mode, form, tol):
    from oracle import oracle

    part = _part(mode)
    freqs = [600.0, 3100.0]
    precision = native.BEM_PRECISION_FP64 if form == "fp64" else native.BEM_PRECISION_MIXED
    p, u, _ = _solve_gpu(gpu_ctx, native, part, freqs, precision, mode)
    for i, f in enumerate(freqs):
        omega = 2 * np.pi * f
        q = np.where(part.tags == meshes.RADIATOR_TAG, 1j * 1.205 * omega, 0).astype(np.complex128)
        ref = oracle.solve_frequency(part, omega / 343.0, q, PTS, symmetry=mode)
        assert np.linalg.norm(p[i, 0] - ref.pressure[:, 0]) / np.linalg.norm(ref.pressure[:, 0]) < tol
        assert np.linalg.norm(u[i, 0] - ref.field[:, 0]) / np.linalg.norm(ref.field[:, 0]) < tol


def test_half_model_matches_full_model(gpu_ctx, native):
    part = _part("x", 1200)
    full, index = meshes.mirror_to_full(part, "x")
    p_h, u_h, st = _solve_gpu(gpu_ctx, native, part, [1500.0], native.BEM_PRECISION_MIXED, "x")
    p_f, u_f, _ = _solve_gpu(gpu_ctx, native, full, [1500.0], native.BEM_PRECISION_MIXED, "off")
    # quadrature orientation of mirrored faces (see the CPU symmetry tests) bounds the agreement
    assert np.linalg.norm(p_h[0, 0] - p_f[0, 0][index]) / np.linalg.norm(p_f[0, 0]) < 2e-5
    assert np.linalg.norm(u_h[0, 0] - u_f[0, 0]) / np.linalg.norm(u_f[0, 0]) < 2e-5
    assert st["regular_pairs"] > part.n_faces ** 2  # images included


def test_mesh_outside_fundamental_domain_is_rejected(gpu_ctx, native):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    with pytest.raises(native.BemError, match="fundamental domain"):
        gpu_ctx.upload_mesh(box.vertices, box.faces, symmetry="x")
