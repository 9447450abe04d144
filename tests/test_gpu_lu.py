"""Dense LU on the GPU against LAPACK getrf (scipy), through the C ABI.

FP64 form: pivots identical to LAPACK's (first maximum of |re| + |im|) and factors
within 1e-11.  Mixed form, backward error ||P A - L U|| / ||A||:
  cuBLAS cgemm trailing updates (IEEE FP32):        <= 2e-6
  tcgen05 3xFP16 trailing updates:                  <= 1e-4
The tensor-core FP32 accumulation is coarser than IEEE round-to-nearest, so the
backward error grows with n (measured 1.9e-6 at n = 200, 3.4e-5 at n = 2600,
5.3e-5 at n = 4000);
the FP64 iterative refinement removes it, which the end-to-end solves below
check against the oracle at 1e-5.
"""

import numpy as np
import pytest
import scipy.linalg

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")


def random_matrix(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(n) + 2.0 * np.eye(n) * (seed % 2)


def unpack(lu, ipiv):
    n = lu.shape[0]
    L = np.tril(lu, -1) + np.eye(n)
    U = np.triu(lu)
    perm = np.arange(n)
    for i, p in enumerate(ipiv):
        perm[[i, p]] = perm[[p, i]]
    return L, U, perm


@pytest.mark.parametrize("n", [1, 7, 64, 65, 200, 700])
def test_fp64_lu_matches_lapack(gpu_ctx, native, n):
    a = random_matrix(n, n)
    lu, ipiv = gpu_ctx.lu_factor_dense(a, precision=native.BEM_PRECISION_FP64)
    lu_ref, piv_ref = scipy.linalg.lu_factor(a)
    assert np.array_equal(ipiv, piv_ref)
    assert np.linalg.norm(lu - lu_ref) / np.linalg.norm(lu_ref) < 1e-11


@pytest.mark.parametrize("gemm", [1, 2])
@pytest.mark.parametrize("n", [40, 200, 1000, 2600])
def test_mixed_lu_backward_error(gpu_ctx, native, n, gemm):
    a = random_matrix(n, 3 * n + gemm)
    lu, ipiv = gpu_ctx.lu_factor_dense(a, precision=native.BEM_PRECISION_MIXED, lu_gemm=gemm)
    L, U, perm = unpack(lu, ipiv)
    err = np.linalg.norm(a[perm] - L @ U) / np.linalg.norm(a)
    assert err < (2e-6 if gemm == 1 else 1e-4), err


def test_tensor_and_cublas_updates_agree(gpu_ctx, native):
    a = random_matrix(900, 11)
    lu1, p1 = gpu_ctx.lu_factor_dense(a, precision=native.BEM_PRECISION_MIXED, lu_gemm=1)
    lu2, p2 = gpu_ctx.lu_factor_dense(a, precision=native.BEM_PRECISION_MIXED, lu_gemm=2)
    assert np.array_equal(p1, p2)
    assert np.linalg.norm(lu1 - lu2) / np.linalg.norm(lu1) < 1e-4


def test_zero_pivot_is_reported(gpu_ctx, native):
    a = random_matrix(50, 4)
    a[:, 17] = 0.0
    for precision in (native.BEM_PRECISION_FP64, native.BEM_PRECISION_MIXED):
        with pytest.raises(native.BemError, match="SINGULAR"):
            gpu_ctx.lu_factor_dense(a, precision=precision)


@pytest.mark.parametrize("gemm", [1, 2])
def test_bm_solve_with_each_trailing_update(gpu_ctx, native, gemm):
    from oracle import oracle

    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 1400, 0.05, "+z")
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    pts = np.array([[0, 0, 2.0], [2.0, 0, 0], [0, 1.2, 1.6]])
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drive)
        m.set_observation_points(pts)
        p, u, st = m.solve([700.0, 4100.0], precision=native.BEM_PRECISION_MIXED, sound_speed=343.0, rho=1.205,
                           lu_gemm=gemm)
    finally:
        m.release()
    assert st["lu_gemm_used"] == gemm
    for i, f in enumerate([700.0, 4100.0]):
        omega = 2 * np.pi * f
        ref = oracle.solve_frequency(mesh, omega / 343.0, drive[0] * 1j * 1.205 * omega, pts)
        assert np.linalg.norm(u[i, 0] - ref.field[:, 0]) / np.linalg.norm(ref.field[:, 0]) < 1e-5
        assert np.linalg.norm(p[i, 0] - ref.pressure[:, 0]) / np.linalg.norm(ref.pressure[:, 0]) < 1e-5
