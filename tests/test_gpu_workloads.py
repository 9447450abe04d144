"""GPU parity on the benchmark's own workloads, through the C ABI, against the FP64 oracle.

* sphere1280: rigid sphere r = 0.1 m, icosphere of 1,280 flat triangles, unit normal
  velocity on the cap below 30 degrees of polar angle, c = 343 m/s, rho = 1.205 kg/m^3,
  16 log-spaced frequencies 100 Hz - 3 kHz, far field at 1,000 Fibonacci points at 2 m:
  every frequency, FP64 form within 1e-9 and mixed form within 1e-5 of the FP64 oracle,
  on the surface pressure and on the far field.
* box10k: the headline box (9,948 triangles, circular piston r = 5 cm on +z) at the top
  of its band, 12 kHz, where k h is largest and the matrix worst conditioned: both
  forms against the FP64 oracle (same bars), pressure and 2 x 73 polar + 2,000
  Fibonacci points.
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


def _oracle_solutions(mesh, freqs, points):
    from oracle import oracle

    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)
    return [oracle.solve_frequency(mesh, 2 * np.pi * f / C, drive * (1j * RHO * 2 * np.pi * f), points)
            for f in freqs]


def _gpu_solve(gpu_ctx, mesh, freqs, points, precision):
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drive)
        m.set_observation_points(points)
        p, u, st = m.solve(freqs, precision=precision, sound_speed=C, rho=RHO)
    finally:
        m.release()
    return p, u, st


@pytest.fixture(scope="module")
def sphere1280():
    mesh = meshes.config_mesh("sphere1280")
    freqs = np.logspace(np.log10(100.0), np.log10(3000.0), 16)
    points = request.fibonacci_sphere(1000, 2.0)
    return mesh, freqs, points, _oracle_solutions(mesh, freqs, points)


def test_sphere1280_is_the_configured_mesh(sphere1280):
    mesh = sphere1280[0]
    assert mesh.n_faces == 1280 and mesh.n_vertices == 642
    r = np.linalg.norm(mesh.vertices, axis=1)
    assert np.allclose(r, 0.1, rtol=1e-12)
    assert 0 < int((mesh.tags == meshes.RADIATOR_TAG).sum()) < mesh.n_faces


@pytest.mark.parametrize("form,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_sphere1280_every_frequency(gpu_ctx, native, sphere1280, form, tol):
    mesh, freqs, points, ref = sphere1280
    precision = native.BEM_PRECISION_FP64 if form == "fp64" else native.BEM_PRECISION_MIXED
    p, u, _ = _gpu_solve(gpu_ctx, mesh, freqs, points, precision)
    errs_p = [rel(p[i, 0], ref[i].pressure[:, 0]) for i in range(len(freqs))]
    errs_u = [rel(u[i, 0], ref[i].field[:, 0]) for i in range(len(freqs))]
    assert max(errs_p) < tol, errs_p
    assert max(errs_u) < tol, errs_u


@pytest.fixture(scope="module")
def box10k_top():
    mesh = meshes.config_mesh("box10k")
    _, horizontal, vertical, _ = request.polar_observation_points({"step_size": 5.0, "distance": 2.0})
    points = np.vstack([horizontal, vertical, request.fibonacci_sphere(2000, 2.0)])
    freqs = np.array([12000.0])
    return mesh, freqs, points, _oracle_solutions(mesh, freqs, points)


@pytest.mark.parametrize("form,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_box10k_top_frequency(gpu_ctx, native, box10k_top, form, tol):
    mesh, freqs, points, ref = box10k_top
    assert 9900 <= mesh.n_faces <= 10100
    precision = native.BEM_PRECISION_FP64 if form == "fp64" else native.BEM_PRECISION_MIXED
    p, u, st = _gpu_solve(gpu_ctx, mesh, freqs, points, precision)
    assert rel(p[0, 0], ref[0].pressure[:, 0]) < tol
    assert rel(u[0, 0], ref[0].field[:, 0]) < tol
