"""Launch-configuration autotuner on the GPU.

The search runs on a real mesh: the library's own configuration is timed first,
every candidate it accepts agrees with that configuration within the mixed
form's tolerance (1e-6 relative pressure), and the winner's solve gives the
same pressure and field as the library's default.  The engine's tuned path
(``CudaEngine(autotune=True)``) gives the results of the untuned engine.
"""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu

autotune = pkg_module("autotune")
engine_mod = pkg_module("engine")
meshes = pkg_module("meshes")

FREQS = np.geomspace(300.0, 4000.0, 6)
PTS = np.array([[0.0, 0.0, 2.0], [2.0, 0.0, 0.0], [0.0, 1.2, 1.6]])
TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def box():
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 1400, 0.05, "+z")
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    return mesh, drive


def test_tune_on_the_gpu(gpu_ctx, native, box):
    mesh, drive = box
    autotune.clear_cache()
    m = gpu_ctx.upload_mesh(mesh.vertices, mesh.faces)
    try:
        m.set_excitation(drive)
        m.set_observation_points(PTS)
        res = autotune.tune(m, FREQS, sound_speed=343.0, rho=1.205, repeats=1)
        assert res.trials[0].config == res.model and res.trials[0].status == "ok"
        ok = [t for t in res.trials if t.status == "ok"]
        assert res.best in [t.config for t in ok]
        assert all(t.rel_diff <= TOL and t.freq_per_s > 0 for t in ok)
        assert not any(t.status.startswith("rejected") for t in res.trials), res.to_dict()
        kw = dict(precision=native.BEM_PRECISION_MIXED, sound_speed=343.0, rho=1.205)
        p0, u0, _ = m.solve(FREQS, **kw)
        b = res.best
        p1, u1, _ = m.solve(FREQS, batch=b.batch, lu_block=b.lu_block, lu_gemm=b.lu_gemm, **kw)
        assert rel(p1, p0) < TOL and rel(u1, u0) < TOL
        again = autotune.tune(m, FREQS, sound_speed=343.0, rho=1.205)
        assert again.cached and again.best == res.best
    finally:
        m.release()
        autotune.clear_cache()


def test_engine_autotune_matches_untuned(native, box):
    mesh, drive = box
    autotune.clear_cache()
    plain, tuned = engine_mod.CudaEngine(), engine_mod.CudaEngine(autotune=True)
    try:
        for e in (plain, tuned):
            e.prepare(mesh.vertices, mesh.faces, drive, PTS)
        r0 = plain.solve(FREQS, 343.0, 1.205)
        r1 = tuned.solve(FREQS, 343.0, 1.205)
        assert tuned.launch is not None and tuned.tune_result is not None
        assert rel(r1.pressure, r0.pressure) < TOL and rel(r1.field, r0.field) < TOL
        # later solves reuse the winner without searching again
        r2 = tuned.solve(FREQS[:3], 343.0, 1.205)
        assert rel(r2.field, r0.field[:3]) < TOL
    finally:
        plain.close()
        tuned.close()
        autotune.clear_cache()
