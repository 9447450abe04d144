"""Backend, worker and server integration on CPU.

The numerical engine is the CPU oracle (tests/oracle_engine.py), selected through
the product's engine hook, so the event contract, cancellation and error paths
are checked without a GPU.  Where Boundary Lab's own Python package is present
(the reference checkout), the backend is also driven through the reference's
registry, its BEAT subprocess adapter and its job server, exactly as the
application would.
"""

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module, reference_checkout

TESTS = Path(__file__).resolve().parent
ROOT = TESTS.parent
_REF = reference_checkout()
REF_SRC = _REF / "src" if _REF is not None else Path("/nonexistent-boundary-lab/src")
meshes = pkg_module("meshes")
job_mod = pkg_module("job")
backend_mod = pkg_module("backend")
contract = pkg_module("contract")
WORKER = ROOT / "boundary-lab_gb300" / "worker.py"


def oracle_factory(**kw):
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    return oracle_engine.make_engine(**kw)


@pytest.fixture(scope="module")
def mesh_file(tmp_path_factory):
    mesh = meshes.sphere_with_cap(0.1, 1, 40.0)  # 80 faces
    path = tmp_path_factory.mktemp("mesh") / "sphere.msh"
    meshes.write_gmsh22(path, mesh.vertices * 1000.0, mesh.faces, mesh.tags)  # millimetres, like the app
    return path


def base_config(mesh_file, **extra):
    cfg = {"mesh_file": str(mesh_file), "scale_factor": 0.001, "rho": 1.205, "sound_speed": 343.0,
           "step_size": 30.0, "distance": 2.0, "radiators": [{"name": "cap", "tag": 2, "channel": "main"}],
           "channels": [{"name": "main"}], "flat_target_normalization_enabled": True}
    cfg.update(extra)
    return cfg


RESULT_KEYS = {"freq_hz", "horizontal_spl_norm_db", "vertical_spl_norm_db", "impedance", "horizontal_spl_db",
               "vertical_spl_db", "sphere_spl_norm_db", "channel_names", "horizontal_pressure", "vertical_pressure",
               "sphere_pressure", "timings", "diagnostics"}


def test_job_events_match_the_reference_contract(mesh_file):
    req = {"schema_version": 2, "config": base_config(mesh_file, spherical_sampling_enabled=True,
                                                        spherical_sampling_points=20),
           "frequencies_hz": [300.0, 900.0, 1800.0]}
    job = job_mod.ExteriorJob(req, engine_factory=oracle_factory)
    init = job.initialized_payload()
    assert len(init["polar_angle_deg"]) == 13 and init["radiator_names"] == ["cap"]
    assert set(init["sphere_metadata"]) == {"r_distance_m", "theta_polar_rad", "phi_azimuth_rad"}
    events = list(job.results())
    assert [e["solved_count"] for e in events] == [1, 2, 3] and all(e["total_count"] == 3 for e in events)
    for e in events:
        r = e["result"]
        assert set(r) == RESULT_KEYS
        assert set(r["timings"]) == {"assembly_s", "solve_s", "field_s"}
        on_axis = int(np.argmin(np.abs(init["polar_angle_deg"])))
        assert abs(r["horizontal_spl_norm_db"][on_axis]) < 1e-5  # flat-target normalisation
        assert np.all(np.isfinite(r["impedance"]))
        assert len(r["horizontal_pressure"]["real"]) == 1 and len(r["sphere_pressure"]["real"][0]) == 20
    json.dumps(events)  # the payload is JSON-serialisable


def test_job_pressure_matches_direct_oracle(mesh_file):
    from oracle import oracle

    req = {"config": base_config(mesh_file, step_size=90.0), "frequencies_hz": [750.0]}
    job = job_mod.ExteriorJob(req, engine_factory=oracle_factory)
    ev = next(job.results())
    mesh = meshes.read_gmsh22(mesh_file, 0.001)
    f = float(np.float32(750.0))
    omega = 2 * np.pi * f
    q = (mesh.tags == 2).astype(complex) * (1j * 1.205 * omega)
    ref = oracle.solve_frequency(mesh, omega / 343.0, q, job.points)
    hp = np.asarray(ev["result"]["horizontal_pressure"]["real"][0]) + 1j * np.asarray(ev["result"]["horizontal_pressure"]["imag"][0])
    assert np.allclose(hp, ref.field[: len(hp), 0], rtol=1e-5)


def test_job_rejections(mesh_file):
    with pytest.raises(Exception, match="symmetry"):
        job_mod.ExteriorJob({"config": base_config(mesh_file, symmetry="z"), "frequencies_hz": [100.0]})
    # the whole sphere is not an x >= 0 fundamental domain (solver.jl:718-719)
    sym_job = job_mod.ExteriorJob({"config": base_config(mesh_file, symmetry="x"), "frequencies_hz": [100.0]},
                                  engine_factory=oracle_factory)
    with pytest.raises(Exception, match="fundamental domain"):
        sym_job.setup()
    with pytest.raises(Exception, match="at least one"):
        job_mod.ExteriorJob({"config": base_config(mesh_file), "frequencies_hz": []})
    job = job_mod.ExteriorJob({"config": base_config(mesh_file, radiators=[{"name": "x", "tag": 7}]),
                               "frequencies_hz": [100.0]}, engine_factory=oracle_factory)
    with pytest.raises(Exception, match="No elements"):
        next(job.results())


def test_session_stream_and_cancel(mesh_file):
    cfg = base_config(mesh_file)
    backend = backend_mod.Gb300BemBackend(engine_factory=oracle_factory)
    req = contract.SolveRequest(cfg, np.asarray([200.0, 400.0, 800.0, 1600.0], np.float32))
    session = backend.create_session(req)
    assert session.metadata.radiator_names.tolist() == ["cap"]
    got = []
    for res in session.solve_stream():
        got.append(res.freq_hz)
        if len(got) == 2:
            session.stop()
    assert got == [200.0, 400.0]
    results = list(backend.create_session(req).solve_stream(stop_requested=lambda: False))
    assert [r.freq_hz for r in results] == [200.0, 400.0, 800.0, 1600.0]
    assert results[0].horizontal_pressure.dtype == np.complex64 and results[0].diagnostics.backend == "gb300_cuda"


def _run_worker(args, stdin=None, env_extra=None, timeout=300):
    env = dict(os.environ)
    env["GB300_BEM_ENGINE"] = "oracle_engine:make_engine"
    env["PYTHONPATH"] = os.pathsep.join([str(TESTS), str(ROOT)] + ([env["PYTHONPATH"]] if env.get("PYTHONPATH") else []))
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(WORKER), *args], input=stdin, capture_output=True, text=True, env=env,
                          timeout=timeout)


def test_worker_one_shot_and_worker_mode(tmp_path, mesh_file):
    req = {"schema_version": 2, "config": base_config(mesh_file), "frequencies_hz": [500.0, 1000.0],
           "cancel_path": str(tmp_path / "cancel")}
    rp = tmp_path / "request.json"
    rp.write_text(json.dumps(req))
    out = _run_worker(["--request", str(rp)])
    events = [json.loads(ln) for ln in out.stdout.splitlines() if ln.strip()]
    types = [e["type"] for e in events]
    assert types[0] == "initialized" and types[-1] == "completed" and types.count("result") == 2
    out = _run_worker(["--worker"], stdin=json.dumps({"request": str(rp)}) + "\n" + json.dumps({"request": "/nonexistent.json"}) + "\n")
    events = [json.loads(ln) for ln in out.stdout.splitlines() if ln.strip()]
    assert events[0]["type"] == "ready" and events[0]["protocol"] == "boundary_lab_julia_worker"
    types = [e["type"] for e in events]
    assert types.count("completed") == 1 and types[-1] == "failed"
    (tmp_path / "cancel").write_text("cancel")
    out = _run_worker(["--request", str(rp)])
    events = [json.loads(ln) for ln in out.stdout.splitlines() if ln.strip()]
    assert events[-1] == {"type": "cancelled", "solved_count": 0}


# ------------------------------------------------ the reference's own stack --

needs_ref = pytest.mark.skipif(not (REF_SRC / "blab").exists(), reason="reference checkout not present")


@pytest.fixture
def blab(monkeypatch):
    monkeypatch.syspath_prepend(str(REF_SRC))
    monkeypatch.setenv("BLAB_SKIP_GUI_TESTS", "1")
    import blab.solvers.registry as registry

    return registry


@needs_ref
def test_registration_and_server_health(blab):
    assert backend_mod.register_with_boundary_lab()
    info = blab.backend_info("gb300_cuda")
    assert info.capabilities.supports_channel_resynthesis
    backend = blab.create_backend("gb300_cuda", julia_executable="julia", julia_threads="auto")
    assert backend.backend_id == "gb300_cuda"
    from blab import server

    assert server.normalize_server_solver_id("gb300_cuda") == "gb300_cuda"
    orch = server.JobOrchestrator(solver_factory=lambda cfg: None)
    srv = server.BlabServer(("127.0.0.1", 0), orch, solver_id="gb300_cuda")
    try:
        health = srv.health_payload()
        assert health["backend"] == "gb300_cuda" and health["solver"] == "gb300_cuda"
    finally:
        srv.server_close()
        orch.shutdown()


@needs_ref
def test_reference_beat_adapter_drives_the_worker(blab, monkeypatch, mesh_file, tmp_path):
    """The reference's subprocess adapter, unchanged, with this worker as its solver script."""
    from blab.config import ChannelConfig, RadiatorConfig, SimulationConfig
    from blab.solvers.base import SolveRequest
    from blab.solvers.beat_engine_backend import BeatEngineBackend, shutdown_beat_engine_workers

    monkeypatch.setenv("GB300_BEM_ENGINE", "oracle_engine:make_engine")
    monkeypatch.setenv("PYTHONPATH", os.pathsep.join([str(TESTS), str(ROOT)]))
    cfg = SimulationConfig(mesh_file=str(mesh_file), scale_factor=0.001, rho=1.205, step_size=45.0,
                           radiators=(RadiatorConfig(name="cap", tag=2),), channels=(ChannelConfig(name="main"),))
    for persistent in (False, True):
        backend = BeatEngineBackend(julia_executable=sys.executable, solver_script=str(WORKER), julia_project=None,
                                    persistent_worker=persistent)
        session = backend.create_session(SolveRequest(cfg, np.asarray([400.0, 1200.0], np.float32)))
        results = list(session.solve_stream())
        assert [r.freq_hz for r in results] == [400.0, 1200.0]
        assert results[0].diagnostics.backend == "gb300_cuda"
        assert session.metadata.polar_angle_deg.size == 9
    bad = SimulationConfig(mesh_file=str(mesh_file), scale_factor=0.001, radiators=(RadiatorConfig(name="x", tag=9),))
    backend = BeatEngineBackend(julia_executable=sys.executable, solver_script=str(WORKER), julia_project=None)
    with pytest.raises(RuntimeError, match="No elements"):
        list(backend.create_session(SolveRequest(bad, np.asarray([400.0], np.float32))).solve_stream())
    shutdown_beat_engine_workers()


@needs_ref
def test_reference_job_server_runs_a_job(blab, monkeypatch, mesh_file, tmp_path):
    """POST-equivalent submit through the reference's JobOrchestrator with this backend: events
    queued, started, initialized, result..., completed and a result.npz artifact."""
    from blab import server
    from blab.config import ChannelConfig, RadiatorConfig, SimulationConfig

    backend_mod.register_with_boundary_lab()
    monkeypatch.setenv("GB300_BEM_ENGINE", "oracle_engine:make_engine")
    sys.path.insert(0, str(TESTS))
    factory = server.create_server_solver_factory("gb300_cuda")
    orch = server.JobOrchestrator(solver_factory=factory, artifact_root=tmp_path / "jobs")
    try:
        cfg = SimulationConfig(mesh_file=str(mesh_file), scale_factor=0.001, step_size=60.0,
                               radiators=(RadiatorConfig(name="cap", tag=2),), channels=(ChannelConfig(name="main"),))
        job = orch.submit(cfg, np.asarray([300.0, 600.0], np.float32))
        import time

        deadline = time.time() + 240
        while time.time() < deadline and orch.get(job.job_id).status not in server.TERMINAL_STATES:
            time.sleep(0.2)
        events, terminal = orch.events_since(job.job_id, 0)
        assert terminal, [e["type"] for e in events]
        types = [e["type"] for e in events]
        assert types == ["queued", "started", "initialized", "result", "result", "completed"], types
        assert orch.get(job.job_id).result_npz.exists()
    finally:
        orch.shutdown()


@pytest.fixture(scope="module")
def half_and_full_files(tmp_path_factory):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")  # 8 x 6 cells: grid line on x = 0
    half = meshes.fundamental_domain(box, "x")
    full, _ = meshes.mirror_to_full(half, "x")
    d = tmp_path_factory.mktemp("sym")
    paths = []
    for name, m in (("half.msh", half), ("full.msh", full)):
        meshes.write_gmsh22(d / name, m.vertices * 1000.0, m.faces, m.tags)
        paths.append(d / name)
    return paths


def test_symmetric_job_matches_full_model(half_and_full_files):
    half_file, full_file = half_and_full_files
    events = {}
    for name, path, sym in (("half", half_file, "x"), ("full", full_file, "off")):
        cfg = base_config(path, symmetry=sym, radiators=[{"name": "piston", "tag": 2, "channel": "main"}])
        job = job_mod.ExteriorJob({"config": cfg, "frequencies_hz": [800.0]}, engine_factory=oracle_factory)
        events[name] = next(job.results())["result"]
    h, f = events["half"], events["full"]
    assert h["diagnostics"]["symmetry"] == "x"
    for key in ("horizontal_pressure", "vertical_pressure"):
        a = np.asarray(h[key]["real"]) + 1j * np.asarray(h[key]["imag"])
        b = np.asarray(f[key]["real"]) + 1j * np.asarray(f[key]["imag"])
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 5e-5
    # impedance: the half model's radiator force times the reduction factor 2
    assert np.allclose(h["impedance"], f["impedance"], rtol=5e-5)


def test_job_solves_in_the_engines_preferred_chunks(mesh_file):
    """The frequency loop calls the engine once per preferred chunk (one full batch of the
    sweep on the CUDA engine); an engine without preferred_chunk gets chunks of 16."""
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    calls = []

    class Recording(oracle_engine.OracleEngine):
        def solve(self, freqs, sound_speed, rho):
            calls.append(len(freqs))
            return super().solve(freqs, sound_speed, rho)

    class Chunked(Recording):
        def preferred_chunk(self, n_freq):
            assert n_freq == 20
            return 7

    freqs = list(np.geomspace(100.0, 2000.0, 20))
    for cls, expect in ((Chunked, [7, 7, 6]), (Recording, [16, 4])):
        calls.clear()
        job = job_mod.ExteriorJob({"config": base_config(mesh_file), "frequencies_hz": freqs},
                                  engine_factory=lambda **kw: cls(**kw))
        out = list(job.results())
        job.close()
        assert calls == expect
        assert [e["solved_count"] for e in out] == list(range(1, 21))


def test_memory_admission_budget():
    """MemoryAdmission: a request that does not fit waits for a release; one larger than
    the whole budget is let through when nothing else is held."""
    import threading
    import time

    adm = backend_mod.MemoryAdmission(100)
    a = adm.acquire(60)
    got = []
    t = threading.Thread(target=lambda: got.append(adm.acquire(70)))
    t.start()
    time.sleep(0.2)
    assert not got and adm.free_bytes() == 40
    adm.release(a)
    t.join(5)
    assert got and adm.in_use() == 70
    adm.release(got[0])
    big = adm.acquire(500)  # larger than the budget: admitted alone
    assert adm.free_bytes() == -400
    adm.release(big)
    assert adm.free_bytes() == 100


def test_concurrent_sessions_hold_their_footprint(mesh_file):
    """With concurrent=True, sessions on two threads share one device admission: with a
    budget of 100 and footprints of 60 and 70 the second job solves only after the first
    has closed; with 200 they overlap.  Results equal the serial ones."""
    import threading
    import time

    timeline, lock = [], threading.Lock()

    class Engine:
        def __init__(self, **kw):
            self.inner = oracle_factory(**kw)
            self.n = None

        def prepare(self, vertices, faces, *a, **k):
            self.n = len(faces)
            self.inner.prepare(vertices, faces, *a, **k)

        def device_bytes(self, n_freq):
            return 60 if self.n == 80 else 70

        def solve(self, *a, **k):
            with lock:
                timeline.append(("solve", self.n))
            time.sleep(0.2)
            return self.inner.solve(*a, **k)

        def close(self):
            with lock:
                timeline.append(("close", self.n))

    small = meshes.sphere_with_cap(0.1, 1, 40.0)
    other = mesh_file.parent / "other.msh"
    meshes.write_gmsh22(other, small.vertices * 1500.0, small.faces[:-4], small.tags[:-4])
    for budget, serial in ((100, True), (200, False)):
        timeline.clear()
        backend_mod._admissions.pop(7, None)
        be = backend_mod.Gb300BemBackend(device=7, concurrent=True, memory_budget_bytes=budget,
                                         engine_factory=lambda **kw: Engine(**kw))
        outs = {}

        def run(path):
            req = contract.SolveRequest(base_config(path, step_size=90.0), np.asarray([300.0, 600.0], np.float32))
            outs[str(path)] = list(be.create_session(req).solve_stream())

        threads = [threading.Thread(target=run, args=(p,)) for p in (mesh_file, other)]
        for t in threads:
            t.start()
        for t in threads:
            t.join(120)
        assert len(outs) == 2 and all(len(v) == 2 for v in outs.values())
        first_close = min(i for i, e in enumerate(timeline) if e[0] == "close")
        closed = timeline[first_close][1]
        other_before = [e for e in timeline[:first_close] if e[0] == "solve" and e[1] != closed]
        assert (not other_before) if serial else other_before
    backend_mod._admissions.pop(7, None)
