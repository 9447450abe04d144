"""The job server (boundary-lab_gb300/job_server.py) on CPU.

Pinned against the reference's own job store: tests/golden/job_server_reference.json
and job_server_*.npz hold the events and result.npz artifacts that the reference's
JobOrchestrator (src/blab/server.py) produced for scripted solvers
(tests/golden/make_job_server_golden.py).  The same scripted solvers run here
through this server and must give the same events (timestamps and job ids
aside) and bitwise the same artifacts.  Then the HTTP interface: routes, status
codes, authentication, asset upload, and event windows read by many clients
at once while several jobs stream results.
"""

import base64
import io
import json
import sys
import threading
import time
import urllib.error
import urllib.request
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

TESTS = Path(__file__).resolve().parent
GOLDEN = TESTS / "golden"
sys.path.insert(0, str(GOLDEN))
import make_job_server_golden as scripted  # noqa: E402

js = pkg_module("job_server")
contract = pkg_module("contract")
meshes = pkg_module("meshes")

REFERENCE = json.loads((GOLDEN / "job_server_reference.json").read_text())["scenarios"]


def from_wire(raw):
    return contract.frequency_result_from_event(raw)


def wait_terminal(orch, job_id, timeout=30.0):
    deadline = time.time() + timeout
    while time.time() < deadline and orch.get(job_id).status not in js.TERMINAL_STATES:
        time.sleep(0.005)
    assert orch.get(job_id).status in js.TERMINAL_STATES


def run_scenario(tmp_path, name):
    sc = REFERENCE[name]
    solver = scripted.ScriptedSolver(sc, from_wire, pause_after=sc.get("cancel_after"), fail=sc.get("fail"))
    orch = js.JobOrchestrator(solver_factory=lambda cfg: solver, artifact_root=tmp_path)
    try:
        job = orch.submit({"distance": 2.0}, np.asarray([100.0, 200.0], np.float32))
        if sc.get("cancel_after") is not None:
            deadline = time.time() + 30
            while time.time() < deadline and len(orch.events_since(job.job_id, 0)[0]) < 3 + sc["cancel_after"]:
                time.sleep(0.005)
            orch.cancel(job.job_id)
            solver.release.set()
        wait_terminal(orch, job.job_id)
        lines, done = orch.lines_since(job.job_id, 0)
        assert done
        events = [json.loads(line) for line in lines]
        assert events == orch.events_since(job.job_id, 0)[0]  # the encoded lines are the stored records
        return scripted.normalise(events, job.job_id), orch.get(job.job_id).result_npz
    finally:
        orch.shutdown()


def assert_npz_equal(path_a, path_b):
    with np.load(path_a) as a, np.load(path_b) as b:
        assert list(a.keys()) == list(b.keys())
        for key in a.keys():
            assert a[key].dtype == b[key].dtype, key
            assert a[key].shape == b[key].shape, key
            np.testing.assert_array_equal(a[key], b[key], err_msg=key)


# ------------------------------------------------------ pinned to the reference --

@pytest.mark.parametrize("name", ["channels", "spl_only", "silent_channel", "cancelled", "failed"])
def test_events_and_artifact_match_reference(tmp_path, name):
    events, artifact = run_scenario(tmp_path, name)
    golden = REFERENCE[name]
    assert [e["type"] for e in events] == [e["type"] for e in golden["events"]]
    assert events == golden["events"]
    if golden["artifact"] is None:
        assert artifact is None
    else:
        assert_npz_equal(artifact, GOLDEN / golden["artifact"])


def test_queued_cancel_matches_reference(tmp_path):
    """A job cancelled while queued behind a running one: the same events as the reference's store
    (including its second "cancelled" when the worker picks the job up)."""
    events = scripted.run_queued_cancel(js.JobOrchestrator, js.TERMINAL_STATES, REFERENCE["spl_only"], from_wire)
    assert events == REFERENCE["queued_cancel"]["events"]


def test_writer_alone_matches_reference(tmp_path):
    """ResultDataset + write_result_artifact, no job loop: results added in stream order."""
    sc = REFERENCE["channels"]
    ds = js.ResultDataset(polar_angle_deg=np.asarray(sc["angles"], np.float32),
                          radiator_names=np.asarray(sc["radiator_names"]),
                          **{f"sphere_{k}": np.asarray(v, np.float32) for k, v in sc["sphere"].items()})
    for raw in sc["results"]:
        ds.add(from_wire(raw))
    out = js.write_result_artifact(ds, tmp_path / "x" / "result.npz")
    assert_npz_equal(out, GOLDEN / sc["artifact"])
    with np.load(out) as z:
        assert list(z["freq_hz"]) == sorted(r["freq_hz"] for r in sc["results"])
        assert z["sphere_spl_norm_db"].shape == (4, 20)
    assert js.write_result_artifact(js.ResultDataset(np.zeros(3, np.float32), np.asarray(["a"])),
                                    tmp_path / "none.npz") is None


def test_partial_sphere_sampling_drops_the_balloon(tmp_path):
    """One frequency without sphere data: the artifact has no sphere_* keys (live.py:197-208)."""
    sc = REFERENCE["spl_only"]
    ds = js.ResultDataset(polar_angle_deg=np.asarray(sc["angles"], np.float32),
                          radiator_names=np.asarray(sc["radiator_names"]),
                          **{f"sphere_{k}": np.asarray(v, np.float32) for k, v in sc["sphere"].items()})
    for i, raw in enumerate(sc["results"]):
        ds.add(from_wire({**raw, "sphere_spl_norm_db": None} if i == 1 else raw))
    with np.load(js.write_result_artifact(ds, tmp_path / "r.npz")) as z:
        assert not any(k.startswith("sphere_") for k in z.keys())
        assert z["impedance_real"].shape == (1, 3)


def test_reference_interpolation_wraps():
    angles = np.arange(-180.0, 181.0, 30.0, dtype=np.float32)
    vals = np.exp(1j * np.deg2rad(angles)).astype(np.complex64)
    assert js._reference_pressure(vals, angles, 0.0) == pytest.approx(1.0)
    # 370 deg wraps to 10 deg: a third of the way from 0 (index 6) to 30 (index 7)
    assert js._reference_pressure(vals, angles, 370.0) == pytest.approx((2 * vals[6] + vals[7]) / 3, abs=1e-6)
    # 195 deg wraps to -165 deg: halfway from -180 (index 0) to -150 (index 1)
    assert js._reference_pressure(vals, angles, 195.0) == pytest.approx((vals[0] + vals[1]) / 2, abs=1e-6)
    # the duplicated +180 column is dropped, so -175 deg interpolates towards -180, not past +180
    assert js._reference_pressure(vals, angles, -175.0) == pytest.approx((5 * vals[0] + vals[1]) / 6, abs=1e-6)
    assert js._reference_pressure(np.array([2 + 1j]), np.array([5.0]), 0.0) == 2 + 1j
    assert js._reference_pressure(np.zeros(0), np.zeros(0), 0.0) == 0j


# ------------------------------------------------------------ job store --

class GatedSolver:
    """Streams ``n`` results; waits for ``gate`` before the first when given."""

    def __init__(self, n=3, gate=None, delay_s=0.0, angles=7):
        self.n, self.gate, self.delay_s = n, gate, delay_s
        self.angles = np.linspace(-90, 90, angles).astype(np.float32)
        self.polar_angle_deg = self.angles
        self.radiator_names = np.asarray(["r"])
        self.sphere_metadata = None

    def solve_stream(self, freqs, *, stop_requested=None):
        if self.gate is not None:
            self.gate.wait(30)
        for i in range(self.n):
            if stop_requested is not None and stop_requested():
                return
            if self.delay_s:
                time.sleep(self.delay_s)
            z = np.full((1, self.angles.size), 0.1 * (i + 1), np.complex64)
            yield from_wire({"freq_hz": 100.0 * (i + 1), "horizontal_spl_norm_db": [0.0] * self.angles.size,
                             "vertical_spl_norm_db": [0.0] * self.angles.size, "impedance": [[1.0, 2.0]],
                             "channel_names": ["main"],
                             "horizontal_pressure": {"real": z.real.tolist(), "imag": z.imag.tolist()},
                             "vertical_pressure": {"real": z.real.tolist(), "imag": z.imag.tolist()}})


def test_submit_validation_and_capacity(tmp_path):
    gate = threading.Event()
    orch = js.JobOrchestrator(max_running_jobs=1, max_queued_jobs=1, max_frequencies=5, artifact_root=tmp_path,
                              solver_factory=lambda cfg: GatedSolver(gate=gate))
    try:
        with pytest.raises(ValueError, match="at least one"):
            orch.submit({}, [])
        with pytest.raises(ValueError, match="server limit is 5"):
            orch.submit({}, np.arange(1, 7))
        with pytest.raises(ValueError, match="finite, positive"):
            orch.submit({}, [100.0, -1.0])
        with pytest.raises(ValueError, match="finite, positive"):
            orch.submit({}, [np.nan])
        a = orch.submit({}, [100.0])
        b = orch.submit({}, [100.0])
        with pytest.raises(js.JobQueueFullError, match="1 running, 1 queued"):
            orch.submit({}, [100.0])
        assert orch.cancel(b.job_id)  # queued: cancelled at once
        assert [e["type"] for e in orch.events_since(b.job_id, 0)[0]] == ["queued", "cancelled"]
        assert orch.get(b.job_id).status == "cancelled"
        c = orch.submit({}, [100.0])  # room again
        gate.set()
        wait_terminal(orch, a.job_id)
        wait_terminal(orch, c.job_id)
        assert orch.get(a.job_id).status == "completed" and orch.get(c.job_id).status == "completed"
        assert orch.get(b.job_id).status == "cancelled"  # the pool does not run a cancelled job
        assert [e["type"] for e in orch.events_since(b.job_id, 0)[0]] == ["queued", "cancelled", "cancelled"]
        assert not orch.cancel("nope")
        with pytest.raises(KeyError):
            orch.events_since("nope", 0)
        snap = orch.get(a.job_id).snapshot()
        assert snap["artifacts"]["result_npz"] == f"/jobs/{a.job_id}/artifacts/result.npz"
        assert snap["solved_count"] == 3 and snap["total_count"] == 1 and snap["event_count"] == 7
    finally:
        gate.set()
        orch.shutdown()


def test_constructor_limits(tmp_path):
    for kw in ({"max_running_jobs": 0}, {"max_queued_jobs": -1}, {"max_asset_bytes": 0},
               {"max_frequencies": 0}, {"job_retention_hours": -1}):
        with pytest.raises(ValueError):
            js.JobOrchestrator(artifact_root=tmp_path, solver_factory=lambda cfg: None, **kw)


def test_wait_for_event_wakes_and_times_out(tmp_path):
    gate = threading.Event()
    orch = js.JobOrchestrator(artifact_root=tmp_path, solver_factory=lambda cfg: GatedSolver(gate=gate))
    try:
        job = orch.submit({}, [100.0])
        deadline = time.time() + 10
        while time.time() < deadline and len(orch.events_since(job.job_id, 0)[0]) < 3:
            time.sleep(0.005)
        t0 = time.monotonic()
        orch.wait_for_event(job.job_id, 3, timeout_s=0.2)  # nothing new: times out
        assert 0.15 < time.monotonic() - t0 < 2.0
        threading.Timer(0.1, gate.set).start()
        t0 = time.monotonic()
        orch.wait_for_event(job.job_id, 3, timeout_s=20.0)  # woken by the first result
        assert time.monotonic() - t0 < 5.0
        assert len(orch.events_since(job.job_id, 0)[0]) > 3
        wait_terminal(orch, job.job_id)
        t0 = time.monotonic()
        orch.wait_for_event(job.job_id, 10**6, timeout_s=20.0)  # ended: returns at once
        orch.wait_for_event("nope", 0, timeout_s=20.0)
        assert time.monotonic() - t0 < 1.0
    finally:
        gate.set()
        orch.shutdown()


def test_running_cancel_and_purge(tmp_path):
    gate = threading.Event()
    orch = js.JobOrchestrator(artifact_root=tmp_path, job_retention_hours=1.0,
                              solver_factory=lambda cfg: GatedSolver(n=50, gate=gate, delay_s=0.01))
    try:
        job = orch.submit({}, [100.0])
        deadline = time.time() + 10
        while time.time() < deadline and orch.get(job.job_id).status != "running":
            time.sleep(0.005)
        assert orch.cancel(job.job_id)
        gate.set()
        wait_terminal(orch, job.job_id)
        types = [e["type"] for e in orch.events_since(job.job_id, 0)[0]]
        assert types[-1] == "cancelled" and "cancelling" in types and "completed" not in types
        assert orch.get(job.job_id).result_npz is None
        done = orch.submit({}, [100.0])
        wait_terminal(orch, done.job_id)
        art_dir = orch.get(done.job_id).artifact_dir
        assert (art_dir / "result.npz").exists()
        assert orch.purge_expired_jobs(now=time.time()) == 0
        assert orch.purge_expired_jobs(now=time.time() + 7200) == 2
        assert orch.get(done.job_id) is None and not art_dir.exists()
    finally:
        gate.set()
        orch.shutdown()


# ------------------------------------------------------------------ HTTP --

class Http:
    def __init__(self, url, token=""):
        self.url, self.token = url, token

    def call(self, path, body=None, method=None, content_type="application/json", raw=False):
        data = None if body is None else (body if isinstance(body, bytes) else json.dumps(body).encode())
        req = urllib.request.Request(self.url + path, data=data, method=method or ("POST" if data else "GET"))
        if data is not None:
            req.add_header("Content-Type", content_type)
        if self.token:
            req.add_header("Authorization", f"Bearer {self.token}")
        try:
            with urllib.request.urlopen(req, timeout=30) as resp:
                payload = resp.read()
                return resp.status, (payload if raw else json.loads(payload))
        except urllib.error.HTTPError as exc:
            return exc.code, json.loads(exc.read())

    def events(self, job_id, since):
        with urllib.request.urlopen(urllib.request.Request(
                f"{self.url}/jobs/{job_id}/events?since={since}",
                headers={"Authorization": f"Bearer {self.token}"} if self.token else {}), timeout=30) as resp:
            assert resp.headers.get_content_type() == "application/x-ndjson"
            return [json.loads(line) for line in resp.read().splitlines() if line]


@pytest.fixture
def served(tmp_path):
    servers = []

    def start(solver_factory, *, token=None, window_s=25.0, max_request_bytes=js.DEFAULT_MAX_REQUEST_BYTES,
              **orch_kw):
        orch = js.JobOrchestrator(artifact_root=tmp_path / "jobs", solver_factory=solver_factory, **orch_kw)
        srv = js.JobHTTPServer(("127.0.0.1", 0), orch, access_token=token, event_stream_window_seconds=window_s,
                               max_request_bytes=max_request_bytes)
        threading.Thread(target=srv.serve_forever, daemon=True).start()
        servers.append((srv, orch))
        return Http(f"http://127.0.0.1:{srv.server_address[1]}", token or ""), orch

    yield start
    for srv, orch in servers:
        srv.shutdown()
        srv.server_close()
        orch.shutdown()


def test_http_routes_and_errors(served):
    captured = {}

    def factory(cfg):
        captured["config"] = cfg
        return GatedSolver(n=2)

    http, orch = served(factory, token="s3cret", max_request_bytes=4096, max_queued_jobs=1)
    assert Http(http.url).call("/health")[0] == 401
    assert Http(http.url, "wrong").call("/health")[0] == 401
    status, health = http.call("/health")
    assert status == 200 and health["status"] == "ok" and health["backend"] == "gb300_cuda"
    assert health["capabilities"]["supports_symmetry"] and health["capabilities"]["supports_streaming"]
    mesh_bytes = b"$MeshFormat\n2.2 0 8\n$EndMeshFormat\n"
    body = {"schema_version": 2, "config": {"mesh_file": "C:/proj/horn.msh", "distance": 2.0,
                                            "meshes": [{"name": "m", "file": "C:/proj/horn.msh"}]},
            "frequencies_hz": [200.0, 400.0],
            "assets": [{"original_path": "C:/proj/horn.msh", "filename": "horn (v2).msh",
                        "content_base64": base64.b64encode(mesh_bytes).decode()}]}
    status, snap = http.call("/jobs", body)
    assert status == 202 and snap["status"] in ("queued", "running", "completed") and snap["total_count"] == 2
    job_id = snap["job_id"]
    wait_terminal(orch, job_id)
    staged = Path(captured["config"]["mesh_file"])
    assert staged.name == "horn_v2_.msh" and staged.read_bytes() == mesh_bytes
    assert captured["config"]["meshes"][0]["file"] == str(staged)
    events = http.events(job_id, 0)
    assert [e["type"] for e in events] == ["queued", "started", "initialized", "result", "result", "completed"]
    assert [e["index"] for e in events] == list(range(6)) and all(e["job_id"] == job_id for e in events)
    assert http.events(job_id, 4) == events[4:] and http.events(job_id, -3) == events
    assert http.events(job_id, 99) == []
    status, data = http.call(f"/jobs/{job_id}/artifacts/result.npz", raw=True)
    assert status == 200 and data == orch.get(job_id).result_npz.read_bytes()
    status, snap = http.call(f"/jobs/{job_id}")
    assert status == 200 and snap["status"] == "completed" and snap["artifacts"]["result_npz"]
    assert http.call(f"/jobs/{job_id}/events?since=x")[0] == 400
    assert http.call("/jobs/nope")[0] == 404
    assert http.call("/jobs/nope/events")[0] == 404
    assert http.call("/jobs/nope/artifacts/result.npz")[0] == 404
    assert http.call("/jobs/nope/cancel", {"x": 1})[0] == 404
    assert http.call("/nowhere")[0] == 404
    assert http.call(f"/jobs/{job_id}/cancel", {"x": 1}) == (200, {"job_id": job_id, "status": "cancelling"})
    # malformed requests
    assert http.call("/jobs", {"config": {}})[0] == 400  # no frequencies_hz
    assert http.call("/jobs", {"frequencies_hz": [1.0]})[0] == 400  # no config
    assert http.call("/jobs", {"schema_version": 7, "config": {}, "frequencies_hz": [1.0]})[0] == 400
    assert http.call("/jobs", {"config": {}, "frequencies_hz": [1.0], "assets": {}})[0] == 400
    assert http.call("/jobs", {"config": {}, "frequencies_hz": [-1.0]})[0] == 400
    assert http.call("/jobs", b"[1, 2]")[0] == 400
    assert http.call("/jobs", b"{}", content_type="text/plain")[0] == 400
    bad_asset = {"config": {"mesh_file": "a.msh"}, "frequencies_hz": [1.0],
                 "assets": [{"original_path": "a.msh", "content_base64": "%%%"}]}
    status, err = http.call("/jobs", bad_asset)
    assert status == 400 and "not valid base64" in err["error"]
    status, err = http.call("/jobs", {"config": {"pad": "x" * 5000}, "frequencies_hz": [1.0]})
    assert status == 413 and "exceeds the server limit" in err["error"]


def test_http_capacity_is_503(served):
    gate = threading.Event()
    http, orch = served(lambda cfg: GatedSolver(gate=gate), max_running_jobs=1, max_queued_jobs=0)
    try:
        status, snap = http.call("/jobs", {"config": {}, "frequencies_hz": [100.0]})
        assert status == 202
        status, err = http.call("/jobs", {"config": {}, "frequencies_hz": [100.0]})
        assert status == 503 and "capacity is full" in err["error"]
    finally:
        gate.set()


def test_event_windows_under_load(served):
    """Six jobs of 120 results each stream on four workers while 24 clients read their event logs
    through 20 ms windows, reconnecting with since = last index + 1: every client sees every
    event exactly once, in order, byte for byte what the store holds."""
    n_jobs, n_results, clients_per_job = 6, 120, 4
    http, orch = served(lambda cfg: GatedSolver(n=n_results, delay_s=0.0005), window_s=0.02,
                        max_running_jobs=4, max_queued_jobs=8)
    job_ids = [http.call("/jobs", {"config": {}, "frequencies_hz": [100.0]})[1]["job_id"] for _ in range(n_jobs)]
    seen: dict[tuple, list] = {}
    windows: dict[tuple, int] = {}
    errors = []

    def client(job_id, c):
        got, n_windows, since = [], 0, 0
        try:
            while True:
                batch = http.events(job_id, since)
                n_windows += 1
                for e in batch:
                    assert e["index"] == since, (e["index"], since)
                    since += 1
                    got.append(e)
                if got and got[-1]["type"] in js.TERMINAL_STATES:
                    break
                assert n_windows < 100000
        except Exception as exc:  # noqa: BLE001 - reported by the main thread
            errors.append(repr(exc))
        seen[(job_id, c)] = got
        windows[(job_id, c)] = n_windows

    threads = [threading.Thread(target=client, args=(j, c)) for j in job_ids for c in range(clients_per_job)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(120)
    assert not errors, errors[:3]
    for job_id in job_ids:
        stored = [json.loads(line) for line in orch.lines_since(job_id, 0)[0]]
        assert len(stored) == n_results + 4
        assert [e["type"] for e in stored][-1] == "completed"
        for c in range(clients_per_job):
            assert seen[(job_id, c)] == stored
    assert max(windows.values()) > 1  # windows were cut and resumed
    for job_id in job_ids:
        status, data = http.call(f"/jobs/{job_id}/artifacts/result.npz", raw=True)
        assert status == 200
        with np.load(io.BytesIO(data)) as z:
            assert z["freq_hz"].shape == (n_results,)


# ------------------------------------- a real job on the CPU oracle engine --

@pytest.fixture(scope="module")
def mesh_file(tmp_path_factory):
    mesh = meshes.sphere_with_cap(0.1, 1, 40.0)  # 80 faces
    path = tmp_path_factory.mktemp("mesh") / "sphere.msh"
    meshes.write_gmsh22(path, mesh.vertices * 1000.0, mesh.faces, mesh.tags)
    return path


def oracle_factory(**kw):
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    return oracle_engine.make_engine(**kw)


def test_http_job_with_uploaded_mesh_on_the_oracle_engine(served, mesh_file):
    """POST a job whose mesh travels as an asset, stream its events, download result.npz; the
    artifact equals the one written from the streamed result events, and the per-frequency
    results equal a direct run of the same request."""
    http, orch = served(js.gb300_solver_factory(engine_factory=oracle_factory))
    cfg = {"mesh_file": "/client/box/sphere.msh", "scale_factor": 0.001, "rho": 1.205, "sound_speed": 343.0,
           "step_size": 30.0, "distance": 2.0, "radiators": [{"name": "cap", "tag": 2, "channel": "main"}],
           "channels": [{"name": "main"}], "spherical_sampling_enabled": True, "spherical_sampling_points": 12}
    body = {"schema_version": 2, "config": cfg, "frequencies_hz": [300.0, 900.0],
            "assets": [{"original_path": "/client/box/sphere.msh", "filename": "sphere.msh",
                        "content_base64": base64.b64encode(mesh_file.read_bytes()).decode()}]}
    status, snap = http.call("/jobs", body)
    assert status == 202
    wait_terminal(orch, snap["job_id"], timeout=240)
    events = http.events(snap["job_id"], 0)
    assert [e["type"] for e in events] == ["queued", "started", "initialized", "result", "result", "completed"]
    init = events[2]
    ds = js.ResultDataset(polar_angle_deg=np.asarray(init["polar_angle_deg"], np.float32),
                          radiator_names=np.asarray(init["radiator_names"]),
                          **{f"sphere_{k}": np.asarray(v, np.float32) for k, v in init["sphere_metadata"].items()})
    for e in events[3:5]:
        ds.add(from_wire(e["result"]))
    local = js.write_result_artifact(ds, orch.artifact_root / "local.npz")
    status, data = http.call(f"/jobs/{snap['job_id']}/artifacts/result.npz", raw=True)
    remote = orch.artifact_root / "remote.npz"
    remote.write_bytes(data)
    assert_npz_equal(remote, local)
    with np.load(remote) as z:
        assert z["sphere_spl_norm_db"].shape == (2, 12) and z["impedance_radiator_names"].tolist() == ["cap"]
    job_mod = pkg_module("job")
    direct = list(job_mod.ExteriorJob({"config": {**cfg, "mesh_file": str(mesh_file)},
                                       "frequencies_hz": [300.0, 900.0]}, engine_factory=oracle_factory).results())
    for e, d in zip(events[3:5], direct):
        for key in ("horizontal_spl_db", "vertical_spl_norm_db", "impedance", "horizontal_pressure"):
            assert e["result"][key] == json.loads(json.dumps(d["result"][key])), key


def test_artifact_matches_the_reference_server_on_the_same_job(served, mesh_file, tmp_path, monkeypatch):
    """The same request through the reference's own job server with this backend registered, and
    through this server: the two result.npz artifacts are equal key for key."""
    ref_src = Path("/root/reference/src")
    if not (ref_src / "blab").exists():
        pytest.skip("reference checkout not present")
    monkeypatch.syspath_prepend(str(ref_src))
    monkeypatch.setenv("GB300_BEM_ENGINE", "oracle_engine:make_engine")
    monkeypatch.syspath_prepend(str(TESTS))
    from blab import server
    from blab.config import ChannelConfig, RadiatorConfig, SimulationConfig

    pkg_module("backend").register_with_boundary_lab()
    ref_orch = server.JobOrchestrator(solver_factory=server.create_server_solver_factory("gb300_cuda"),
                                      artifact_root=tmp_path / "ref")
    try:
        cfg = SimulationConfig(mesh_file=str(mesh_file), scale_factor=0.001, step_size=45.0, rho=1.205,
                               radiators=(RadiatorConfig(name="cap", tag=2),), channels=(ChannelConfig(name="main"),),
                               spherical_sampling_enabled=True, spherical_sampling_points=10)
        ref_job = ref_orch.submit(cfg, np.asarray([350.0, 1100.0], np.float32))
        deadline = time.time() + 240
        while time.time() < deadline and ref_orch.get(ref_job.job_id).status not in server.TERMINAL_STATES:
            time.sleep(0.05)
        ref_npz = ref_orch.get(ref_job.job_id).result_npz
        assert ref_npz is not None
    finally:
        ref_orch.shutdown()
    from blab.protocol import simulation_config_to_dict

    http, orch = served(js.gb300_solver_factory())
    status, snap = http.call("/jobs", {"config": simulation_config_to_dict(cfg), "frequencies_hz": [350.0, 1100.0]})
    assert status == 202
    wait_terminal(orch, snap["job_id"], timeout=240)
    assert orch.get(snap["job_id"]).status == "completed", orch.get(snap["job_id"]).error
    assert_npz_equal(orch.get(snap["job_id"]).result_npz, ref_npz)


def test_cli_parses_and_builds(monkeypatch, tmp_path):
    """main() wires the options through (serve_forever replaced so it returns at once)."""
    seen = {}

    def fake_serve(self):
        seen["addr"] = self.server_address
        seen["window"] = self.event_stream_window_seconds
        seen["running"] = self.orchestrator.max_running_jobs

    monkeypatch.setattr(js.JobHTTPServer, "serve_forever", fake_serve)
    assert js.main(["--port", "0", "--max-running-jobs", "3", "--event-stream-window-seconds", "5",
                    "--artifact-dir", str(tmp_path)]) == 0
    assert seen["running"] == 3 and seen["window"] == 5.0 and seen["addr"][0] == "127.0.0.1"


def test_scenario_helpers_are_self_consistent():
    """The scripted solver replays exactly the recorded results (guards the fixture itself)."""
    sc = REFERENCE["channels"]
    solver = scripted.ScriptedSolver(sc, from_wire)
    got = [js.frequency_result_to_wire(r) for r in solver.solve_stream(None)]
    assert json.loads(json.dumps(got)) == sc["results"]


def test_dataclass_config_assets_are_staged(tmp_path):
    """A config object with mesh_file / meshes[].file attributes (the reference's SimulationConfig)
    gets its uploaded mesh paths rewritten like a dict config."""
    from dataclasses import dataclass

    @dataclass(frozen=True)
    class Mesh:
        name: str
        file: str

    @dataclass(frozen=True)
    class Config:
        mesh_file: str
        meshes: tuple
        distance: float = 2.0

    seen = {}

    def factory(cfg):
        seen["cfg"] = cfg
        return GatedSolver(n=1)

    orch = js.JobOrchestrator(artifact_root=tmp_path, solver_factory=factory)
    try:
        cfg = Config(mesh_file="/c/a.msh", meshes=(Mesh("m", "/c/a.msh"), Mesh("n", "/c/other.msh")))
        asset = {"original_path": "/c/a.msh", "filename": "a.msh", "content_base64": base64.b64encode(b"x").decode()}
        job = orch.submit(cfg, [100.0], [asset])
        wait_terminal(orch, job.job_id)
        got = seen["cfg"]
        assert isinstance(got, Config) and Path(got.mesh_file).read_bytes() == b"x"
        assert got.meshes[0].file == got.mesh_file and got.meshes[1].file == "/c/other.msh"
        assert orch.get(job.job_id).status == "completed"
    finally:
        orch.shutdown()


def test_memory_admission_serialises_jobs_that_do_not_fit(served, mesh_file, tmp_path):
    """Two real jobs (CPU oracle engine) whose footprints (60 and 70 units) do not fit together
    in a budget of 100: the second starts solving only after the first has closed.  A budget of
    200 lets them overlap.  MemoryAdmission itself: a job larger than the budget runs alone."""
    timeline = []
    lock = threading.Lock()

    class Engine:
        def __init__(self, **kw):
            sys.path.insert(0, str(TESTS))
            import oracle_engine

            self.inner = oracle_engine.make_engine(**kw)
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

    big = meshes.sphere_with_cap(0.1, 1, 40.0)
    other = tmp_path / "other.msh"
    v = big.vertices * 1.5
    meshes.write_gmsh22(other, v * 1000.0, big.faces[:-4], big.tags[:-4])
    for budget, serial in ((100, True), (200, False)):
        timeline.clear()
        http, orch = served(js.gb300_solver_factory(engine_factory=lambda **kw: Engine(**kw), memory_budget_bytes=budget),
                            max_running_jobs=2)
        ids = []
        for path in (mesh_file, other):
            cfg = {"mesh_file": str(path), "scale_factor": 0.001, "step_size": 90.0,
                   "radiators": [{"name": "cap", "tag": 2, "channel": "main"}], "channels": [{"name": "main"}]}
            ids.append(http.call("/jobs", {"config": cfg, "frequencies_hz": [300.0, 600.0]})[1]["job_id"])
        for j in ids:
            wait_terminal(orch, j, timeout=120)
            assert orch.get(j).status == "completed", orch.get(j).error
        first_close = min(i for i, e in enumerate(timeline) if e[0] == "close")
        solves_after = [e for e in timeline[first_close:] if e[0] == "solve"]
        closed = timeline[first_close][1]
        later_job_solves_before_close = [e for e in timeline[:first_close] if e[0] == "solve" and e[1] != closed]
        if serial:
            assert not later_job_solves_before_close and solves_after
        else:
            assert later_job_solves_before_close
    adm = js.MemoryAdmission(10)
    t = adm.acquire(50)  # larger than the budget: admitted when nothing else holds memory
    assert adm.free_bytes() == -40
    adm.release(t)
    assert adm.free_bytes() == 10
