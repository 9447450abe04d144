"""The job server on the GPU: jobs posted over HTTP (mesh uploaded as an asset) run on
the CUDA engine, several at once on per-worker contexts, while clients read
their event windows.  Checks: the streamed results match the same request on
the FP64 CPU oracle within the field tolerance (relative 1e-5 on the complex
pressures at the observation points), jobs run side by side give bitwise the
same results as a job run alone, and each job's result.npz equals the
artifact written from its streamed events."""

import base64
import json
import sys
import threading
import time
import urllib.request
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
TESTS = Path(__file__).resolve().parent
js = pkg_module("job_server")
contract = pkg_module("contract")
meshes = pkg_module("meshes")
job_mod = pkg_module("job")


def oracle_factory(**kw):
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    return oracle_engine.make_engine(**kw)


def post(url, body):
    req = urllib.request.Request(url + "/jobs", data=json.dumps(body).encode(), method="POST",
                                 headers={"Content-Type": "application/json"})
    with urllib.request.urlopen(req, timeout=60) as resp:
        assert resp.status == 202
        return json.loads(resp.read())["job_id"]


def stream_all(url, job_id, timeout_s=600.0):
    """Read the job's events window after window until its terminal event."""
    got, since, deadline = [], 0, time.time() + timeout_s
    while time.time() < deadline:
        with urllib.request.urlopen(f"{url}/jobs/{job_id}/events?since={since}", timeout=60) as resp:
            for line in resp.read().splitlines():
                if line:
                    event = json.loads(line)
                    assert event["index"] == since
                    since += 1
                    got.append(event)
        if got and got[-1]["type"] in js.TERMINAL_STATES:
            return got
    raise AssertionError(f"job {job_id} did not finish")


def pressures(result):
    rows = [result["horizontal_pressure"], result["vertical_pressure"], result["sphere_pressure"]]
    return np.concatenate([np.asarray(r["real"], np.float64) + 1j * np.asarray(r["imag"], np.float64)
                           for r in rows], axis=1)


@pytest.fixture(scope="module")
def request_body(tmp_path_factory):
    mesh = meshes.sphere_with_cap(0.1, 2, 30.0)  # 320 faces
    path = tmp_path_factory.mktemp("mesh") / "sphere.msh"
    meshes.write_gmsh22(path, mesh.vertices * 1000.0, mesh.faces, mesh.tags)
    cfg = {"mesh_file": "/client/sphere.msh", "scale_factor": 0.001, "rho": 1.205, "sound_speed": 343.0,
           "step_size": 15.0, "distance": 2.0, "radiators": [{"name": "cap", "tag": 2, "channel": "main"}],
           "channels": [{"name": "main"}], "spherical_sampling_enabled": True, "spherical_sampling_points": 16}
    body = {"schema_version": 2, "config": cfg, "frequencies_hz": [250.0, 1200.0, 3100.0],
            "assets": [{"original_path": "/client/sphere.msh", "filename": "sphere.msh",
                        "content_base64": base64.b64encode(path.read_bytes()).decode()}]}
    return body, path


def test_http_jobs_on_the_gpu(native, tmp_path, request_body):
    body, mesh_path = request_body
    # with a memory budget, so every job's footprint is estimated on the device and admitted
    orch = js.JobOrchestrator(max_running_jobs=3, max_queued_jobs=4, artifact_root=tmp_path / "jobs",
                              solver_factory=js.gb300_solver_factory(memory_budget_bytes=64 << 30))
    srv = js.JobHTTPServer(("127.0.0.1", 0), orch, event_stream_window_seconds=0.5)
    threading.Thread(target=srv.serve_forever, daemon=True).start()
    url = f"http://127.0.0.1:{srv.server_address[1]}"
    try:
        alone_id = post(url, body)
        alone = stream_all(url, alone_id)
        ids = [post(url, body) for _ in range(4)]
        streams: dict[str, list] = {}
        readers = [threading.Thread(target=lambda j=j: streams.__setitem__(j, stream_all(url, j))) for j in ids]
        for t in readers:
            t.start()
        for t in readers:
            t.join(900)
        for job_id, events in [(alone_id, alone)] + [(j, streams[j]) for j in ids]:
            assert [e["type"] for e in events] == ["queued", "started", "initialized", "result", "result", "result",
                                                   "completed"], (job_id, orch.get(job_id).error)
        # bitwise the same alone and side by side (timings aside)
        for j in ids:
            for a, b in zip(alone[3:6], streams[j][3:6]):
                ra = {k: v for k, v in a["result"].items() if k not in ("timings", "diagnostics")}
                rb = {k: v for k, v in b["result"].items() if k not in ("timings", "diagnostics")}
                assert ra == rb
        # the artifact is the one written from the streamed events
        init = alone[2]
        ds = js.ResultDataset(polar_angle_deg=np.asarray(init["polar_angle_deg"], np.float32),
                              radiator_names=np.asarray(init["radiator_names"]),
                              **{f"sphere_{k}": np.asarray(v, np.float32)
                                 for k, v in init["sphere_metadata"].items()})
        for e in alone[3:6]:
            ds.add(contract.frequency_result_from_event(e["result"]))
        local = js.write_result_artifact(ds, tmp_path / "local.npz")
        with urllib.request.urlopen(f"{url}/jobs/{alone_id}/artifacts/result.npz", timeout=60) as resp:
            (tmp_path / "remote.npz").write_bytes(resp.read())
        with np.load(local) as a, np.load(tmp_path / "remote.npz") as b:
            assert list(a.keys()) == list(b.keys())
            for key in a.keys():
                np.testing.assert_array_equal(a[key], b[key], err_msg=key)
        assert alone[3]["result"]["diagnostics"]["backend"] == "gb300_cuda"
    finally:
        srv.shutdown()
        srv.server_close()
        orch.shutdown()

    # the same request on the FP64 CPU oracle
    ref = list(job_mod.ExteriorJob({"config": {**body["config"], "mesh_file": str(mesh_path)},
                                    "frequencies_hz": body["frequencies_hz"]}, engine_factory=oracle_factory).results())
    for got, want in zip(alone[3:6], ref):
        p, q = pressures(got["result"]), pressures(want["result"])
        assert np.linalg.norm(p - q) / np.linalg.norm(q) < 1e-5, got["result"]["freq_hz"]
        imp_g = np.asarray(got["result"]["impedance"])
        imp_w = np.asarray(want["result"]["impedance"])
        assert np.linalg.norm(imp_g - imp_w) / np.linalg.norm(imp_w) < 1e-5
