"""Generate the job-server golden fixtures by running the reference's own job store.

Imports Boundary Lab's Python package from a checkout (``src/blab``) and runs its
``JobOrchestrator`` (src/blab/server.py:154-523) over scripted solvers that
replay fixed per-frequency results.  Records, per scenario:
  * the solver's metadata and the results it streams (float32 wire dicts),
  * every event the reference stores (timestamps dropped, the job id replaced by
    "<job>"),
  * the ``result.npz`` artifact the reference writes (copied next to this file).
Scenarios: two channels with sphere pressures on a full circle of angles
(wrap-around reference interpolation) streamed out of frequency order; SPL-only
results (no channel basis, a missing raw level, sphere levels); a silent
channel (flat-target correction falls back to 1) with a repeated frequency and
no sphere; a job cancelled after two results; a solver that fails; a job cancelled while
queued behind a running one.
Usage: python tests/golden/make_job_server_golden.py /path/to/boundary-lab
"""

from __future__ import annotations

import json
import shutil
import sys
import tempfile
import threading
import time
from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = Path(__file__).resolve().parent


def complex_rows(rng, n_rows, n_cols, scale=1.0):
    z = (rng.normal(size=(n_rows, n_cols)) + 1j * rng.normal(size=(n_rows, n_cols))) * scale
    return {"real": z.real.astype(np.float32).tolist(), "imag": z.imag.astype(np.float32).tolist()}


def f32(rng, *shape, loc=0.0, scale=10.0):
    return (rng.normal(size=shape) * scale + loc).astype(np.float32).tolist()


def scenario_channels(rng):
    angles = np.arange(-180.0, 181.0, 30.0)
    n = angles.size
    results = []
    for f in (800.0, 200.0, 3200.0, 400.0):
        results.append({
            "freq_hz": f, "horizontal_spl_norm_db": f32(rng, n), "vertical_spl_norm_db": f32(rng, n),
            "impedance": f32(rng, 2, 2, scale=400.0), "horizontal_spl_db": f32(rng, n, loc=90.0),
            "vertical_spl_db": f32(rng, n, loc=90.0), "sphere_spl_norm_db": f32(rng, 20),
            "channel_names": ["hf", "lf"],
            "horizontal_pressure": complex_rows(rng, 2, n, 0.3), "vertical_pressure": complex_rows(rng, 2, n, 0.3),
            "sphere_pressure": complex_rows(rng, 2, 20, 0.3),
            "timings": {"assembly_s": 0.01, "solve_s": 0.002, "field_s": 0.001},
            "diagnostics": {"convergence_info": 0, "message": "scripted", "backend": "scripted",
                            "symmetry": "off", "regular_assembly_mode": "scripted"},
        })
    sphere = {"r_distance_m": [2.0] * 20, "theta_polar_rad": np.linspace(0.1, 3.0, 20).tolist(),
              "phi_azimuth_rad": np.linspace(0.0, 6.0, 20).tolist()}
    return {"angles": angles.tolist(), "radiator_names": ["tweeter", "woofer"], "sphere": sphere,
            "results": results}


def scenario_spl_only(rng):
    angles = np.arange(0.0, 91.0, 15.0)
    n = angles.size
    results = []
    for i, f in enumerate((150.0, 1500.0, 600.0)):
        results.append({
            "freq_hz": f, "horizontal_spl_norm_db": f32(rng, n), "vertical_spl_norm_db": f32(rng, n),
            "impedance": f32(rng, 1, 2, scale=400.0),
            "horizontal_spl_db": None if i == 1 else f32(rng, n, loc=85.0),
            "vertical_spl_db": f32(rng, n, loc=85.0), "sphere_spl_norm_db": f32(rng, 6),
            "channel_names": None, "horizontal_pressure": None, "vertical_pressure": None, "sphere_pressure": None,
            "timings": {"assembly_s": 0.0, "solve_s": 0.0, "field_s": 0.0}, "diagnostics": None,
        })
    sphere = {"r_distance_m": [1.5] * 6, "theta_polar_rad": [0.2, 0.4, 0.6, 0.8, 1.0, 1.2],
              "phi_azimuth_rad": [0.0, 1.0, 2.0, 3.0, 4.0, 5.0]}
    return {"angles": angles.tolist(), "radiator_names": ["main"], "sphere": sphere, "results": results}


def scenario_silent_channel(rng):
    angles = np.arange(-90.0, 91.0, 10.0)
    n = angles.size
    results = []
    for f in (500.0, 250.0, 500.0):
        h = complex_rows(rng, 2, n, 0.5)
        v = complex_rows(rng, 2, n, 0.5)
        for rows in (h, v):
            rows["real"][1] = [0.0] * n
            rows["imag"][1] = [0.0] * n
        results.append({
            "freq_hz": f, "horizontal_spl_norm_db": f32(rng, n), "vertical_spl_norm_db": f32(rng, n),
            "impedance": f32(rng, 1, 2, scale=400.0), "horizontal_spl_db": f32(rng, n, loc=80.0),
            "vertical_spl_db": f32(rng, n, loc=80.0), "sphere_spl_norm_db": None,
            "channel_names": ["main", "aux"], "horizontal_pressure": h, "vertical_pressure": v,
            "sphere_pressure": None, "timings": {"assembly_s": 0.0, "solve_s": 0.0, "field_s": 0.0},
            "diagnostics": None,
        })
    return {"angles": angles.tolist(), "radiator_names": ["main"], "sphere": None, "results": results}


class ScriptedSolver:
    """Replays a scenario's results; optionally pauses after ``pause_after`` results until released."""

    def __init__(self, scenario, from_dict, pause_after=None, fail=None):
        self.s = scenario
        self.from_dict = from_dict
        self.pause_after = pause_after
        self.fail = fail
        self.release = threading.Event()

    def initialize(self, frequencies):
        if self.fail:
            raise RuntimeError(self.fail)

    @property
    def polar_angle_deg(self):
        return np.asarray(self.s["angles"], np.float32)

    @property
    def radiator_names(self):
        return np.asarray(self.s["radiator_names"])

    @property
    def sphere_metadata(self):
        sph = self.s["sphere"]
        return None if sph is None else {k: np.asarray(v, np.float32) for k, v in sph.items()}

    def solve_stream(self, frequencies, *, stop_requested=None):
        for i, raw in enumerate(self.s["results"]):
            if self.pause_after is not None and i == self.pause_after:
                self.release.wait(30)
            yield self.from_dict(raw)


def normalise(events, job_id):
    out = []
    for e in events:
        e = {k: v for k, v in e.items() if k != "timestamp"}
        e["job_id"] = "<job>"
        if "artifact" in e:
            e["artifact"] = e["artifact"].replace(job_id, "<job>")
        out.append(e)
    return out


def run(orch_cls, terminal, solver, cancel_after=None, timeout=30.0):
    tmp = Path(tempfile.mkdtemp(prefix="golden-jobs-"))
    orch = orch_cls(solver_factory=lambda cfg: solver, artifact_root=tmp)
    try:
        config = SimpleNamespace(distance=2.0, axial_offset=0.0, sound_speed=343.0)
        job = orch.submit(config, np.asarray([100.0, 200.0], np.float32))
        deadline = time.time() + timeout
        if cancel_after is not None:
            while time.time() < deadline and len(orch.events_since(job.job_id, 0)[0]) < 3 + cancel_after:
                time.sleep(0.01)
            orch.cancel(job.job_id)
            solver.release.set()
        while time.time() < deadline and orch.get(job.job_id).status not in terminal:
            time.sleep(0.01)
        events, done = orch.events_since(job.job_id, 0)
        assert done
        npz = orch.get(job.job_id).result_npz
        data = None if npz is None else npz.read_bytes()
        return normalise(events, job.job_id), data
    finally:
        orch.shutdown()
        shutil.rmtree(tmp, ignore_errors=True)


def run_queued_cancel(orch_cls, terminal, scenario, from_dict, timeout=30.0):
    """One worker: job A runs (held before its first result) while job B waits in the queue and
    is cancelled there; then A is released.  Returns B's events."""
    tmp = Path(tempfile.mkdtemp(prefix="golden-jobs-"))
    first = ScriptedSolver(scenario, from_dict, pause_after=0)
    made = []

    def factory(cfg):
        made.append(cfg)
        return first if len(made) == 1 else ScriptedSolver(scenario, from_dict)

    orch = orch_cls(max_running_jobs=1, max_queued_jobs=1, solver_factory=factory, artifact_root=tmp)
    try:
        config = SimpleNamespace(distance=2.0, axial_offset=0.0, sound_speed=343.0)
        a = orch.submit(config, np.asarray([100.0], np.float32))
        deadline = time.time() + timeout
        while time.time() < deadline and orch.get(a.job_id).status != "running":
            time.sleep(0.01)
        b = orch.submit(config, np.asarray([100.0], np.float32))
        orch.cancel(b.job_id)
        first.release.set()
        while time.time() < deadline and (orch.get(a.job_id).status not in terminal
                                          or len(orch.events_since(b.job_id, 0)[0]) < 3):
            time.sleep(0.01)
        return normalise(orch.events_since(b.job_id, 0)[0], b.job_id)
    finally:
        orch.shutdown()
        shutil.rmtree(tmp, ignore_errors=True)


def main(checkout: Path) -> None:
    sys.path.insert(0, str(checkout / "src"))
    from blab import server  # noqa: PLC0415
    from blab.protocol import frequency_result_from_dict  # noqa: PLC0415

    rng = np.random.default_rng(20260301)
    scenarios = {"channels": scenario_channels(rng), "spl_only": scenario_spl_only(rng),
                 "silent_channel": scenario_silent_channel(rng)}
    golden = {"source": "src/blab/server.py JobOrchestrator, run by tests/golden/make_job_server_golden.py",
              "scenarios": {}}
    for name, sc in scenarios.items():
        events, data = run(server.JobOrchestrator, server.TERMINAL_STATES,
                           ScriptedSolver(sc, frequency_result_from_dict))
        (HERE / f"job_server_{name}.npz").write_bytes(data)
        golden["scenarios"][name] = {**sc, "events": events, "artifact": f"job_server_{name}.npz"}
    events, data = run(server.JobOrchestrator, server.TERMINAL_STATES,
                       ScriptedSolver(scenarios["channels"], frequency_result_from_dict, pause_after=2),
                       cancel_after=2)
    assert data is None
    golden["scenarios"]["cancelled"] = {**scenarios["channels"], "cancel_after": 2, "events": events,
                                        "artifact": None}
    events, data = run(server.JobOrchestrator, server.TERMINAL_STATES,
                       ScriptedSolver(scenarios["spl_only"], frequency_result_from_dict, fail="mesh file not found"))
    golden["scenarios"]["failed"] = {**scenarios["spl_only"], "fail": "mesh file not found", "events": events,
                                     "artifact": None}
    # a job cancelled while queued: the reference stores "cancelled" at the cancel and again
    # when its worker later picks the job up (server.py:339-342, 369-374)
    golden["scenarios"]["queued_cancel"] = {
        "events": run_queued_cancel(server.JobOrchestrator, server.TERMINAL_STATES, scenarios["spl_only"],
                                    frequency_result_from_dict)}
    (HERE / "job_server_reference.json").write_text(json.dumps(golden, separators=(",", ":")))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(Path(sys.argv[1]))
