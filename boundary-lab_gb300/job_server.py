"""HTTP job server for exterior solves on one GB300: the reference's job server
(src/blab/server.py) with this backend behind it.

Same interface as the reference, route for route:

  GET  /health                           server, solver and capability summary
  POST /jobs                             {"schema_version", "config", "frequencies_hz", "assets"} -> 202 + snapshot
  GET  /jobs/{id}                        job snapshot
  GET  /jobs/{id}/events?since=N         NDJSON event window (server.py:651-678)
  GET  /jobs/{id}/artifacts/result.npz   the compressed result artifact (server.py:477-511)
  POST /jobs/{id}/cancel                 cooperative cancel

with the same status codes (400 bad request, 401 missing bearer token, 404,
413 request too large, 503 capacity full), event records (``index``,
``job_id``, ``type``, ``timestamp`` plus the payload of server.py:330-475) and
the same ``result.npz`` keys and arrays.

What differs is how the work is carried:

* every worker thread of the pool solves on its own library context (its own
  CUDA stream and scratch), so ``max_running_jobs`` jobs share the GPU at the
  same time instead of queueing behind one solver process;
* each job has its own condition variable on the store's lock, so an appended
  event wakes only the streams reading that job (the reference wakes every
  waiting stream of every job);
* each event is encoded to its NDJSON line once, when it is appended, and the
  same bytes go to every client that reads the window.

Results do not depend on the load: each job's frequencies are solved by the
same deterministic kernels whatever runs beside it.
"""

from __future__ import annotations

import argparse
import base64
import dataclasses
import hmac
import json
import logging
import re
import shutil
import threading
import time
import uuid
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from http import HTTPStatus
from http.server import BaseHTTPRequestHandler, ThreadingHTTPServer
from pathlib import Path
from typing import Any, Callable
from urllib.parse import parse_qs, urlparse

import numpy as np

from . import contract

TERMINAL_STATES = {"completed", "cancelled", "failed"}
DEFAULT_ARTIFACT_ROOT = Path("runs") / "server_jobs"
MEBIBYTE = 1024 * 1024
DEFAULT_MAX_REQUEST_BYTES = 20 * MEBIBYTE
DEFAULT_MAX_ASSET_BYTES = 14 * MEBIBYTE
DEFAULT_MAX_FREQUENCIES = 1000
DEFAULT_MAX_QUEUED_JOBS = 4
DEFAULT_JOB_RETENTION_HOURS = 24.0
DEFAULT_EVENT_STREAM_WINDOW_SECONDS = 25.0
PROTOCOL_VERSION = 2
REFERENCE_PRESSURE_PA = 20e-6
ASSET_NAME_UNSAFE = re.compile(r"[^A-Za-z0-9._-]+")
LOGGER = logging.getLogger("gb300_bem.job_server")


class JobQueueFullError(RuntimeError):
    """Raised when running + queued jobs are at capacity (server.py:216-223)."""


class RequestTooLargeError(ValueError):
    """Raised before an oversized request body is read (server.py:709-712)."""


# --------------------------------------------------------------------- wire --
# The float32 wire of src/blab/protocol.py:170-218.

def ndarray_to_wire(array) -> list | None:
    return None if array is None else np.asarray(array, dtype=np.float32).tolist()


def complex_ndarray_to_wire(array) -> dict | None:
    if array is None:
        return None
    values = np.asarray(array, dtype=np.complex64)
    return {"real": values.real.astype(np.float32).tolist(), "imag": values.imag.astype(np.float32).tolist()}


def frequency_result_to_wire(result) -> dict:
    """The `result` payload of a FrequencyResult (protocol.py:202-218, 220-248)."""
    timings = result.timings
    diagnostics = result.diagnostics
    return {
        "freq_hz": float(result.freq_hz),
        "horizontal_spl_norm_db": ndarray_to_wire(result.horizontal_spl_norm_db),
        "vertical_spl_norm_db": ndarray_to_wire(result.vertical_spl_norm_db),
        "impedance": ndarray_to_wire(result.impedance),
        "horizontal_spl_db": ndarray_to_wire(result.horizontal_spl_db),
        "vertical_spl_db": ndarray_to_wire(result.vertical_spl_db),
        "sphere_spl_norm_db": ndarray_to_wire(result.sphere_spl_norm_db),
        "channel_names": None if result.channel_names is None else [str(n) for n in result.channel_names],
        "horizontal_pressure": complex_ndarray_to_wire(result.horizontal_pressure),
        "vertical_pressure": complex_ndarray_to_wire(result.vertical_pressure),
        "sphere_pressure": complex_ndarray_to_wire(result.sphere_pressure),
        "timings": {
            "assembly_s": float(getattr(timings, "assembly_s", 0.0)),
            "solve_s": float(getattr(timings, "solve_s", 0.0)),
            "field_s": float(getattr(timings, "field_s", 0.0)),
        },
        "diagnostics": None if diagnostics is None else {
            "convergence_info": diagnostics.convergence_info,
            "message": diagnostics.message,
            "backend": diagnostics.backend,
            "symmetry": diagnostics.symmetry,
            "regular_assembly_mode": diagnostics.regular_assembly_mode,
        },
    }


def solve_request_to_job_inputs(raw: dict) -> tuple[dict, np.ndarray, list]:
    """(config, frequencies, assets) of a POST /jobs body (protocol.py:281-301)."""
    if int(raw.get("schema_version", PROTOCOL_VERSION)) not in (1, PROTOCOL_VERSION):
        raise ValueError(f"Unsupported solve request schema_version {raw.get('schema_version')}.")
    if "config" not in raw:
        raise ValueError("Solve request must include config.")
    if "frequencies_hz" not in raw:
        raise ValueError("Solve request must include frequencies_hz.")
    config = raw["config"]
    if not isinstance(config, dict):
        raise ValueError("Solve request config must be an object.")
    assets = raw.get("assets", [])
    if assets is None:
        assets = []
    if not isinstance(assets, list):
        raise ValueError("Solve request assets must be a list.")
    return dict(config), np.asarray(raw["frequencies_hz"], dtype=np.float32), assets


# ----------------------------------------------------------------- artifact --
# The server's result.npz (server.py:477-511) from the per-frequency results.  The
# server builds its dataset without channel edits, so every channel is driven at
# unit gain and the flat-target corrections are taken at 0 degrees
# (live.py:24-36, 210-237; channel_synthesis.py:36-116).  Each array goes
# through the same numpy operations in the same dtypes as there (complex64
# pressures, float32 levels), so the artifact is bitwise the reference's.

def _reference_pressure(values: np.ndarray, angles_deg: np.ndarray, reference_angle_deg: float) -> complex:
    """Complex pressure at the reference angle, linear in angle with 360-degree wrap
    (channel_synthesis.py:132-160)."""
    angles = np.asarray(angles_deg, dtype=float)
    vals = np.asarray(values, dtype=np.complex64)
    if angles.size == 0:
        return 0j
    if angles.size == 1:
        return complex(vals[0])
    target = ((float(reference_angle_deg) + 180.0) % 360.0) - 180.0
    if np.isclose(angles[0], -180.0) and np.isclose(angles[-1], 180.0):
        angles, vals = angles[:-1], vals[:-1]
    xp = np.concatenate([angles - 360.0, angles, angles + 360.0])
    fp = np.concatenate([vals, vals, vals])
    return complex(np.interp(target, xp, fp.real), np.interp(target, xp, fp.imag))


def _flat_target_corrections(pressure: np.ndarray, angles_deg: np.ndarray, reference_angle_deg: float,
                             enabled: bool = True, floor_pa: float = 1e-12) -> np.ndarray:
    """Per-channel 1/|p(reference angle)| in float32, 1 where that is not finite or below the
    floor (channel_synthesis.py:51-73)."""
    if not enabled:
        return np.ones(pressure.shape[0], dtype=np.float32)
    mags = np.abs(np.asarray([_reference_pressure(row, angles_deg, reference_angle_deg) for row in pressure]))
    keep = np.isfinite(mags) & (mags > floor_pa)
    out = np.ones(pressure.shape[0], dtype=np.float32)
    out[keep] = (1.0 / mags[keep]).astype(np.float32)
    return out


def _spl(pressure: np.ndarray) -> np.ndarray:
    return 20.0 * np.log10(np.abs(pressure) / REFERENCE_PRESSURE_PA)


def _has_channel_basis(result) -> bool:
    return (result.channel_names is not None and result.horizontal_pressure is not None
            and result.vertical_pressure is not None)


@dataclass
class ResultDataset:
    """Per-frequency results of one job, keyed (and later ordered) by frequency (live.py:24-63)."""

    polar_angle_deg: np.ndarray
    radiator_names: np.ndarray
    polar_observation_distance_m: float = 0.0
    exterior_sound_speed_m_per_s: float = 343.0
    sphere_r_distance_m: np.ndarray | None = None
    sphere_theta_polar_rad: np.ndarray | None = None
    sphere_phi_azimuth_rad: np.ndarray | None = None
    flat_target_reference_angle_deg: float = 0.0
    flat_target_normalization_enabled: bool = True
    results: dict = field(default_factory=dict)

    def add(self, result) -> None:
        self.results[float(result.freq_hz)] = result

    def ordered_results(self) -> list:
        return [self.results[f] for f in sorted(self.results)]

    @property
    def solved_count(self) -> int:
        return len(self.results)

    def _unit_drive_weights(self, result) -> tuple[np.ndarray, np.ndarray]:
        horizontal = np.asarray(result.horizontal_pressure, dtype=np.complex64)
        angles = np.asarray(self.polar_angle_deg, dtype=np.float32)
        corrections = _flat_target_corrections(horizontal, angles, self.flat_target_reference_angle_deg,
                                               enabled=self.flat_target_normalization_enabled)
        # a channel without edits has drive exactly 1 (level 0 dB, polarity +1, no delay, no filters)
        return np.asarray([corrections[i] for i in range(horizontal.shape[0])], dtype=np.complex64), angles

    def _synthesis(self, result, with_sphere: bool) -> dict:
        weights, angles = self._unit_drive_weights(result)
        horizontal = np.asarray(result.horizontal_pressure, dtype=np.complex64)
        vertical = np.asarray(result.vertical_pressure, dtype=np.complex64)
        h_spl = _spl(np.sum(horizontal * weights[:, np.newaxis], axis=0))
        v_spl = _spl(np.sum(vertical * weights[:, np.newaxis], axis=0))
        ref = h_spl[int(np.argmin(np.abs(angles)))]
        out = {"h": h_spl.astype(np.float32), "v": v_spl.astype(np.float32),
               "h_norm": (h_spl - ref).astype(np.float32), "v_norm": (v_spl - ref).astype(np.float32)}
        if with_sphere and result.sphere_pressure is not None:
            sphere = np.asarray(result.sphere_pressure, dtype=np.complex64)
            out["sphere_norm"] = (_spl(np.sum(sphere * weights[:, np.newaxis], axis=0)) - ref).astype(np.float32)
        return out

    def polar_arrays(self) -> tuple[np.ndarray, ...]:
        """(freqs, angles, horizontal_norm, vertical_norm, horizontal_raw, vertical_raw), rows in
        frequency order (live.py:65-87)."""
        if not self.results:
            raise ValueError("No solved polar data available.")
        rows = []
        for r in self.ordered_results():
            if _has_channel_basis(r):
                s = self._synthesis(r, with_sphere=False)
                rows.append((s["h_norm"], s["v_norm"], s["h"], s["v"]))
            else:
                rows.append((r.horizontal_spl_norm_db, r.vertical_spl_norm_db,
                             r.horizontal_spl_db if r.horizontal_spl_db is not None else r.horizontal_spl_norm_db,
                             r.vertical_spl_db if r.vertical_spl_db is not None else r.vertical_spl_norm_db))
        freqs = np.asarray([r.freq_hz for r in self.ordered_results()], dtype=np.float32)
        stacked = [np.vstack([row[i] for row in rows]).astype(np.float32, copy=False) for i in range(4)]
        return (freqs, self.polar_angle_deg.astype(np.float32, copy=False), *stacked)

    def balloon_bundle(self) -> dict | None:
        """Sphere sampling of every frequency, or None when any frequency lacks it (live.py:175-208)."""
        if (not self.results or self.sphere_r_distance_m is None or self.sphere_theta_polar_rad is None
                or self.sphere_phi_azimuth_rad is None):
            return None
        if not all((_has_channel_basis(r) and r.sphere_pressure is not None) or r.sphere_spl_norm_db is not None
                   for r in self.results.values()):
            return None
        rows = []
        for r in self.ordered_results():
            if _has_channel_basis(r) and r.sphere_pressure is not None:
                rows.append(self._synthesis(r, with_sphere=True)["sphere_norm"])
            else:
                rows.append(r.sphere_spl_norm_db)
            if rows[-1] is None:
                return None
        return {
            "r_distance_m": np.asarray(self.sphere_r_distance_m, dtype=np.float32),
            "theta_polar_rad": np.asarray(self.sphere_theta_polar_rad, dtype=np.float32),
            "phi_azimuth_rad": np.asarray(self.sphere_phi_azimuth_rad, dtype=np.float32),
            "spl_norm": np.vstack(rows).astype(np.float32, copy=False),
        }


def write_result_artifact(dataset: ResultDataset | None, output_path: Path) -> Path | None:
    """Write ``result.npz`` (np.savez_compressed) with the keys of server.py:484-510; None when
    nothing was solved."""
    if dataset is None or dataset.solved_count == 0:
        return None
    output_path = Path(output_path)
    output_path.parent.mkdir(parents=True, exist_ok=True)
    freqs, angles, h_norm, v_norm, h_raw, v_raw = dataset.polar_arrays()
    impedance = np.stack([r.impedance for r in dataset.ordered_results()], axis=1)
    bundle: dict[str, Any] = {
        "freq_hz": freqs,
        "polar_angle_deg": angles,
        "horizontal_spl_db": h_raw,
        "vertical_spl_db": v_raw,
        "horizontal_spl_norm_db": h_norm,
        "vertical_spl_norm_db": v_norm,
        "impedance_freq_hz": freqs,
        "impedance_radiator_names": dataset.radiator_names,
        "impedance_real": impedance[:, :, 0],
        "impedance_imag": impedance[:, :, 1],
    }
    balloon = dataset.balloon_bundle()
    if balloon is not None:
        bundle["sphere_r_distance_m"] = balloon["r_distance_m"]
        bundle["sphere_theta_polar_rad"] = balloon["theta_polar_rad"]
        bundle["sphere_phi_azimuth_rad"] = balloon["phi_azimuth_rad"]
        bundle["sphere_spl_norm_db"] = balloon["spl_norm"]
    np.savez_compressed(output_path, **bundle)
    return output_path


# ------------------------------------------------------------------- solver --

def _server_engine_factory(**kwargs):
    from .engine import engine_from_env  # noqa: PLC0415 - the CUDA library loads on first use

    return engine_from_env(context="thread", **kwargs)


class MemoryAdmission:
    """Device-memory admission shared by the jobs of one server: a job holds its estimated
    footprint (mesh caches plus one frequency batch) from mesh upload to the end of its solve,
    and waits while it does not fit beside the running jobs.  A job larger than the whole
    budget runs when nothing else holds memory."""

    def __init__(self, budget_bytes: int):
        if budget_bytes <= 0:
            raise ValueError("budget_bytes must be > 0")
        self.budget = int(budget_bytes)
        self.used = 0
        self.holders = 0
        self._cond = threading.Condition()

    def free_bytes(self) -> int:
        with self._cond:
            return self.budget - self.used

    def acquire(self, nbytes: int) -> int:
        nbytes = max(0, int(nbytes))
        with self._cond:
            while self.holders > 0 and self.used + nbytes > self.budget:
                self._cond.wait()
            self.used += nbytes
            self.holders += 1
        return nbytes

    def release(self, token: int) -> None:
        with self._cond:
            self.used -= int(token)
            self.holders -= 1
            self._cond.notify_all()


def default_memory_budget(device: int) -> int:
    """85% of the device memory free now (torch's view of the device); 64 GiB without one."""
    try:
        import torch  # noqa: PLC0415

        free, _total = torch.cuda.mem_get_info(device)
        return int(0.85 * free)
    except Exception:  # noqa: BLE001 - no torch or no GPU
        return 64 << 30


class ServerSolver:
    """A job's solve session behind the interface the job loop uses (server.py:63-109):
    ``initialize(frequencies)``, the metadata properties, ``solve_stream``."""

    def __init__(self, config: dict, *, precision: str = "mixed", device: int = 0, batch: int = 0,
                 engine_factory: Callable | None = None, admission: MemoryAdmission | None = None):
        self.config = config
        self.precision = precision
        self.device = device
        self.batch = batch
        self.engine_factory = engine_factory or _server_engine_factory
        self.admission = admission
        self.status_callback: Callable[[str], None] | None = None
        self.session = None

    def set_status_callback(self, callback) -> None:
        self.status_callback = callback

    def initialize(self, frequencies_hz) -> None:
        from .backend import Gb300BemSession  # noqa: PLC0415

        request = contract.SolveRequest(self.config, np.asarray(frequencies_hz, dtype=np.float32),
                                        status_callback=self.status_callback)
        self.session = Gb300BemSession(request, engine_factory=self.engine_factory, precision=self.precision,
                                       device=self.device, batch=self.batch, admission=self.admission)

    def _meta(self):
        if self.session is None:
            raise RuntimeError("Server solver has not initialized.")
        return self.session.metadata

    @property
    def polar_angle_deg(self) -> np.ndarray:
        return self._meta().polar_angle_deg

    @property
    def radiator_names(self) -> np.ndarray:
        return self._meta().radiator_names

    @property
    def sphere_metadata(self) -> dict | None:
        return self._meta().sphere_metadata

    def solve_stream(self, frequencies, *, stop_requested=None):
        if self.session is None:
            self.initialize(np.asarray(frequencies, dtype=np.float32))
        yield from self.session.solve_stream(stop_requested=stop_requested)


def gb300_solver_factory(*, precision: str = "mixed", device: int = 0, batch: int = 0,
                         engine_factory: Callable | None = None,
                         memory_budget_bytes: int | None = None) -> Callable[[dict], ServerSolver]:
    """Solvers for the job loop.  With a memory budget, every solver this factory makes shares
    one MemoryAdmission, so concurrent jobs start their solves only when they fit."""
    admission = MemoryAdmission(memory_budget_bytes) if memory_budget_bytes else None
    return lambda config: ServerSolver(config, precision=precision, device=device, batch=batch,
                                       engine_factory=engine_factory, admission=admission)


# -------------------------------------------------------------- job store ---

@dataclass(eq=False)
class JobRecord:
    """One job and its event log (server.py:112-151)."""

    job_id: str
    config: dict
    frequencies_hz: np.ndarray
    artifact_dir: Path
    status: str = "queued"
    created_at: float = field(default_factory=time.time)
    started_at: float | None = None
    finished_at: float | None = None
    error: str | None = None
    solved_count: int = 0
    event_count: int = 0
    result_npz: Path | None = None
    cancel_event: threading.Event = field(default_factory=threading.Event)
    events: list = field(default_factory=list)
    lines: list = field(default_factory=list)   # events[i] encoded once as its NDJSON line
    dataset: ResultDataset | None = None
    changed: threading.Condition | None = None

    @property
    def total_count(self) -> int:
        return int(self.frequencies_hz.size)

    def snapshot(self) -> dict:
        return {
            "job_id": self.job_id,
            "status": self.status,
            "created_at": self.created_at,
            "started_at": self.started_at,
            "finished_at": self.finished_at,
            "error": self.error,
            "solved_count": self.solved_count,
            "total_count": self.total_count,
            "event_count": self.event_count,
            "artifacts": {
                "result_npz": None if self.result_npz is None else f"/jobs/{self.job_id}/artifacts/result.npz",
            },
        }


def _config_value(config, key: str, default):
    """A field of a request config: a dict (the wire form) or an object with attributes (the
    reference's SimulationConfig)."""
    if isinstance(config, dict):
        return config.get(key, default)
    return getattr(config, key, default)


def _safe_asset_filename(filename: str, index: int) -> str:
    cleaned = ASSET_NAME_UNSAFE.sub("_", Path(filename).name).strip("._")
    return cleaned or f"asset_{index}.msh"


def _rewrite_mesh_paths(config, staged: dict[str, str]):
    """The config with every uploaded mesh path replaced by its staged copy (server.py:847-850);
    a dict config gives a dict, a dataclass config (the reference's SimulationConfig) a copy."""
    if dataclasses.is_dataclass(config) and not isinstance(config, type):
        meshes = tuple(dataclasses.replace(m, file=staged.get(m.file, m.file)) for m in getattr(config, "meshes", ()))
        return dataclasses.replace(config, mesh_file=staged.get(config.mesh_file, config.mesh_file), meshes=meshes)
    out = dict(config)
    if out.get("mesh_file") in staged:
        out["mesh_file"] = staged[out["mesh_file"]]
    if isinstance(out.get("meshes"), (list, tuple)):
        meshes = []
        for mesh in out["meshes"]:
            if isinstance(mesh, dict) and mesh.get("file") in staged:
                mesh = {**mesh, "file": staged[mesh["file"]]}
            meshes.append(mesh)
        out["meshes"] = meshes
    return out


class JobOrchestrator:
    """Bounded job queue, worker pool and event store (server.py:154-523)."""

    def __init__(self, *, max_running_jobs: int = 1, max_queued_jobs: int = DEFAULT_MAX_QUEUED_JOBS,
                 max_asset_bytes: int = DEFAULT_MAX_ASSET_BYTES, max_frequencies: int = DEFAULT_MAX_FREQUENCIES,
                 job_retention_hours: float = DEFAULT_JOB_RETENTION_HOURS,
                 artifact_root: Path = DEFAULT_ARTIFACT_ROOT, solver_factory: Callable | None = None):
        if max_running_jobs < 1:
            raise ValueError("max_running_jobs must be >= 1.")
        if max_queued_jobs < 0:
            raise ValueError("max_queued_jobs must be >= 0.")
        if max_asset_bytes < 1:
            raise ValueError("max_asset_bytes must be >= 1.")
        if max_frequencies < 1:
            raise ValueError("max_frequencies must be >= 1.")
        if job_retention_hours < 0:
            raise ValueError("job_retention_hours must be >= 0.")
        self.artifact_root = Path(artifact_root)
        self.solver_factory = solver_factory or gb300_solver_factory()
        self.max_running_jobs = max_running_jobs
        self.max_queued_jobs = max_queued_jobs
        self.max_asset_bytes = max_asset_bytes
        self.max_frequencies = max_frequencies
        self.job_retention_seconds = job_retention_hours * 3600.0
        self._executor = ThreadPoolExecutor(max_workers=max_running_jobs, thread_name_prefix="gb300-bem-job")
        self._jobs: dict[str, JobRecord] = {}
        self._submitting = 0
        self._lock = threading.RLock()

    # -- submission ---------------------------------------------------------
    def submit(self, config: dict, frequencies_hz, assets: list | None = None) -> JobRecord:
        self.purge_expired_jobs()
        freqs = np.asarray(frequencies_hz, dtype=np.float32).reshape(-1)
        if freqs.size == 0:
            raise ValueError("frequencies_hz must contain at least one frequency.")
        if freqs.size > self.max_frequencies:
            raise ValueError(f"frequencies_hz contains {freqs.size} values; the server limit is "
                             f"{self.max_frequencies}.")
        if not np.all(np.isfinite(freqs)) or np.any(freqs <= 0):
            raise ValueError("frequencies_hz must contain only finite, positive values.")
        with self._lock:
            active = sum(job.status not in TERMINAL_STATES for job in self._jobs.values())
            if active + self._submitting >= self.max_running_jobs + self.max_queued_jobs:
                raise JobQueueFullError(f"Server job capacity is full ({self.max_running_jobs} running, "
                                        f"{self.max_queued_jobs} queued).")
            self._submitting += 1
        job_id = uuid.uuid4().hex
        artifact_dir = self.artifact_root / job_id
        try:
            if assets:
                config = self._stage_assets(config, assets, artifact_dir / "assets")
            job = JobRecord(job_id=job_id, config=config, frequencies_hz=freqs, artifact_dir=artifact_dir)
            job.changed = threading.Condition(self._lock)
            with self._lock:
                self._submitting -= 1
                self._jobs[job_id] = job
                self._add_event_locked(job, "queued", total_count=job.total_count)
        except Exception:
            with self._lock:
                self._submitting -= 1
            self._remove_artifact_directory(artifact_dir)
            raise
        LOGGER.info("job received job_id=%s frequencies=%s", job_id, freqs.size)
        self._executor.submit(self._run_job, job_id)
        return job

    def _stage_assets(self, config: dict, assets: list, asset_dir: Path) -> dict:
        """Decode uploaded mesh files into the job's directory (server.py:258-292)."""
        asset_dir.mkdir(parents=True, exist_ok=True)
        staged: dict[str, str] = {}
        used: set[str] = set()
        total = 0
        for index, asset in enumerate(assets):
            if not isinstance(asset, dict):
                raise ValueError("Each asset must be an object.")
            original = str(asset.get("original_path", ""))
            if not original:
                raise ValueError("Each asset must include original_path.")
            encoded = asset.get("content_base64")
            if not isinstance(encoded, str):
                raise ValueError(f"Asset {original} must include content_base64.")
            name = _safe_asset_filename(str(asset.get("filename") or Path(original).name), index)
            while name in used:
                name = f"{index}_{name}"
            used.add(name)
            try:
                data = base64.b64decode(encoded.encode("ascii"), validate=True)
            except Exception as exc:
                raise ValueError(f"Asset {original} is not valid base64.") from exc
            if total + len(data) > self.max_asset_bytes:
                raise ValueError(f"Uploaded assets exceed the server limit of {self.max_asset_bytes / MEBIBYTE:g} MiB.")
            path = asset_dir / name
            path.write_bytes(data)
            total += len(data)
            staged[original] = str(path)
        return _rewrite_mesh_paths(config, staged)

    # -- queries ------------------------------------------------------------
    def get(self, job_id: str) -> JobRecord | None:
        with self._lock:
            return self._jobs.get(job_id)

    def events_since(self, job_id: str, start_index: int) -> tuple[list[dict], bool]:
        with self._lock:
            job = self._jobs.get(job_id)
            if job is None:
                raise KeyError(job_id)
            return list(job.events[start_index:]), job.status in TERMINAL_STATES

    def lines_since(self, job_id: str, start_index: int) -> tuple[list[bytes], bool]:
        """The encoded NDJSON lines of events[start_index:] and whether the job has ended."""
        with self._lock:
            job = self._jobs.get(job_id)
            if job is None:
                raise KeyError(job_id)
            return job.lines[max(0, start_index):], job.status in TERMINAL_STATES

    def wait_for_event(self, job_id: str, start_index: int, timeout_s: float = 15.0) -> None:
        """Block until the job has more than ``start_index`` events, ends, or the timeout passes."""
        deadline = time.monotonic() + timeout_s
        with self._lock:
            job = self._jobs.get(job_id)
            while job is not None and len(job.events) <= start_index and job.status not in TERMINAL_STATES:
                remaining = deadline - time.monotonic()
                if remaining <= 0:
                    return
                job.changed.wait(timeout=remaining)
                job = self._jobs.get(job_id)

    # -- cancel, retention, shutdown -----------------------------------------
    def cancel(self, job_id: str) -> bool:
        with self._lock:
            job = self._jobs.get(job_id)
            if job is None:
                return False
            job.cancel_event.set()
            if job.status == "queued":
                job.status = "cancelled"
                job.finished_at = time.time()
                self._add_event_locked(job, "cancelled")
            else:
                self._add_event_locked(job, "cancelling")
            return True

    def purge_expired_jobs(self, *, now: float | None = None) -> int:
        if self.job_retention_seconds <= 0:
            return 0
        cutoff = (time.time() if now is None else now) - self.job_retention_seconds
        with self._lock:
            expired = [j for j in self._jobs.values()
                       if j.status in TERMINAL_STATES and j.finished_at is not None and j.finished_at <= cutoff]
            for job in expired:
                self._jobs.pop(job.job_id, None)
                job.changed.notify_all()
        for job in expired:
            self._remove_artifact_directory(job.artifact_dir)
        return len(expired)

    def _remove_artifact_directory(self, artifact_dir: Path) -> None:
        try:
            root = self.artifact_root.resolve()
            target = artifact_dir.resolve()
            if target.parent != root:
                LOGGER.error("refusing to remove a directory outside the artifact root: %s", target)
                return
            shutil.rmtree(target, ignore_errors=True)
        except OSError:
            LOGGER.exception("failed to remove artifact directory %s", artifact_dir)

    def shutdown(self) -> None:
        with self._lock:
            for job in self._jobs.values():
                if job.status not in TERMINAL_STATES:
                    job.cancel_event.set()
                job.changed.notify_all()
        self._executor.shutdown(wait=False, cancel_futures=True)

    # -- the job loop ---------------------------------------------------------
    def _run_job(self, job_id: str) -> None:
        """server.py:366-475: started, initialized, one result per frequency, then completed
        (with the artifact), cancelled or failed."""
        with self._lock:
            job = self._jobs.get(job_id)
            if job is None:
                return
            if job.cancel_event.is_set():
                # as the reference: a job cancelled while queued gets a second "cancelled"
                # event when its worker picks it up (server.py:369-374)
                job.status = "cancelled"
                job.finished_at = time.time()
                self._add_event_locked(job, "cancelled")
                return
            job.status = "running"
            job.started_at = time.time()
            self._add_event_locked(job, "started")
        try:
            solver = self.solver_factory(job.config)
            set_status = getattr(solver, "set_status_callback", None)
            if callable(set_status):
                set_status(lambda message: LOGGER.info("job %s: %s", job_id, message))
            initialize = getattr(solver, "initialize", None)
            if callable(initialize):
                initialize(job.frequencies_hz)
            sphere = solver.sphere_metadata or {}
            config = job.config
            dataset = ResultDataset(
                polar_angle_deg=np.asarray(solver.polar_angle_deg, dtype=np.float32),
                radiator_names=np.asarray(solver.radiator_names),
                polar_observation_distance_m=abs(float(_config_value(config, "distance", 2.0))
                                                 + float(_config_value(config, "axial_offset", 0.0))),
                exterior_sound_speed_m_per_s=float(_config_value(config, "sound_speed", 343.0)),
                sphere_r_distance_m=sphere.get("r_distance_m"),
                sphere_theta_polar_rad=sphere.get("theta_polar_rad"),
                sphere_phi_azimuth_rad=sphere.get("phi_azimuth_rad"),
            )
            with self._lock:
                job.dataset = dataset
                self._add_event_locked(
                    job, "initialized",
                    polar_angle_deg=ndarray_to_wire(dataset.polar_angle_deg),
                    radiator_names=np.asarray(dataset.radiator_names).astype(str).tolist(),
                    sphere_metadata={k: ndarray_to_wire(v) for k, v in sphere.items()} if sphere else None)
            for result in solver.solve_stream(job.frequencies_hz, stop_requested=job.cancel_event.is_set):
                if job.cancel_event.is_set():
                    break
                dataset.add(result)
                wire = frequency_result_to_wire(result)
                with self._lock:
                    job.solved_count = dataset.solved_count
                    self._add_event_locked(job, "result", result=wire, solved_count=job.solved_count,
                                           total_count=job.total_count)
            with self._lock:
                if job.cancel_event.is_set():
                    job.status = "cancelled"
                    job.finished_at = time.time()
                    self._add_event_locked(job, "cancelled", solved_count=job.solved_count)
                    return
            artifact = write_result_artifact(dataset, job.artifact_dir / "result.npz")
            with self._lock:
                job.result_npz = artifact
                job.status = "completed"
                job.finished_at = time.time()
                self._add_event_locked(job, "completed", solved_count=job.solved_count,
                                       artifact=f"/jobs/{job.job_id}/artifacts/result.npz")
            LOGGER.info("job completed job_id=%s solved=%s/%s", job_id, job.solved_count, job.total_count)
        except Exception as exc:  # noqa: BLE001 - every failure ends the job with a `failed` event
            with self._lock:
                job.status = "failed"
                job.error = str(exc)
                job.finished_at = time.time()
                self._add_event_locked(job, "failed", error=job.error)
            LOGGER.exception("job failed job_id=%s", job_id)

    def _add_event_locked(self, job: JobRecord, event_type: str, **payload: Any) -> None:
        event = {"index": len(job.events), "job_id": job.job_id, "type": event_type, "timestamp": time.time(),
                 **payload}
        job.events.append(event)
        job.lines.append(json.dumps(event, separators=(",", ":")).encode("utf-8") + b"\n")
        job.event_count = len(job.events)
        job.changed.notify_all()


# --------------------------------------------------------------------- HTTP --

class JobHTTPServer(ThreadingHTTPServer):
    """One thread per connection (server.py:526-570)."""

    daemon_threads = True

    def __init__(self, server_address, orchestrator: JobOrchestrator, *, solver_id: str = "gb300_cuda",
                 access_token: str | None = None,
                 max_request_bytes: int = DEFAULT_MAX_REQUEST_BYTES,
                 event_stream_window_seconds: float = DEFAULT_EVENT_STREAM_WINDOW_SECONDS):
        if max_request_bytes < 1:
            raise ValueError("max_request_bytes must be >= 1.")
        if event_stream_window_seconds <= 0:
            raise ValueError("event_stream_window_seconds must be > 0.")
        super().__init__(server_address, JobRequestHandler)
        self.orchestrator = orchestrator
        self.solver_id = solver_id
        self.access_token = str(access_token or "")
        self.max_request_bytes = max_request_bytes
        self.event_stream_window_seconds = event_stream_window_seconds

    def health_payload(self) -> dict:
        from .backend import CAPABILITIES, LABEL  # noqa: PLC0415

        self.orchestrator.purge_expired_jobs()
        caps = CAPABILITIES
        return {
            "status": "ok",
            "solver": self.solver_id,
            "backend": self.solver_id,
            "solver_label": LABEL,
            "capabilities": {name: bool(getattr(caps, name)) for name in (
                "supports_spherical_sampling", "supports_impedance", "supports_burton_miller",
                "supports_flat_target_normalization", "supports_channel_resynthesis", "supports_cancellation",
                "supports_streaming", "supports_symmetry")},
        }


class JobRequestHandler(BaseHTTPRequestHandler):
    server: JobHTTPServer
    protocol_version = "HTTP/1.0"

    def do_GET(self) -> None:  # noqa: N802 - stdlib override
        parsed = urlparse(self.path)
        parts = [p for p in parsed.path.split("/") if p]
        if not self._authorize():
            return
        if parsed.path == "/health":
            self._send_json(self.server.health_payload())
        elif len(parts) == 2 and parts[0] == "jobs":
            job = self.server.orchestrator.get(parts[1])
            if job is None:
                self._send_error(HTTPStatus.NOT_FOUND, "Job not found.")
            else:
                self._send_json(job.snapshot())
        elif len(parts) == 3 and parts[0] == "jobs" and parts[2] == "events":
            try:
                since = int(parse_qs(parsed.query).get("since", ["0"])[0])
            except ValueError:
                self._send_error(HTTPStatus.BAD_REQUEST, "since must be an integer.")
                return
            self._stream_events(parts[1], since)
        elif len(parts) == 4 and parts[0] == "jobs" and parts[2] == "artifacts" and parts[3] == "result.npz":
            self._send_artifact(parts[1])
        else:
            self._send_error(HTTPStatus.NOT_FOUND, "Unknown endpoint.")

    def do_POST(self) -> None:  # noqa: N802 - stdlib override
        parsed = urlparse(self.path)
        parts = [p for p in parsed.path.split("/") if p]
        if not self._authorize():
            return
        if parsed.path == "/jobs":
            self._create_job()
        elif len(parts) == 3 and parts[0] == "jobs" and parts[2] == "cancel":
            if not self.server.orchestrator.cancel(parts[1]):
                self._send_error(HTTPStatus.NOT_FOUND, "Job not found.")
            else:
                self._send_json({"job_id": parts[1], "status": "cancelling"})
        else:
            self._send_error(HTTPStatus.NOT_FOUND, "Unknown endpoint.")

    def log_message(self, format: str, *args) -> None:  # noqa: A002 - stdlib signature
        return

    def _create_job(self) -> None:
        try:
            payload = self._read_json()
            config, freqs, assets = solve_request_to_job_inputs(payload)
            job = self.server.orchestrator.submit(config, freqs, assets)
        except RequestTooLargeError as exc:
            self._send_error(HTTPStatus.REQUEST_ENTITY_TOO_LARGE, str(exc))
            return
        except JobQueueFullError as exc:
            self._send_error(HTTPStatus.SERVICE_UNAVAILABLE, str(exc))
            return
        except Exception as exc:  # noqa: BLE001 - any malformed request is a 400
            self._send_error(HTTPStatus.BAD_REQUEST, str(exc))
            return
        self._send_json(job.snapshot(), status=HTTPStatus.ACCEPTED)

    def _stream_events(self, job_id: str, start_index: int) -> None:
        """One event window: every event from ``since`` on as NDJSON, until the job ends or the
        window closes; the client reconnects with since = last index + 1 (server.py:651-678)."""
        orch = self.server.orchestrator
        if orch.get(job_id) is None:
            self._send_error(HTTPStatus.NOT_FOUND, "Job not found.")
            return
        self.send_response(HTTPStatus.OK)
        self.send_header("Content-Type", "application/x-ndjson")
        self.send_header("Cache-Control", "no-cache")
        self.end_headers()
        next_index = max(0, start_index)
        deadline = time.monotonic() + self.server.event_stream_window_seconds
        try:
            while True:
                try:
                    lines, terminal = orch.lines_since(job_id, next_index)
                except KeyError:
                    return  # purged while streaming
                if lines:
                    self.wfile.write(b"".join(lines))
                    self.wfile.flush()
                    next_index += len(lines)
                if terminal:
                    return
                remaining = deadline - time.monotonic()
                if remaining <= 0:
                    return
                orch.wait_for_event(job_id, next_index, timeout_s=min(remaining, 15.0))
        except (BrokenPipeError, ConnectionResetError):
            LOGGER.warning("event stream of job %s disconnected at index %s", job_id, next_index)

    def _send_artifact(self, job_id: str) -> None:
        job = self.server.orchestrator.get(job_id)
        if job is None:
            self._send_error(HTTPStatus.NOT_FOUND, "Job not found.")
            return
        if job.result_npz is None or not job.result_npz.exists():
            self._send_error(HTTPStatus.NOT_FOUND, "Result artifact not available.")
            return
        data = job.result_npz.read_bytes()
        self.send_response(HTTPStatus.OK)
        self.send_header("Content-Type", "application/octet-stream")
        self.send_header("Content-Length", str(len(data)))
        self.end_headers()
        self.wfile.write(data)

    def _read_json(self) -> dict:
        try:
            length = int(self.headers.get("Content-Length", "0"))
        except ValueError as exc:
            raise ValueError("Content-Length must be an integer.") from exc
        if length <= 0:
            raise ValueError("Request body must contain JSON.")
        if length > self.server.max_request_bytes:
            raise RequestTooLargeError(
                f"Request body exceeds the server limit of {self.server.max_request_bytes / MEBIBYTE:g} MiB.")
        if self.headers.get_content_type() != "application/json":
            raise ValueError("Content-Type must be application/json.")
        payload = json.loads(self.rfile.read(length).decode("utf-8"))
        if not isinstance(payload, dict):
            raise ValueError("Request JSON must be an object.")
        return payload

    def _authorize(self) -> bool:
        expected = self.server.access_token
        if not expected:
            return True
        scheme, sep, provided = self.headers.get("Authorization", "").partition(" ")
        if sep and scheme.lower() == "bearer" and hmac.compare_digest(provided.strip(), expected):
            return True
        data = json.dumps({"error": "Authentication required."}, separators=(",", ":")).encode("utf-8")
        self.send_response(HTTPStatus.UNAUTHORIZED)
        self.send_header("WWW-Authenticate", "Bearer")
        self.send_header("Content-Type", "application/json")
        self.send_header("Content-Length", str(len(data)))
        self.end_headers()
        self.wfile.write(data)
        return False

    def _send_json(self, payload: dict, *, status: HTTPStatus = HTTPStatus.OK) -> None:
        data = json.dumps(payload, separators=(",", ":")).encode("utf-8")
        self.send_response(status)
        self.send_header("Content-Type", "application/json")
        self.send_header("Content-Length", str(len(data)))
        self.end_headers()
        self.wfile.write(data)

    def _send_error(self, status: HTTPStatus, message: str) -> None:
        self._send_json({"error": message}, status=status)


# ---------------------------------------------------------------------- CLI --

def main(argv: list[str] | None = None) -> int:
    """``python -m boundary-lab_gb300.job_server --port 8765 --max-running-jobs 4`` (the options of
    server.py:760-839 that apply to this backend)."""
    parser = argparse.ArgumentParser(description="Serve exterior BEM jobs on one GB300.")
    parser.add_argument("--host", default="127.0.0.1")
    parser.add_argument("--port", type=int, default=8765)
    parser.add_argument("--device", type=int, default=0)
    parser.add_argument("--precision", choices=("mixed", "fp64"), default="mixed")
    parser.add_argument("--max-running-jobs", type=int, default=1)
    parser.add_argument("--max-queued-jobs", type=int, default=DEFAULT_MAX_QUEUED_JOBS)
    parser.add_argument("--max-request-mb", type=float, default=DEFAULT_MAX_REQUEST_BYTES / MEBIBYTE)
    parser.add_argument("--max-asset-mb", type=float, default=DEFAULT_MAX_ASSET_BYTES / MEBIBYTE)
    parser.add_argument("--max-frequencies", type=int, default=DEFAULT_MAX_FREQUENCIES)
    parser.add_argument("--job-retention-hours", type=float, default=DEFAULT_JOB_RETENTION_HOURS)
    parser.add_argument("--event-stream-window-seconds", type=float, default=DEFAULT_EVENT_STREAM_WINDOW_SECONDS)
    parser.add_argument("--artifact-dir", type=Path, default=DEFAULT_ARTIFACT_ROOT)
    parser.add_argument("--access-token", default="", help="require 'Authorization: Bearer <token>'")
    parser.add_argument("--memory-budget-gb", type=float, default=None,
                        help="device memory the running jobs may hold together (default with more than one "
                             "running job: 85%% of the free memory; 0 turns admission off)")
    parser.add_argument("--log-level", default="INFO")
    args = parser.parse_args(argv)
    if args.memory_budget_gb is None:
        budget = default_memory_budget(args.device) if args.max_running_jobs > 1 else None
    else:
        budget = int(args.memory_budget_gb * (1 << 30)) or None
    logging.basicConfig(level=getattr(logging, str(args.log_level).upper(), logging.INFO))
    orch = JobOrchestrator(
        max_running_jobs=args.max_running_jobs, max_queued_jobs=args.max_queued_jobs,
        max_asset_bytes=max(1, int(args.max_asset_mb * MEBIBYTE)), max_frequencies=args.max_frequencies,
        job_retention_hours=args.job_retention_hours, artifact_root=args.artifact_dir,
        solver_factory=gb300_solver_factory(precision=args.precision, device=args.device,
                                            memory_budget_bytes=budget))
    server = JobHTTPServer((args.host, args.port), orch, access_token=args.access_token or None,
                           max_request_bytes=max(1, int(args.max_request_mb * MEBIBYTE)),
                           event_stream_window_seconds=args.event_stream_window_seconds)
    LOGGER.info("serving on http://%s:%s", *server.server_address[:2])
    try:
        server.serve_forever()
    except KeyboardInterrupt:
        pass
    finally:
        server.server_close()
        orch.shutdown()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
