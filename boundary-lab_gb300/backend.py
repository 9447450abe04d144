"""Solver backend for Boundary Lab: the drop-in beside ``beat_cuda``.

Mirrors the reference's backend protocol (src/blab/solvers/base.py:70-110) and
the behaviour of its BEAT adapter (src/blab/solvers/beat_engine_backend.py):
``create_session(SolveRequest)`` returns a session whose ``metadata`` is ready
at once and whose ``solve_stream()`` yields one ``FrequencyResult`` per
frequency; ``stop()`` cancels cooperatively between frequencies; errors
surface as ``RuntimeError``.  Unlike the adapter there is no subprocess: the
session runs in-process and drives the CUDA library through its C ABI.

``register_with_boundary_lab()`` adds the backend ID ``gb300_cuda`` to the
application's registry (registry.py:21-83) and to the job server's solver
sets (server.py:46-52), so ``create_backend("gb300_cuda")`` and
``blab server --solver gb300_cuda`` find it.

Concurrent jobs.  The reference's job server runs ``max_running_jobs`` jobs
on a thread pool (server.py:185); its BEAT adapter then serialises them on
one worker per GPU.  With ``concurrent=True`` (or GB300_BEM_CONCURRENT_JOBS=1
in the environment) each server thread solves on its own library context (its
own CUDA stream and scratch), so those jobs share the GPU, and a process-wide
``MemoryAdmission`` per device holds each job's device footprint (mesh caches
plus one frequency batch) from its mesh upload to its end: a job waits while
it does not fit beside the running ones.
"""

from __future__ import annotations

import dataclasses
import os
import threading
from typing import Any, Callable, Iterator

import numpy as np

from . import contract
from .job import BACKEND_ID, ExteriorJob, JobCancelled

LABEL = "GB300 BEM (CUDA, sm_103a)"
CAPABILITIES = contract.SolverCapabilities(
    supports_remote_assets=False,
    supports_parallel_workers=False,
    supports_symmetry=True,
    supports_channel_resynthesis=True,
    is_remote=False,
)


class MemoryAdmission:
    """Device-memory budget shared by concurrent jobs on one GPU.  ``acquire(n)`` blocks
    until n bytes fit beside the bytes already held (a request larger than the whole
    budget is let through once nothing else is held) and returns a token for
    ``release``."""

    def __init__(self, budget_bytes: int):
        if budget_bytes <= 0:
            raise ValueError("budget_bytes must be > 0")
        self.budget = int(budget_bytes)
        self._held: dict[int, int] = {}
        self._next = 0
        self._cv = threading.Condition()

    def in_use(self) -> int:
        with self._cv:
            return sum(self._held.values())

    def free_bytes(self) -> int:
        return self.budget - self.in_use()

    def acquire(self, nbytes: int) -> int:
        want = max(0, int(nbytes))
        with self._cv:
            self._cv.wait_for(lambda: not self._held or sum(self._held.values()) + want <= self.budget)
            self._next += 1
            self._held[self._next] = want
            return self._next

    def release(self, token: int) -> None:
        with self._cv:
            self._held.pop(int(token), None)
            self._cv.notify_all()


def default_memory_budget(device: int) -> int:
    """85% of the device memory that is free now; 64 GiB when it cannot be queried."""
    try:
        import torch  # noqa: PLC0415

        free, _ = torch.cuda.mem_get_info(device)
        return int(0.85 * free)
    except Exception:  # noqa: BLE001 - no torch or no GPU
        return 64 << 30


_admission_lock = threading.Lock()
_admissions: dict[int, MemoryAdmission] = {}


def device_admission(device: int, budget_bytes: int | None = None) -> MemoryAdmission:
    """The process-wide admission of ``device`` (created on first use)."""
    with _admission_lock:
        if device not in _admissions:
            _admissions[device] = MemoryAdmission(budget_bytes or default_memory_budget(device))
        return _admissions[device]


def config_to_dict(config: Any) -> dict:
    """SimulationConfig dataclass (config.py:68-93) or dict -> request config dict."""
    if isinstance(config, dict):
        return dict(config)
    if dataclasses.is_dataclass(config):
        return dataclasses.asdict(config)
    raise TypeError(f"unsupported config type {type(config).__name__}")


def request_dict(request) -> dict:
    freqs = np.asarray(request.frequencies_hz, dtype=np.float32).reshape(-1)
    return {"schema_version": 2, "config": config_to_dict(request.config), "frequencies_hz": freqs.tolist()}


class Gb300BemSession:
    def __init__(self, request, *, engine_factory: Callable | None = None, precision: str = "mixed",
                 device: int = 0, batch: int = 0, admission=None):
        self._request = request
        self._stop = threading.Event()
        self._status = getattr(request, "status_callback", None)
        try:
            self._job = ExteriorJob(request_dict(request), engine_factory=engine_factory, status=self._emit,
                                    precision=precision, device=device, batch=batch, admission=admission)
            meta = self._job.initialized_payload()
            sphere = meta["sphere_metadata"]
            self._metadata = contract.SolveMetadata(
                polar_angle_deg=np.asarray(meta["polar_angle_deg"], dtype=np.float32),
                radiator_names=np.asarray(meta["radiator_names"]),
                sphere_metadata=None if sphere is None else {k: np.asarray(v, np.float32) for k, v in sphere.items()},
            )
        except Exception as exc:
            raise RuntimeError(str(exc)) from exc

    def _emit(self, message: str) -> None:
        if self._status is not None:
            self._status(message)

    @property
    def metadata(self):
        return self._metadata

    def solve_stream(self, *, stop_requested: Callable[[], bool] | None = None) -> Iterator:
        def stop() -> bool:
            return self._stop.is_set() or (stop_requested is not None and stop_requested())

        try:
            for event in self._job.results(stop=stop):
                if stop():
                    return
                yield contract.frequency_result_from_event(event["result"])
        except JobCancelled:
            return
        except Exception as exc:
            raise RuntimeError(str(exc)) from exc
        finally:
            self._job.close()

    def stop(self) -> None:
        self._stop.set()


class Gb300BemBackend:
    backend_id = BACKEND_ID
    label = LABEL
    capabilities = CAPABILITIES

    def __init__(self, *, device: int = 0, precision: str = "mixed", batch: int = 0,
                 engine_factory: Callable | None = None, concurrent: bool | None = None,
                 memory_budget_bytes: int | None = None, **_ignored: Any):
        # _ignored absorbs the keyword arguments the application passes to every
        # backend factory (julia_executable, julia_threads, ...; server.py:870-889).
        self.device = device
        self.precision = precision
        self.batch = batch
        if concurrent is None:
            concurrent = os.environ.get("GB300_BEM_CONCURRENT_JOBS", "").strip().lower() in ("1", "true", "yes")
        self.concurrent = bool(concurrent)
        self.memory_budget_bytes = memory_budget_bytes
        self.engine_factory = engine_factory
        if self.concurrent and engine_factory is None:
            from .engine import engine_from_env  # noqa: PLC0415

            self.engine_factory = lambda **kw: engine_from_env(context="thread", **kw)

    def create_session(self, request) -> Gb300BemSession:
        admission = device_admission(self.device, self.memory_budget_bytes) if self.concurrent else None
        return Gb300BemSession(request, engine_factory=self.engine_factory, precision=self.precision,
                               device=self.device, batch=self.batch, admission=admission)

    def warm_up(self, mode: str = "worker", *, status_callback: Callable[[str], None] | None = None) -> None:
        """`worker`: load the library and create the CUDA context; `tiny`: also solve a tetrahedron at
        100 Hz (the reference's warm-up, beat_engine_backend.py:522-553, 610-653)."""
        mode = str(mode or "off").strip().lower()
        if mode in ("off", "0", "false", "no", "none"):
            return
        from . import engine as engmod

        engmod.shared_context(self.device)
        if mode in ("tiny", "solve", "job"):
            import tempfile
            from pathlib import Path

            from . import meshes

            with tempfile.TemporaryDirectory(prefix="gb300-bem-warmup-") as tmp:
                path = Path(tmp) / "warmup_tetrahedron.msh"
                v = np.array([[0, 0, 0], [0.08, 0, 0], [0, 0.08, 0], [0, 0, 0.08]], float)
                f = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [2, 0, 3]])
                meshes.write_gmsh22(path, v, f, np.full(4, 2))
                cfg = {"mesh_file": str(path), "scale_factor": 1.0, "distance": 1.0, "step_size": 90.0,
                       "min_angle": 0.0, "max_angle": 0.0, "tag_throat": 2,
                       "radiators": [{"name": "warmup", "tag": 2, "channel": "main"}],
                       "channels": [{"name": "main"}], "flat_target_normalization_enabled": False}
                req = contract.SolveRequest(cfg, np.asarray([100.0], np.float32), status_callback=status_callback)
                list(self.create_session(req).solve_stream())


def register_with_boundary_lab() -> bool:
    """Register ``gb300_cuda`` with the application's backend registry and job server.
    Returns False when Boundary Lab's package is not importable."""
    try:
        from blab.solvers import registry  # type: ignore
    except Exception:  # noqa: BLE001
        return False
    caps = registry.SolverCapabilities(**{f.name: getattr(CAPABILITIES, f.name)
                                          for f in dataclasses.fields(CAPABILITIES)})
    registry._BACKENDS[BACKEND_ID] = registry.SolverBackendInfo(
        backend_id=BACKEND_ID,
        label=LABEL,
        capabilities=caps,
        factory=lambda **kwargs: Gb300BemBackend(**kwargs),
        description="Exterior Burton-Miller BEM on NVIDIA GB300 (sm_103a CUDA kernels, FP64-refined mixed precision).",
    )
    try:
        from blab import server  # type: ignore

        server.SERVER_SOLVER_BACKENDS.add(BACKEND_ID)
        server.SERVER_SOLVER_BACKEND_IDS[BACKEND_ID] = BACKEND_ID
    except Exception:  # noqa: BLE001 - the registry alone is still useful
        pass
    return True
