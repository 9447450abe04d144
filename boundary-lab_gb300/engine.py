"""Numerical engine behind a solve session.

``CudaEngine`` drives the C ABI.  By default it uses one context per process
and device, shared by sessions, with a lock that serialises calls on it (like
the reference's per-worker lock, src/blab/solvers/beat_engine_backend.py:314-334).
With ``context="thread"`` each calling thread gets its own context (its own
CUDA stream and scratch), so the worker threads of a job server run their jobs
on the GPU at the same time.  Any object with the same
three methods can stand in for it (``engine_factory`` arguments and the
``GB300_BEM_ENGINE=module:callable`` environment variable), which is how the
CPU tests drive the session and worker logic without a GPU.
"""

from __future__ import annotations

import importlib
import os
import threading
from dataclasses import dataclass

import numpy as np

from . import native

PRECISIONS = {"fp64": native.BEM_PRECISION_FP64, "mixed": native.BEM_PRECISION_MIXED}
TRIM_ABOVE_BYTES = 8 << 30  # per-thread contexts keep at most this much scratch between jobs


@dataclass
class EngineResult:
    pressure: np.ndarray  # [n_freq, n_rhs, n_vertices] complex128
    field: np.ndarray  # [n_freq, n_rhs, n_points] complex128
    stats: dict


_contexts: dict[int, native.Context] = {}
_context_locks: dict[int, threading.Lock] = {}
_pool_lock = threading.Lock()
_per_thread = threading.local()


def shared_context(device: int) -> tuple[native.Context, threading.Lock]:
    with _pool_lock:
        if device not in _contexts:
            _contexts[device] = native.Context(device)
            _context_locks[device] = threading.Lock()
        return _contexts[device], _context_locks[device]


def thread_context(device: int) -> tuple[native.Context, threading.Lock]:
    """The calling thread's own context on ``device`` (created on first use, kept for the thread's life)."""
    contexts = getattr(_per_thread, "contexts", None)
    if contexts is None:
        contexts = _per_thread.contexts = {}
    if device not in contexts:
        contexts[device] = (native.Context(device), threading.Lock())
    return contexts[device]


class CudaEngine:
    """One uploaded mesh on one GPU."""

    name = "gb300_cuda"

    def __init__(self, device: int = 0, precision: str = "mixed", batch: int = 0, refine_tol: float = 1e-10,
                 context: str = "shared", autotune: bool = False, lanes: int = 2):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        if context not in ("shared", "thread"):
            raise ValueError("context must be 'shared' or 'thread'")
        self.device = device
        self.precision = precision
        self.batch = batch
        self.refine_tol = refine_tol
        self.ctx, self.lock = shared_context(device) if context == "shared" else thread_context(device)
        self.context = context
        self.mesh: native.Mesh | None = None
        # autotune: the first solve on a mesh times the candidate launch configurations
        # (autotune.tune, cached per device and problem shape) and later solves use the winner
        self.autotune = autotune
        # lanes = 2: a call of two or more batches runs them side by side on two streams
        # (bem_solve_options.lanes), so the job loop asks for two batches per call
        self.lanes = max(1, min(2, int(lanes)))
        self.launch = None  # autotune.LaunchConfig once tuned
        self.tune_result = None

    def prepare(self, vertices, faces, drives, points, regular_order: int = 4, singular_order: int = 4,
                symmetry: str = "off") -> None:
        with self.lock:
            self.launch = None
            self.mesh = self.ctx.upload_mesh(vertices, faces, regular_order, singular_order, symmetry=symmetry)
            self.mesh.set_excitation(drives)
            self.mesh.set_observation_points(points)
            self.n_rhs = int(np.asarray(drives).reshape(-1, len(faces)).shape[0])
            self.n_points = int(len(points))

    def device_bytes(self, n_freq: int) -> int:
        """Device memory of a solve of n_freq frequencies on this mesh: the mesh caches plus the
        scratch of the batch the solve will use (bem_estimate_device_bytes)."""
        if self.mesh is None:
            raise RuntimeError("engine.prepare() must run before device_bytes()")
        prec = PRECISIONS[self.precision]
        with self.lock:
            batch = self.batch or self.mesh.auto_batch(n_freq, prec)
            if self.autotune and not self.batch:
                # the tuner tries up to one frequency more than the library's own batch
                batch = self.launch.batch if self.launch is not None else min(batch + 1, max(1, n_freq))
            lanes = self.lanes if n_freq >= 2 * batch else 1  # each lane holds a batch's scratch
            return self.ctx.estimate_device_bytes(self.mesh.n_vertices, self.mesh.n_faces,
                                                  self.mesh.n_singular_pairs, self.n_rhs, self.n_points,
                                                  batch * lanes, prec)

    def preferred_chunk(self, n_freq: int) -> int:
        """Frequencies per solve call for a sweep of n_freq: one batch of the size the solve
        uses (bem_auto_batch splits a sweep into equal batches whose LU panels are resident
        in one wave) per lane, so no call leaves a partial batch behind and, with two lanes,
        each call keeps both streams busy."""
        if self.mesh is None:
            raise RuntimeError("engine.prepare() must run before preferred_chunk()")
        if self.batch:
            b = max(1, int(self.batch))
        elif self.autotune and self.launch is not None:
            b = max(1, int(self.launch.batch))
        else:
            with self.lock:
                b = max(1, int(self.mesh.auto_batch(max(1, int(n_freq)), PRECISIONS[self.precision])))
        return b * self.lanes if n_freq >= b * self.lanes else b

    def tune_sweep(self, freqs_hz, sound_speed: float, rho: float) -> None:
        """With autotune on, time the candidate launch configurations on the whole sweep
        (autotune.tune scores each by the sweep's rate, n_freq / (ceil(n_freq / batch) x
        batch time)) before the first solve; later chunks use the winner's batch."""
        if self.mesh is None:
            raise RuntimeError("engine.prepare() must run before tune_sweep()")
        if not self.autotune or self.batch or self.launch is not None:
            return
        with self.lock:
            self._tune(freqs_hz, sound_speed, rho)

    def _tune(self, freqs_hz, sound_speed: float, rho: float) -> None:
        from . import autotune  # noqa: PLC0415

        self.tune_result = autotune.tune(self.mesh, freqs_hz, precision=PRECISIONS[self.precision],
                                         sound_speed=sound_speed, rho=rho, refine_tol=self.refine_tol,
                                         device=self.device)
        self.launch = self.tune_result.best

    def solve(self, freqs_hz, sound_speed: float, rho: float) -> EngineResult:
        if self.mesh is None:
            raise RuntimeError("engine.prepare() must run before solve()")
        with self.lock:
            kw = dict(batch=self.batch)
            if self.autotune and not self.batch:
                if self.launch is None:
                    self._tune(freqs_hz, sound_speed, rho)
                kw = dict(batch=self.launch.batch, lu_block=self.launch.lu_block, lu_gemm=self.launch.lu_gemm)
            p, u, stats = self.mesh.solve(freqs_hz, precision=PRECISIONS[self.precision], sound_speed=sound_speed,
                                          rho=rho, refine_tol=self.refine_tol, lanes=self.lanes, **kw)
        return EngineResult(p, u, stats)

    def close(self) -> None:
        with self.lock:
            if self.mesh is not None:
                self.mesh.release()
                self.mesh = None
            self.launch = None
            # a worker thread's own context keeps its solve scratch between jobs; a large
            # job's scratch (matrices of a whole batch) is returned to the pool afterwards
            if self.context == "thread" and self.ctx.scratch_bytes > TRIM_ABOVE_BYTES:
                self.ctx.trim()


def engine_from_env(**kwargs):
    """Engine factory named by GB300_BEM_ENGINE ("module:callable"), else CudaEngine."""
    spec = os.environ.get("GB300_BEM_ENGINE", "").strip()
    if not spec:
        return CudaEngine(**kwargs)
    module, _, attr = spec.partition(":")
    return getattr(importlib.import_module(module), attr or "make_engine")(**kwargs)
