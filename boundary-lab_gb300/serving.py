"""Serving scheduler: a stream of exterior jobs on one GB300.

The reference serves jobs through ``JobOrchestrator`` (src/blab/server.py:174-256,
366-475): a bounded number of running plus queued jobs (a submission beyond
``max_running + max_queued`` is rejected, server.py:216-223), a thread pool of
``max_running`` workers, per-frequency result events, and cooperative cancel
between frequencies.  Each worker drives one solver process that holds one job
at a time per GPU (beat_engine_backend.py:314-334).

This module keeps that contract and replaces the per-GPU serialisation:

* every worker thread owns one library context (its own CUDA stream and
  stream-ordered scratch), so up to ``max_running`` jobs run on the GPU at the
  same time -- a 1k-triangle job occupies a few SMs for a few milliseconds and
  would otherwise leave the GPU idle behind a 15k-triangle sweep;
* admission control: a job starts only when its device footprint (mesh caches
  plus the scratch of one frequency batch, ``bem_estimate_device_bytes``) fits
  in the memory budget together with the footprints of the jobs running now;
* policy ``"fifo"`` (arrival order, as the reference) or ``"sjf"`` (least
  estimated GPU work first; a job that has waited ``aging_s`` goes first, the
  aged jobs in arrival order).  The default ``aging_s`` of 2 s comes from a
  sweep on bench.py's seeded stream (40 jobs of 1k-15k triangles arriving at
  20/s, four running): against 30 s it cut the p99 latency from 6.2-6.7 s to
  5.0 s with p50 unchanged (1.0-1.1 s); 1 s raised p50 to 3.6 s, as nearly every
  job then ages and the queue runs in arrival order;
* long sweeps run in frequency chunks, so results stream per chunk and cancel
  takes effect between chunks;
* small jobs share launches: a worker that takes a job of at most
  ``group_faces`` triangles also takes the queued small jobs of similar size
  (largest / smallest vertex count <= ``group_size_ratio``, same physics and
  excitation count, memory permitting, ``group_max_freqs`` frequencies in all)
  and solves them in one ``bem_solve_jobs`` call: their matrices, padded to the
  largest, are factored, solved and refined in one launch sequence.

Results are independent of the mix: every frequency's assembly, LU and field
are computed by the same kernels on the same inputs whatever runs beside it
(deterministic kernels), so a job that runs on its own is bitwise the same alone
or under load.  A job solved in a group is the same up to the rounding of its
sums (FP64 form) or its refinement (a group refines until every system in it
reaches the tolerance): within 1e-8 in the mixed form.

The executor doing the GPU work is injectable (``executor_factory``), which lets
the scheduling logic be tested on hosts without a GPU.
"""

from __future__ import annotations

import itertools
import math
import threading
import time
from dataclasses import dataclass
from dataclasses import field as dc_field
from typing import Callable, Iterable, Sequence

import numpy as np


class JobQueueFullError(RuntimeError):
    """Raised by submit() when running + queued jobs are at capacity (server.py:216-223)."""


class JobCancelledError(RuntimeError):
    pass


@dataclass(eq=False)  # jobs compare by identity (they hold arrays)
class ServingJob:
    """One exterior job: a mesh, its excitations and observation points, and a frequency list."""

    vertices: np.ndarray            # [n_vertices, 3] float64, metres
    faces: np.ndarray               # [n_faces, 3] int32, 0-based
    drive: np.ndarray               # [n_rhs, n_faces] complex unit drive (v_n = 1 on radiator faces)
    points: np.ndarray              # [n_points, 3] observation points
    freqs_hz: np.ndarray            # [n_freq]
    precision: int = 1              # BEM_PRECISION_MIXED
    sound_speed: float = 343.0
    rho: float = 1.205
    chunk: int = 16                 # frequencies per solve call (one LU batch)
    job_id: str = ""
    # filled in by the scheduler
    status: str = "created"         # queued, running, completed, cancelled, failed
    arrival_s: float = math.nan
    start_s: float = math.nan
    first_result_s: float = math.nan
    finish_s: float = math.nan
    solved_count: int = 0
    error: str | None = None
    pressure: np.ndarray | None = None   # [n_freq, n_rhs, n_vertices] complex128
    field: np.ndarray | None = None      # [n_freq, n_rhs, n_points] complex128
    estimated_bytes: int = 0
    estimated_work: float = 0.0
    group_size: int = 1             # jobs solved together with this one (bem_solve_jobs), itself included
    _cancel: threading.Event = dc_field(default_factory=threading.Event, repr=False)
    _done: threading.Event = dc_field(default_factory=threading.Event, repr=False)

    @property
    def n_faces(self) -> int:
        return int(len(self.faces))

    @property
    def n_vertices(self) -> int:
        return int(len(self.vertices))

    @property
    def latency_s(self) -> float:
        return self.finish_s - self.arrival_s

    @property
    def first_result_latency_s(self) -> float:
        return self.first_result_s - self.arrival_s

    def cancel(self) -> None:
        self._cancel.set()

    def wait(self, timeout: float | None = None) -> bool:
        return self._done.wait(timeout)


def estimated_work(n_faces: int, n_vertices: int, n_freq: int, q_points: int = 6) -> float:
    """Relative GPU work of a job: regular q-pairs plus LU flops (complex, 8/3 n^3),
    weighted by the measured cost of each on GB300 (about 2.3 ns per 1e3 q-pairs and
    1e3 LU flop respectively at 10k triangles); used only to order jobs."""
    qpairs = float(n_faces) ** 2 * q_points ** 2
    lu_flop = 8.0 / 3.0 * float(n_vertices) ** 3
    return n_freq * (qpairs + 0.7 * lu_flop)


class NativeExecutor:
    """GPU work of a worker thread: one library context on ``device``."""

    def __init__(self, device: int = 0, trim_above_bytes: int = 8 << 30):
        from . import native  # noqa: PLC0415 - the CUDA library loads on first use

        self._native = native
        native.load()
        self.ctx = native.Context(device)
        self.trim_above_bytes = trim_above_bytes

    def footprint(self, job: ServingJob) -> int:
        n_pairs = 14 * job.n_faces  # vertex-sharing pairs of a closed valence-6 mesh: about 13-14 per face
        batch = max(1, min(job.chunk, len(job.freqs_hz)))
        scratch = self.ctx.estimate_device_bytes(job.n_vertices, job.n_faces, n_pairs, int(job.drive.shape[0]),
                                                 int(len(job.points)), batch, job.precision)
        mesh = job.n_faces * (160 + 288 + 64) + n_pairs * (24 * 8 + 32)
        return int(scratch + mesh)

    def run(self, job: ServingJob, on_chunk: Callable[[int, np.ndarray, np.ndarray], None],
            should_stop: Callable[[], bool]) -> None:
        m = self.ctx.upload_mesh(job.vertices, job.faces)
        try:
            m.set_excitation(job.drive)
            m.set_observation_points(job.points)
            freqs = np.asarray(job.freqs_hz, dtype=np.float64)
            for start in range(0, len(freqs), job.chunk):
                if should_stop():
                    raise JobCancelledError(job.job_id)
                sel = freqs[start:start + job.chunk]
                p, u, _ = m.solve(sel, precision=job.precision, sound_speed=job.sound_speed, rho=job.rho,
                                  batch=len(sel))
                on_chunk(start, p, u)
        finally:
            m.release()
        if self.ctx.scratch_bytes > self.trim_above_bytes:
            self.ctx.trim()

    def run_group(self, jobs: Sequence[ServingJob],
                  on_chunks: Sequence[Callable[[int, np.ndarray, np.ndarray], None]]) -> None:
        """Solve several jobs (same precision, physics and excitation count) in one
        bem_solve_jobs call; each job's results are delivered as one chunk."""
        meshes = []
        try:
            for job in jobs:
                m = self.ctx.upload_mesh(job.vertices, job.faces)
                meshes.append(m)
                m.set_excitation(job.drive)
                m.set_observation_points(job.points)
            j0 = jobs[0]
            outs, _ = self.ctx.solve_jobs([(m, j.freqs_hz) for m, j in zip(meshes, jobs)], precision=j0.precision,
                                          sound_speed=j0.sound_speed, rho=j0.rho)
        finally:
            for m in meshes:
                m.release()
        for (p, u), cb in zip(outs, on_chunks):
            cb(0, p, u)
        if self.ctx.scratch_bytes > self.trim_above_bytes:
            self.ctx.trim()

    def close(self) -> None:
        self.ctx.close()


class ServingScheduler:
    """Run ServingJobs on one GPU with up to ``max_running`` concurrent jobs."""

    def __init__(self, device: int = 0, *, max_running: int = 4, max_queued: int = 256,
                 memory_budget_bytes: int | None = None, policy: str = "sjf", aging_s: float = 2.0,
                 executor_factory: Callable[[int], object] | None = None,
                 on_result: Callable[[ServingJob, int, np.ndarray, np.ndarray], None] | None = None,
                 group_faces: int = 3000, group_max_freqs: int = 64, group_size_ratio: float = 1.25):
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        if max_running < 1:
            raise ValueError("max_running must be >= 1")
        self.device = device
        self.max_running = max_running
        self.max_queued = max_queued
        self.policy = policy
        self.aging_s = aging_s
        self.on_result = on_result
        self.group_faces = int(group_faces)
        self.group_max_freqs = int(group_max_freqs)
        self.group_size_ratio = float(group_size_ratio)
        self._factory = executor_factory or (lambda dev: NativeExecutor(dev))
        self._budget = memory_budget_bytes if memory_budget_bytes is not None else self._default_budget(device)
        self._lock = threading.Condition()
        self._queue: list[ServingJob] = []
        self._running: list[ServingJob] = []
        self._reserved = 0
        self._done_jobs: list[ServingJob] = []
        self._closing = False
        self._ids = itertools.count()
        self._t0 = time.perf_counter()
        self._executors: list[object] = []
        self._estimator = None
        self._errors: list[BaseException] = []
        self._threads = []
        ready = threading.Barrier(max_running + 1)
        for i in range(max_running):
            t = threading.Thread(target=self._worker, args=(ready,), name=f"bem-serving-{i}", daemon=True)
            t.start()
            self._threads.append(t)
        ready.wait()
        if self._errors:
            self.close()
            raise RuntimeError(f"serving worker failed to start: {self._errors[0]}")

    @staticmethod
    def _default_budget(device: int) -> int:
        try:
            import torch  # noqa: PLC0415

            free, _total = torch.cuda.mem_get_info(device)
            return int(0.85 * free)
        except Exception:  # noqa: BLE001 - no torch / no GPU: a fixed budget
            return 64 << 30

    @property
    def memory_budget_bytes(self) -> int:
        return self._budget

    def now(self) -> float:
        return time.perf_counter() - self._t0

    # ------------------------------------------------------------------ submit
    def submit(self, job: ServingJob) -> ServingJob:
        freqs = np.asarray(job.freqs_hz, dtype=np.float64).reshape(-1)
        if freqs.size == 0:
            raise ValueError("freqs_hz must contain at least one frequency.")
        if not np.all(np.isfinite(freqs)) or np.any(freqs <= 0):
            raise ValueError("freqs_hz must contain only finite, positive values.")
        if job.chunk < 1:
            raise ValueError("chunk must be >= 1")
        job.freqs_hz = freqs
        with self._lock:
            if self._closing:
                raise RuntimeError("scheduler is closed")
            if len(self._queue) + len(self._running) >= self.max_running + self.max_queued:
                raise JobQueueFullError(
                    f"job capacity is full ({self.max_running} running, {self.max_queued} queued)")
            if not job.job_id:
                job.job_id = f"job-{next(self._ids)}"
            job.estimated_bytes = self._estimate_bytes(job)
            if job.estimated_bytes > self._budget:
                raise ValueError(f"job {job.job_id} needs ~{job.estimated_bytes / 2**30:.1f} GiB of device memory; "
                                 f"the budget is {self._budget / 2**30:.1f} GiB")
            job.estimated_work = estimated_work(job.n_faces, job.n_vertices, len(freqs))
            job.arrival_s = self.now()
            job.status = "queued"
            self._queue.append(job)
            self._lock.notify_all()
        return job

    def _estimate_bytes(self, job: ServingJob) -> int:
        ex = self._estimator
        return int(ex.footprint(job)) if ex is not None else 0

    # ---------------------------------------------------------------- schedule
    def _pick_locked(self) -> ServingJob | None:
        """Next job that fits in the memory budget, by policy; None if none fits now."""
        if not self._queue:
            return None
        free = self._budget - self._reserved
        if self.policy == "fifo":
            head = self._queue[0]
            return head if head.estimated_bytes <= free or not self._running else None
        now = self.now()
        aged = [j for j in self._queue if now - j.arrival_s >= self.aging_s]
        order = aged if aged else sorted(self._queue, key=lambda j: (j.estimated_work, j.arrival_s))
        for j in order:
            if j.estimated_bytes <= free or not self._running:
                return j
            if aged:  # an aged job waits for memory rather than being overtaken again
                return None
        return None

    def _group_locked(self, job: ServingJob, ex) -> list[ServingJob]:
        """``job`` and the queued jobs that can share its launches (see the module notes)."""
        if (self.group_faces <= 0 or job.n_faces > self.group_faces or not callable(getattr(ex, "run_group", None))
                or len(job.freqs_hz) >= self.group_max_freqs):
            return [job]
        free = self._budget - self._reserved - job.estimated_bytes
        lo = hi = job.n_vertices
        nfreq = len(job.freqs_hz)
        group = [job]
        order = self._queue if self.policy == "fifo" else sorted(self._queue, key=lambda j: (j.estimated_work, j.arrival_s))
        for j in order:
            if j is job or j.n_faces > self.group_faces:
                continue
            if (j.precision, j.sound_speed, j.rho, j.drive.shape[0]) != (job.precision, job.sound_speed, job.rho,
                                                                         job.drive.shape[0]):
                continue
            nlo, nhi = min(lo, j.n_vertices), max(hi, j.n_vertices)
            if nhi > self.group_size_ratio * nlo or nfreq + len(j.freqs_hz) > self.group_max_freqs:
                continue
            if j.estimated_bytes > free:
                continue
            group.append(j)
            lo, hi, nfreq = nlo, nhi, nfreq + len(j.freqs_hz)
            free -= j.estimated_bytes
        return group

    def _worker(self, ready: threading.Barrier) -> None:
        try:
            ex = self._factory(self.device)
        except BaseException as e:  # noqa: BLE001 - reported by the constructor
            self._errors.append(e)
            ready.wait()
            return
        with self._lock:
            self._executors.append(ex)
            if self._estimator is None:
                self._estimator = ex
        ready.wait()
        try:
            while True:
                with self._lock:
                    while True:
                        if self._closing and not self._queue:
                            return
                        job = self._pick_locked()
                        if job is not None:
                            break
                        self._lock.wait(timeout=0.05 if self.policy == "sjf" else None)
                    group = self._group_locked(job, ex)
                    for j in group:
                        j.group_size = len(group)
                        self._queue.remove(j)
                        self._running.append(j)
                        self._reserved += j.estimated_bytes
                        j.status = "running"
                        j.start_s = self.now()
                try:
                    if len(group) == 1:
                        self._run_one(ex, job)
                    else:
                        self._run_group(ex, group)
                finally:
                    with self._lock:
                        for j in group:
                            self._running.remove(j)
                            self._reserved -= j.estimated_bytes
                            j.finish_s = self.now()
                            self._done_jobs.append(j)
                        self._lock.notify_all()
                    for j in group:
                        j._done.set()
        finally:
            close = getattr(ex, "close", None)
            if close:
                close()

    def _chunk_sink(self, job: ServingJob) -> Callable[[int, np.ndarray, np.ndarray], None]:
        n = len(job.freqs_hz)

        def on_chunk(start: int, p: np.ndarray, u: np.ndarray) -> None:
            if job.pressure is None:
                job.pressure = np.zeros((n,) + p.shape[1:], dtype=np.complex128)
                job.field = np.zeros((n,) + u.shape[1:], dtype=np.complex128)
            job.pressure[start:start + len(p)] = p
            job.field[start:start + len(u)] = u
            job.solved_count = start + len(p)
            if math.isnan(job.first_result_s):
                job.first_result_s = self.now()
            if self.on_result is not None:
                self.on_result(job, start, p, u)

        return on_chunk

    def _run_one(self, ex, job: ServingJob) -> None:
        try:
            ex.run(job, self._chunk_sink(job), job._cancel.is_set)
            job.status = "completed"
        except JobCancelledError:
            job.status = "cancelled"
        except Exception as e:  # noqa: BLE001 - a failed job does not stop the worker
            job.status = "failed"
            job.error = f"{type(e).__name__}: {e}"

    def _run_group(self, ex, group: list[ServingJob]) -> None:
        live = []
        for j in group:
            if j._cancel.is_set():
                j.status = "cancelled"
            else:
                live.append(j)
        if not live:
            return
        try:
            ex.run_group(live, [self._chunk_sink(j) for j in live])
            for j in live:
                j.status = "completed"
        except Exception as e:  # noqa: BLE001 - a failed group does not stop the worker
            for j in live:
                j.status = "failed"
                j.error = f"{type(e).__name__}: {e}"

    # ------------------------------------------------------------------- close
    def drain(self, timeout: float | None = None) -> bool:
        """Wait until every submitted job has finished."""
        deadline = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while self._queue or self._running:
                left = None if deadline is None else deadline - time.perf_counter()
                if left is not None and left <= 0:
                    return False
                self._lock.wait(left)
        return True

    def close(self, cancel_pending: bool = False) -> None:
        with self._lock:
            if cancel_pending:
                for j in self._queue:
                    j.status = "cancelled"
                    j.finish_s = self.now()
                    j._done.set()
                self._queue.clear()
                for j in self._running:
                    j.cancel()
            self._closing = True
            self._lock.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close(cancel_pending=exc[0] is not None)

    # ------------------------------------------------------------------- stats
    def finished_jobs(self) -> list[ServingJob]:
        with self._lock:
            return list(self._done_jobs)


def latency_summary(jobs: Sequence[ServingJob]) -> dict:
    """p50/p99 job latency (arrival -> last result) and first-result latency, in ms."""
    done = [j for j in jobs if j.status == "completed"]
    if not done:
        return {"jobs": 0}
    lat = np.array([j.latency_s for j in done]) * 1e3
    first = np.array([j.first_result_latency_s for j in done]) * 1e3
    span = max(j.finish_s for j in done) - min(j.arrival_s for j in done)
    freqs = sum(len(j.freqs_hz) for j in done)
    return {
        "jobs": len(done),
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "first_result_p50_ms": float(np.percentile(first, 50)),
        "first_result_p99_ms": float(np.percentile(first, 99)),
        "makespan_s": float(span),
        "frequency_solves_per_s": float(freqs / span) if span > 0 else None,
        "failed": sum(j.status == "failed" for j in jobs),
        "jobs_in_shared_launches": sum(j.group_size > 1 for j in done),
    }


def poisson_jobs(n_jobs: int, rate_per_s: float, seed: int,
                 sizes: Iterable[int] = (1000, 2000, 5000, 10000, 15000), max_freqs: int = 32,
                 n_far: int = 1000) -> list[tuple[float, ServingJob]]:
    """Seeded serving stream: Poisson arrivals at ``rate_per_s``; each job a box or
    cube-sphere with a seeded piston (``meshes.seeded_piston_mesh``), size drawn
    uniformly from ``sizes`` (triangles), 1..max_freqs log-spaced frequencies in
    100 Hz - 8 kHz, observation points 2 x 73 polar + ``n_far`` Fibonacci at 2 m."""
    from . import meshes, request  # noqa: PLC0415

    rng = np.random.default_rng(seed)
    sizes = list(sizes)
    t = 0.0
    out = []
    _, horizontal, vertical, _ = request.polar_observation_points({"step_size": 5.0, "distance": 2.0})
    points = np.concatenate([horizontal, vertical, request.fibonacci_sphere(n_far, 2.0)])
    for i in range(n_jobs):
        t += float(rng.exponential(1.0 / rate_per_s))
        target = int(sizes[int(rng.integers(len(sizes)))])
        mesh = meshes.seeded_piston_mesh(target, int(rng.integers(1 << 30)))
        nfreq = int(rng.integers(1, max_freqs + 1))
        f_lo = float(rng.uniform(100.0, 1000.0))
        freqs = np.geomspace(f_lo, 8000.0, nfreq) if nfreq > 1 else np.array([f_lo])
        drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
        job = ServingJob(vertices=mesh.vertices, faces=mesh.faces, drive=drive, points=points, freqs_hz=freqs,
                         job_id=f"stream-{i}")
        out.append((t, job))
    return out


def replay(scheduler: ServingScheduler, stream: Sequence[tuple[float, ServingJob]],
           timeout_s: float = 600.0) -> list[ServingJob]:
    """Submit each job at its arrival offset (wall clock) and wait for all of them."""
    t0 = time.perf_counter()
    jobs = []
    for offset, job in stream:
        delay = offset - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        jobs.append(scheduler.submit(job))
    scheduler.drain(timeout_s)
    return jobs
