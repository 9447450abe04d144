"""Timing autotuner for the launch configuration of a frequency sweep.

The library picks its runtime launch configuration from a model of the device:

* ``bem_auto_batch``: the largest batch of frequencies whose LU cluster panels
  are resident on the GPU at once (15 at 10k triangles on a GB300);
* the LU's panel width and cluster size: the pair that runs every panel of
  the batch in the fewest waves (``lu_block`` 0);
* the trailing update of the mixed form: tcgen05 3xFP16 when the device has it
  (``lu_gemm`` 0).

``tune`` checks that model by timing.  It solves a few frequencies of the
caller's sweep on the uploaded mesh with each candidate configuration, keeps the
fastest one whose results agree with the model's choice, and caches the winner
per device and problem shape.  The knobs are searched one at a time, starting
from the model's choice (a coordinate search):

1. batch: the model's B, B - 1, B + 1 and B / 2 (within 1 .. min(64, n_freq));
2. LU panel width: automatic, 32 and 64, at the best batch;
3. LU trailing update, mixed form only: tcgen05 3xFP16 or cuBLAS cgemm.

A candidate that the library refuses (``BemError``) is skipped and recorded.
A candidate whose pressure differs from the model choice's by more than the
tolerance is rejected: the tuner never trades accuracy for time.

The reference has no tuner: its CUDA backend launches fixed block sizes
(128 threads for the assembly, src/blab/solvers/julia_local/src/BeatEngineCudaAssembly.jl:31;
256 for the field, BeatEngineCudaField.jl:216, :232).  The configuration chosen
here only changes how the same sweep is scheduled, never the discretisation.
"""

from __future__ import annotations

import json
import os
import threading
import time
from dataclasses import asdict, dataclass, field
from typing import Callable

import numpy as np

from . import native

CACHE_ENV = "GB300_BEM_AUTOTUNE_CACHE"  # optional JSON file that keeps winners across processes


@dataclass(frozen=True)
class LaunchConfig:
    batch: int  # frequencies factored together (bem_solve_options.batch)
    lu_block: int = 0  # 0 automatic, 32 or 64
    lu_gemm: int = 0  # 0 automatic, 1 cuBLAS cgemm, 2 tcgen05 3xFP16


@dataclass
class Trial:
    config: LaunchConfig
    freq_per_s: float | None  # frequency solves per second of one batch (best of the repeats)
    sweep_freq_per_s: float | None  # the same for the whole sweep: ceil(n_freq / batch) batches
    rel_diff: float | None  # max relative pressure difference against the model's choice
    status: str  # "ok", "rejected: ...", "failed: ..."


@dataclass
class TuneResult:
    best: LaunchConfig
    model: LaunchConfig  # the library's own choice (the starting point)
    key: str
    trials: list[Trial] = field(default_factory=list)
    cached: bool = False

    def to_dict(self) -> dict:
        return {"best": asdict(self.best), "model": asdict(self.model), "key": self.key, "cached": self.cached,
                "trials": [{"config": asdict(t.config), "freq_per_s": t.freq_per_s,
                            "sweep_freq_per_s": t.sweep_freq_per_s, "rel_diff": t.rel_diff, "status": t.status}
                           for t in self.trials]}


_cache: dict[str, dict] = {}
_cache_lock = threading.Lock()


def device_name(device: int) -> str:
    try:
        import torch  # noqa: PLC0415 - plumbing only, for the device's name

        return torch.cuda.get_device_name(device)
    except Exception:  # noqa: BLE001 - no torch or no GPU: the ordinal stands in
        return f"cuda:{device}"


def cache_key(dev_name: str, precision: int, mesh, n_freq: int) -> str:
    return (f"{dev_name}|precision={precision}|nv={mesh.n_vertices}|nf={mesh.n_faces}|rhs={mesh.n_rhs}"
            f"|points={mesh.n_points}|nfreq={n_freq}")


def _load_file(path: str) -> dict:
    try:
        with open(path, encoding="utf-8") as fh:
            data = json.load(fh)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(key: str, best: LaunchConfig, path: str | None) -> None:
    with _cache_lock:
        _cache[key] = asdict(best)
        if path:
            data = _load_file(path)
            data[key] = asdict(best)
            os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
            tmp = f"{path}.{os.getpid()}.tmp"
            with open(tmp, "w", encoding="utf-8") as fh:
                json.dump(data, fh, indent=1, sort_keys=True)
            os.replace(tmp, path)


def _lookup(key: str, path: str | None) -> LaunchConfig | None:
    with _cache_lock:
        hit = _cache.get(key)
        if hit is None and path:
            hit = _load_file(path).get(key)
            if hit is not None:
                _cache[key] = hit
    if hit is None:
        return None
    try:
        return LaunchConfig(int(hit["batch"]), int(hit.get("lu_block", 0)), int(hit.get("lu_gemm", 0)))
    except (KeyError, TypeError, ValueError):
        return None


def clear_cache() -> None:
    """Forget the winners kept in this process (the JSON file, if any, is left alone)."""
    with _cache_lock:
        _cache.clear()


def _sample(freqs_hz, n: int) -> np.ndarray:
    f = np.asarray(freqs_hz, dtype=np.float64).reshape(-1)
    if len(f) <= n:
        return f.copy()
    return f[np.round(np.linspace(0, len(f) - 1, n)).astype(int)]


def tune(mesh, freqs_hz, *, precision: int = native.BEM_PRECISION_MIXED, sound_speed: float = 343.0,
         rho: float = 1.21, refine_tol: float = 1e-10, repeats: int = 2, tol: float | None = None,
         device: int | None = None, cache_path: str | None = None, use_cache: bool = True,
         clock: Callable[[], float] = time.perf_counter) -> TuneResult:
    """Pick the fastest launch configuration for solving ``freqs_hz`` on ``mesh``.

    ``mesh`` is an uploaded ``native.Mesh`` with its excitation and observation
    points set (anything with the same ``solve``/``auto_batch`` methods and
    ``n_vertices``/``n_faces``/``n_rhs``/``n_points`` attributes works).  Each
    candidate solves its first ``batch`` frequencies of an evenly spread sample
    of the sweep: one warm-up solve, then ``repeats`` timed ones.  It is scored
    by the sweep's rate, n_freq / (ceil(n_freq / batch) x best time).  ``tol`` bounds the relative pressure difference against
    the model's choice on the sample's first frequency (default 1e-6 for the
    mixed form, 1e-9 for FP64).  ``cache_path`` (default: the
    ``GB300_BEM_AUTOTUNE_CACHE`` environment variable) keeps winners in a JSON
    file; the process-wide cache is always used unless ``use_cache`` is false.
    """
    freqs = np.asarray(freqs_hz, dtype=np.float64).reshape(-1)
    if freqs.size == 0:
        raise ValueError("autotune needs at least one frequency")
    if repeats < 1:
        raise ValueError("repeats must be >= 1")
    n_freq = len(freqs)
    mixed = precision == native.BEM_PRECISION_MIXED
    tol = (1e-6 if mixed else 1e-9) if tol is None else float(tol)
    dev = getattr(getattr(mesh, "ctx", None), "device", 0) if device is None else device
    path = cache_path if cache_path is not None else (os.environ.get(CACHE_ENV) or None)
    key = cache_key(device_name(dev), precision, mesh, n_freq)
    b0 = max(1, min(int(mesh.auto_batch(n_freq, precision)), n_freq, 64))
    model = LaunchConfig(b0)
    if use_cache:
        hit = _lookup(key, path)
        if hit is not None:
            return TuneResult(best=hit, model=model, key=key, cached=True)

    cap = min(64, n_freq)
    batches = []
    for b in (b0, b0 - 1, b0 + 1, b0 // 2):
        if 1 <= b <= cap and b not in batches:
            batches.append(b)
    sample = _sample(freqs, max(batches))
    trials: list[Trial] = []
    reference: dict[str, np.ndarray] = {}

    def run(cfg: LaunchConfig) -> Trial:
        fs = sample[:cfg.batch]
        kw = dict(precision=precision, sound_speed=sound_speed, rho=rho, refine_tol=refine_tol, batch=cfg.batch,
                  lu_block=cfg.lu_block, lu_gemm=cfg.lu_gemm, want_field=True)
        try:
            p, _u, _st = mesh.solve(fs, **kw)  # warm-up: lazy loading, scratch growth
            best = None
            for _ in range(repeats):
                t0 = clock()
                mesh.solve(fs, **kw)
                dt = clock() - t0
                best = dt if best is None else min(best, dt)
        except native.BemError as exc:
            return Trial(cfg, None, None, None, f"failed: {exc}")
        first = np.asarray(p)[0]
        if "p" not in reference:
            reference["p"] = first
            diff = 0.0
        else:
            ref = reference["p"]
            scale = float(np.max(np.abs(ref))) or 1.0
            diff = float(np.max(np.abs(first - ref))) / scale
        best = max(best, 1e-9)
        rate = cfg.batch / best
        # a sweep runs ceil(n_freq / batch) batches; the last, partial one costs about a full
        # one (the LU panels are latency-bound whatever the number of matrices)
        sweep = n_freq / (-(-n_freq // cfg.batch) * best)
        if not np.isfinite(diff) or diff > tol:
            return Trial(cfg, rate, sweep, diff, f"rejected: pressure differs from the model choice by {diff:.3g}")
        return Trial(cfg, rate, sweep, diff, "ok")

    def best_ok(pool: list[Trial]) -> Trial | None:
        ok = [t for t in pool if t.status == "ok"]
        return max(ok, key=lambda t: t.sweep_freq_per_s) if ok else None

    # 1. batch (the model's choice first: it is the accuracy reference)
    stage = [run(LaunchConfig(b)) for b in batches]
    trials += stage
    if stage[0].status != "ok":
        # the model's own configuration failed: nothing to compare against
        raise native.BemError(2, f"autotune: the library's own configuration failed ({stage[0].status})")
    cur = best_ok(stage)
    # 2. LU panel width at the best batch
    stage = [cur] + [run(LaunchConfig(cur.config.batch, lb, 0)) for lb in (32, 64)]
    trials += stage[1:]
    cur = best_ok(stage)
    # 3. trailing update (mixed form): cuBLAS cgemm against the automatic tcgen05 choice
    if mixed:
        stage = [cur, run(LaunchConfig(cur.config.batch, cur.config.lu_block, 1))]
        trials += stage[1:]
        cur = best_ok(stage)
    result = TuneResult(best=cur.config, model=model, key=key, trials=trials)
    if use_cache:
        _store(key, cur.config, path)
    return result
