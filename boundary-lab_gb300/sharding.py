"""Frequency sharding across GPUs (one process per GPU).

Frequencies are independent given the mesh caches (each rank uploads the mesh
once), so a sweep shards by frequency batch with no data-path collective:
batch b of the sweep (frequencies [b*B, (b+1)*B)) goes to rank b % world.  The
only exchange is gathering the per-frequency results afterwards, as the
reference gathers result events on the host (solver.jl:957-996 emits one event
per frequency; the server collects them, server.py:420-439).
"""

from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def batch_owner(batch_index: int, world: int) -> int:
    return batch_index % world


def rank_batches(n_freq: int, batch: int, rank: int, world: int) -> list[np.ndarray]:
    """Index arrays of the batches owned by `rank` (round robin over batches)."""
    if batch < 1 or world < 1 or not (0 <= rank < world):
        raise ValueError("batch >= 1, world >= 1 and 0 <= rank < world are required")
    starts = range(0, n_freq, batch)
    return [np.arange(s, min(s + batch, n_freq)) for b, s in enumerate(starts) if batch_owner(b, world) == rank]


def step_batch(step: int, rank: int, world: int, batch: int, n_freq: int) -> np.ndarray:
    """Indices of the batch a rank solves at a benchmark step: batch (step * world + rank)
    of the sweep, wrapping around (weak scaling: each rank always does one batch)."""
    start = ((step * world + rank) * batch) % n_freq
    return np.array([(start + i) % n_freq for i in range(batch)])


def sweep(solve: Callable[[np.ndarray], Sequence[np.ndarray]], freqs: np.ndarray, batch: int,
          rank: int = 0, world: int = 1, dist=None) -> list[np.ndarray] | None:
    """Solve this rank's batches with ``solve(freqs_of_batch) -> arrays [len(batch), ...]``
    and gather every rank's results.  Returns, on every rank, the per-output arrays
    for the whole sweep in frequency order (``dist`` = torch.distributed or None)."""
    freqs = np.asarray(freqs, dtype=np.float64)
    mine = rank_batches(len(freqs), batch, rank, world)
    local = [(idx, [np.asarray(a) for a in solve(freqs[idx])]) for idx in mine]
    if world > 1:
        if dist is None:
            raise ValueError("world > 1 needs torch.distributed")
        gathered: list = [None] * world
        dist.all_gather_object(gathered, local)
        parts = [p for r in gathered for p in r]
    else:
        parts = local
    if not parts:
        return None
    n_out = len(parts[0][1])
    out = []
    for o in range(n_out):
        shape = parts[0][1][o].shape[1:]
        arr = np.empty((len(freqs),) + shape, dtype=parts[0][1][o].dtype)
        for idx, arrays in parts:
            arr[idx] = arrays[o]
        out.append(arr)
    return out
