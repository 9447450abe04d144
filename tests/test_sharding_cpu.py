"""Frequency sharding over 2 gloo ranks on the CPU: every batch solved exactly
once, results gathered in frequency order and equal to the single-process sweep
(solver: the FP64 oracle on a small sphere)."""

import os
import socket

import numpy as np
import pytest

from conftest import pkg_module

sharding = pkg_module("sharding")
meshes = pkg_module("meshes")


def test_rank_batches_partition_the_sweep():
    for n, b, w in ((64, 16, 1), (64, 16, 2), (65, 16, 4), (7, 3, 5), (1, 4, 2)):
        seen = np.concatenate([np.concatenate(sharding.rank_batches(n, b, r, w) or [np.array([], int)])
                               for r in range(w)])
        assert np.array_equal(np.sort(seen), np.arange(n))
    assert [list(x) for x in sharding.rank_batches(10, 3, 1, 2)] == [[3, 4, 5], [9]]
    assert list(sharding.step_batch(1, 1, 2, 4, 10)) == [2, 3, 4, 5]
    with pytest.raises(ValueError):
        sharding.rank_batches(10, 0, 0, 1)


def _problem():
    mesh = meshes.sphere_with_cap(0.1, 1, 40.0)
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)
    pts = np.array([[0.0, 0.0, 1.5], [1.5, 0.0, 0.0], [0.3, 0.4, -1.2]])
    return mesh, drive, pts


def _solve(freqs):
    from oracle import oracle

    mesh, drive, pts = _problem()
    p, u = [], []
    for f in freqs:
        omega = 2 * np.pi * f
        sol = oracle.solve_frequency(mesh, omega / 343.0, drive * 1j * 1.205 * omega, pts, threads=1)
        p.append(sol.pressure[:, 0])
        u.append(sol.field[:, 0])
    return np.array(p), np.array(u)


def _rank_main(rank, world, port, freqs, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = sharding.sweep(_solve, freqs, 2, rank, world, dist)
        if rank == 0:
            np.savez(out_path, p=res[0], u=res[1])
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_single_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.build import build_oracle

    build_oracle()
    freqs = np.array([150.0, 400.0, 900.0, 1500.0, 2200.0])
    out = tmp_path / "sharded.npz"
    mp.spawn(_rank_main, args=(2, _free_port(), freqs, str(out)), nprocs=2, join=True)
    got = np.load(out)
    p_ref, u_ref = sharding.sweep(_solve, freqs, 2)
    assert np.array_equal(got["p"], p_ref) and np.array_equal(got["u"], u_ref)
    assert torch is not None


def test_bench_gpus_flag_starts_one_rank_per_gpu():
    """``bench.py --gpus 2`` started without a launcher starts two ranks itself
    (torch.distributed.run); in --plan mode each rank reports its frequency batches
    (no GPU work) and rank 0 prints them: two ranks, disjoint batches in every step."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    env = {k: v for k, v in __import__("os").environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--gpus", "2", "--plan", "--batch", "8",
                          "--lanes", "1", "--steps", "3", "--warmup", "3"], capture_output=True, text=True, timeout=240,
                         env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    plan = json.loads(lines[0])
    assert plan["n_gpus"] == 2 and len(plan["rank_batches"]) == 2
    for step in range(3 + 3):
        a, b = (set(plan["rank_batches"][r][step]) for r in range(2))
        assert len(a) == len(b) == 8 and not (a & b)
