"""Serving scheduler logic on the CPU with a fake executor (no GPU).

Mirrors the reference's job-orchestrator tests: capacity rejection
(server.py:216-223), input validation (:206-214), cancel between frequency
chunks, a failing job reported without stopping the server; plus what the GB300
scheduler adds: concurrent running jobs, memory admission, shortest-job-first
with aging, and per-chunk result streaming.
"""

import threading
import time

import numpy as np
import pytest

from conftest import pkg_module

serving = pkg_module("serving")


class FakeExecutor:
    """Sleeps `per_freq_s` per frequency; footprint = 1 MiB per face."""

    log: list = []
    lock = threading.Lock()
    active = 0
    max_active = 0

    def __init__(self, device, per_freq_s=0.002, fail_on=None):
        self.per_freq_s = per_freq_s
        self.fail_on = fail_on

    def footprint(self, job):
        return job.n_faces << 20

    def run(self, job, on_chunk, should_stop):
        cls = FakeExecutor
        with cls.lock:
            cls.active += 1
            cls.max_active = max(cls.max_active, cls.active)
            cls.log.append(job.job_id)
        try:
            if self.fail_on and job.job_id == self.fail_on:
                raise RuntimeError("solver exploded")
            n = len(job.freqs_hz)
            for start in range(0, n, job.chunk):
                if should_stop():
                    raise serving.JobCancelledError(job.job_id)
                k = min(job.chunk, n - start)
                time.sleep(self.per_freq_s * k)
                p = np.full((k, 1, job.n_vertices), job.n_faces, dtype=np.complex128)
                u = np.full((k, 1, len(job.points)), start, dtype=np.complex128)
                on_chunk(start, p, u)
        finally:
            with cls.lock:
                cls.active -= 1

    def close(self):
        pass


def make_job(n_faces, n_freq, job_id="", chunk=4):
    return serving.ServingJob(vertices=np.zeros((n_faces // 2 + 2, 3)), faces=np.zeros((n_faces, 3), np.int32),
                              drive=np.ones((1, n_faces), np.complex128), points=np.zeros((5, 3)),
                              freqs_hz=np.geomspace(100, 1000, n_freq), chunk=chunk, job_id=job_id)


@pytest.fixture(autouse=True)
def reset_fake():
    FakeExecutor.log = []
    FakeExecutor.active = 0
    FakeExecutor.max_active = 0


def test_jobs_complete_and_results_stream_per_chunk():
    seen = []
    with serving.ServingScheduler(max_running=2, memory_budget_bytes=1 << 40, executor_factory=FakeExecutor,
                                  on_result=lambda j, s, p, u: seen.append((j.job_id, s, len(p)))) as sch:
        jobs = [sch.submit(make_job(100 * (i + 1), 10, f"j{i}")) for i in range(4)]
        assert sch.drain(30)
    for j in jobs:
        assert j.status == "completed" and j.solved_count == 10
        assert j.pressure.shape == (10, 1, j.n_vertices)
        assert np.all(j.pressure.real == j.n_faces)
        assert j.arrival_s <= j.start_s <= j.first_result_s <= j.finish_s
    assert sorted(s for jid, s, _ in seen if jid == "j0") == [0, 4, 8]
    summary = serving.latency_summary(jobs)
    assert summary["jobs"] == 4 and summary["p50_ms"] <= summary["p99_ms"]


def test_concurrent_jobs_share_the_gpu():
    with serving.ServingScheduler(max_running=3, memory_budget_bytes=1 << 40,
                                  executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.01)) as sch:
        for i in range(6):
            sch.submit(make_job(100, 8, f"c{i}"))
        assert sch.drain(30)
    assert FakeExecutor.max_active == 3


def test_memory_admission_limits_concurrency():
    # budget fits one 600-face job (600 MiB) at a time although 3 workers exist
    with serving.ServingScheduler(max_running=3, memory_budget_bytes=700 << 20, policy="fifo",
                                  executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.005)) as sch:
        for i in range(4):
            sch.submit(make_job(600, 6, f"m{i}"))
        assert sch.drain(30)
    assert FakeExecutor.max_active == 1
    assert FakeExecutor.log == ["m0", "m1", "m2", "m3"]


def test_job_larger_than_budget_is_rejected():
    with serving.ServingScheduler(max_running=1, memory_budget_bytes=100 << 20, executor_factory=FakeExecutor) as sch:
        with pytest.raises(ValueError, match="budget"):
            sch.submit(make_job(200, 2))


def test_capacity_rejection_and_validation():
    with serving.ServingScheduler(max_running=1, max_queued=2, memory_budget_bytes=1 << 40,
                                  executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.05)) as sch:
        for i in range(3):
            sch.submit(make_job(10, 4, f"q{i}"))
        with pytest.raises(serving.JobQueueFullError):
            sch.submit(make_job(10, 4, "overflow"))
        with pytest.raises(ValueError):
            sch.submit(make_job(10, 0))
        bad = make_job(10, 3)
        bad.freqs_hz = np.array([100.0, -1.0, 200.0])
        with pytest.raises(ValueError):
            sch.submit(bad)
        sch.close(cancel_pending=True)


def test_sjf_runs_small_jobs_first_and_fifo_keeps_order():
    def run(policy):
        FakeExecutor.log = []
        with serving.ServingScheduler(max_running=1, memory_budget_bytes=1 << 40, policy=policy, aging_s=60.0,
                                      executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.01)) as sch:
            sch.submit(make_job(50, 4, "blocker"))  # occupies the single worker while the others queue
            time.sleep(0.01)
            for name, nf in (("big", 5000), ("small", 100), ("mid", 1000)):
                sch.submit(make_job(nf, 4, name))
            assert sch.drain(30)
        return FakeExecutor.log

    assert run("fifo") == ["blocker", "big", "small", "mid"]
    assert run("sjf") == ["blocker", "small", "mid", "big"]


def test_aging_prevents_starvation():
    with serving.ServingScheduler(max_running=1, memory_budget_bytes=1 << 40, policy="sjf", aging_s=0.05,
                                  executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.02)) as sch:
        sch.submit(make_job(50, 3, "blocker"))
        time.sleep(0.005)
        sch.submit(make_job(9000, 2, "old-big"))
        time.sleep(0.1)  # old-big is now past aging_s
        sch.submit(make_job(10, 2, "new-small"))
        assert sch.drain(30)
    assert FakeExecutor.log.index("old-big") < FakeExecutor.log.index("new-small")


def test_cancel_between_chunks_and_failure_isolated():
    with serving.ServingScheduler(max_running=2, memory_budget_bytes=1 << 40,
                                  executor_factory=lambda d: FakeExecutor(d, per_freq_s=0.01, fail_on="bad")) as sch:
        long = sch.submit(make_job(100, 40, "long", chunk=2))
        bad = sch.submit(make_job(100, 4, "bad"))
        time.sleep(0.05)
        long.cancel()
        ok = sch.submit(make_job(100, 4, "ok"))
        assert sch.drain(30)
    assert long.status == "cancelled" and 0 < long.solved_count < 40
    assert bad.status == "failed" and "solver exploded" in bad.error
    assert ok.status == "completed"


def test_poisson_stream_is_seeded():
    a = serving.poisson_jobs(6, 20.0, seed=3, sizes=(1000, 2000), max_freqs=4, n_far=10)
    b = serving.poisson_jobs(6, 20.0, seed=3, sizes=(1000, 2000), max_freqs=4, n_far=10)
    assert [t for t, _ in a] == [t for t, _ in b]
    for (_, x), (_, y) in zip(a, b):
        assert np.array_equal(x.faces, y.faces) and np.array_equal(x.freqs_hz, y.freqs_hz)
        assert 1 <= len(x.freqs_hz) <= 4 and np.any(x.drive != 0)
    gaps = np.diff([0.0] + [t for t, _ in serving.poisson_jobs(200, 20.0, seed=5, sizes=(1000,), max_freqs=1,
                                                                  n_far=4)])
    assert 0.035 < gaps.mean() < 0.07  # exponential gaps, mean 1 / 20 s


class GroupingExecutor(FakeExecutor):
    """FakeExecutor that also solves groups of jobs (bem_solve_jobs): records each group."""

    groups: list = []

    def run_group(self, jobs, on_chunks):
        cls = GroupingExecutor
        with cls.lock:
            cls.groups.append([j.job_id for j in jobs])
        time.sleep(self.per_freq_s * sum(len(j.freqs_hz) for j in jobs) / 4)
        for j, cb in zip(jobs, on_chunks):
            n = len(j.freqs_hz)
            cb(0, np.full((n, 1, j.n_vertices), j.n_faces, dtype=np.complex128),
               np.zeros((n, 1, len(j.points)), dtype=np.complex128))


def test_small_jobs_of_similar_size_share_launches():
    """Queued small jobs of similar size are taken together by one worker; a large job, a
    job of a very different size and jobs beyond the frequency cap are not."""
    GroupingExecutor.groups = []
    gate = threading.Event()

    class Gated(GroupingExecutor):
        def run(self, job, on_chunk, should_stop):
            if job.job_id == "blocker":
                gate.wait(10)
            super().run(job, on_chunk, should_stop)

    with serving.ServingScheduler(max_running=1, memory_budget_bytes=1 << 40, executor_factory=Gated,
                                  policy="fifo", group_faces=3000, group_max_freqs=40) as sch:
        sch.submit(make_job(20000, 2, "blocker"))  # holds the only worker while the queue fills
        time.sleep(0.1)
        a = [sch.submit(make_job(1000 + 20 * i, 8, f"a{i}")) for i in range(4)]  # similar sizes, 32 freqs
        b = sch.submit(make_job(1100, 12, "b"))        # similar size, but beyond the 40-frequency cap
        c = sch.submit(make_job(2800, 4, "c"))         # small, but 2.7x the vertices of a0
        big = sch.submit(make_job(6000, 4, "big"))     # not small
        gate.set()
        assert sch.drain(30)
    groups = GroupingExecutor.groups
    assert ["a0", "a1", "a2", "a3"] in groups
    assert all(len(g) <= 5 for g in groups)
    assert all("c" not in g or g == ["c"] for g in groups) and all("big" not in g for g in groups)
    assert all(j.status == "completed" and j.group_size == 4 for j in a)
    assert b.status == c.status == big.status == "completed"
    assert np.all(a[2].pressure == a[2].n_faces) and a[2].pressure.shape == (8, 1, a[2].n_vertices)


def test_grouping_can_be_switched_off():
    GroupingExecutor.groups = []
    with serving.ServingScheduler(max_running=1, memory_budget_bytes=1 << 40, executor_factory=GroupingExecutor,
                                  group_faces=0) as sch:
        jobs = [sch.submit(make_job(1000, 4, f"s{i}")) for i in range(4)]
        assert sch.drain(30)
    assert GroupingExecutor.groups == [] and all(j.group_size == 1 for j in jobs)
