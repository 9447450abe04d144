"""Launch-configuration autotuner on the CPU with a fake mesh and a fake clock.

The fake mesh charges a modelled time per solve to the clock the tuner reads,
so the search itself (coordinate order, sweep scoring, rejection of candidates
whose results differ, skipping of refused ones, the caches) is checked without
a GPU.  The GPU test runs the same search on a real mesh.
"""

import json

import numpy as np
import pytest

from conftest import pkg_module

autotune = pkg_module("autotune")
native = pkg_module("native")


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeMesh:
    """cost(batch, lu_block, lu_gemm) seconds per solve of one batch; pressure = f(freqs),
    off by a relative bad_by for the configurations in bad."""

    def __init__(self, clock, cost, model_batch=6, bad=None, refuse=None, n_vertices=50, bad_by=1e-3):
        self.clock = clock
        self.bad_by = bad_by
        self.cost = cost
        self.model_batch = model_batch
        self.bad = bad or set()  # configs whose pressure is off by bad_by
        self.refuse = refuse or set()  # configs the library refuses
        self.n_vertices, self.n_faces, self.n_rhs, self.n_points = n_vertices, 96, 1, 10
        self.calls = []

    def auto_batch(self, n_freq, precision=native.BEM_PRECISION_MIXED):
        return min(self.model_batch, n_freq)

    def solve(self, freqs, *, batch, lu_block, lu_gemm, **kw):
        cfg = (batch, lu_block, lu_gemm)
        self.calls.append(cfg)
        if cfg in self.refuse:
            raise native.BemError(1, "panel width not usable on this mesh")
        assert len(freqs) == batch
        self.clock.t += self.cost(*cfg)
        f = np.asarray(freqs, dtype=np.float64)
        p = np.exp(1j * np.outer(f, np.arange(1, self.n_vertices + 1) * 1e-3))[:, None, :]
        if cfg in self.bad:
            p = p * (1 + self.bad_by)
        return p, None, {}


def batch_cost(best_batch):
    """Per-batch time: 10 ms + 1 ms per frequency, with a 5 ms penalty per frequency
    above best_batch (the panels no longer resident in one wave)."""
    def cost(b, lb, g):
        return 0.010 + 0.001 * b + 0.005 * max(0, b - best_batch)
    return cost


@pytest.fixture(autouse=True)
def fresh_cache(monkeypatch):
    monkeypatch.delenv(autotune.CACHE_ENV, raising=False)
    autotune.clear_cache()
    yield
    autotune.clear_cache()


FREQS = np.geomspace(200.0, 12000.0, 64)


def test_search_order_and_model_first():
    clock = FakeClock()
    mesh = FakeMesh(clock, batch_cost(6))
    res = autotune.tune(mesh, FREQS, clock=clock, repeats=2)
    configs = [t.config for t in res.trials]
    # batch stage: the model's choice first, then B-1, B+1, B/2; then panel widths; then the update
    assert configs[:4] == [autotune.LaunchConfig(b) for b in (6, 5, 7, 3)]
    assert [c.lu_block for c in configs[4:6]] == [32, 64]
    assert configs[6].lu_gemm == 1
    assert res.model == autotune.LaunchConfig(6)
    assert not res.cached
    # one warm-up and two timed solves per candidate
    assert len(mesh.calls) == 3 * len(configs)


def test_scored_by_the_sweep_not_the_batch():
    # per-batch rate favours larger batches, but 64 freqs in batches of 7 need 10 batches
    # against 11 of 6: the sweep score decides
    clock = FakeClock()
    res = autotune.tune(FakeMesh(clock, lambda b, lb, g: 0.020 + 0.0005 * b), FREQS, clock=clock)
    by_batch = {t.config.batch: t for t in res.trials if t.config.lu_block == 0 and t.config.lu_gemm == 0}
    for b, t in by_batch.items():
        n_batches = -(-64 // b)
        assert t.sweep_freq_per_s == pytest.approx(64 / (n_batches * (0.020 + 0.0005 * b)))
        assert t.freq_per_s == pytest.approx(b / (0.020 + 0.0005 * b))
    assert res.best.batch == max(by_batch, key=lambda b: by_batch[b].sweep_freq_per_s)


def test_picks_the_fastest_knob_by_knob():
    clock = FakeClock()

    def cost(b, lb, g):
        c = 0.010 + 0.001 * b + 0.005 * max(0, b - 5)
        if lb == 64:
            c *= 0.8
        if g == 1:
            c *= 1.5
        return c

    res = autotune.tune(FakeMesh(clock, cost), FREQS, clock=clock)
    assert res.best == autotune.LaunchConfig(5, 64, 0)


def test_rejects_a_candidate_whose_results_differ():
    clock = FakeClock()

    def cost(b, lb, g):
        return 0.001 if (b, lb, g) == (7, 0, 0) else 0.05

    res = autotune.tune(FakeMesh(clock, cost, bad={(7, 0, 0)}), FREQS, clock=clock)
    t7 = next(t for t in res.trials if t.config == autotune.LaunchConfig(7))
    assert t7.status.startswith("rejected")
    assert t7.rel_diff == pytest.approx(1e-3, rel=1e-6)
    assert res.best.batch != 7


def test_skips_a_refused_candidate():
    clock = FakeClock()
    res = autotune.tune(FakeMesh(clock, batch_cost(6), refuse={(6, 64, 0)}), FREQS, clock=clock)
    t = next(t for t in res.trials if t.config == autotune.LaunchConfig(6, 64, 0))
    assert t.status.startswith("failed") and t.freq_per_s is None
    assert res.best.lu_block != 64


def test_model_choice_failing_raises():
    clock = FakeClock()
    with pytest.raises(native.BemError):
        autotune.tune(FakeMesh(clock, batch_cost(6), refuse={(6, 0, 0)}), FREQS, clock=clock)


def test_fp64_form_has_no_update_stage_and_tighter_tolerance():
    clock = FakeClock()
    res = autotune.tune(FakeMesh(clock, batch_cost(6)), FREQS, clock=clock, precision=native.BEM_PRECISION_FP64)
    assert all(t.config.lu_gemm == 0 for t in res.trials)
    # a 1e-8 difference from the model's choice passes the mixed form's 1e-6, not FP64's 1e-9
    for precision, expect in ((native.BEM_PRECISION_MIXED, "ok"), (native.BEM_PRECISION_FP64, "rejected")):
        clock2 = FakeClock()
        res2 = autotune.tune(FakeMesh(clock2, batch_cost(6), bad={(5, 0, 0)}, bad_by=1e-8), FREQS, clock=clock2,
                             precision=precision, use_cache=False)
        t5 = next(t for t in res2.trials if t.config == autotune.LaunchConfig(5))
        assert t5.status.startswith(expect)


def test_small_sweeps_clamp_the_batches():
    clock = FakeClock()
    mesh = FakeMesh(clock, batch_cost(6), model_batch=6)
    res = autotune.tune(mesh, FREQS[:2], clock=clock)
    assert {t.config.batch for t in res.trials} <= {1, 2}
    res1 = autotune.tune(FakeMesh(clock, batch_cost(6)), FREQS[:1], clock=clock)
    assert res1.best.batch == 1
    with pytest.raises(ValueError):
        autotune.tune(mesh, [], clock=clock)


def test_process_cache_and_json_file(tmp_path, monkeypatch):
    clock = FakeClock()
    mesh = FakeMesh(clock, batch_cost(6))
    path = tmp_path / "tune" / "cache.json"
    first = autotune.tune(mesh, FREQS, clock=clock, cache_path=str(path))
    n_calls = len(mesh.calls)
    again = autotune.tune(mesh, FREQS, clock=clock, cache_path=str(path))
    assert again.cached and again.best == first.best and len(mesh.calls) == n_calls
    # a new process: only the file remains
    autotune.clear_cache()
    monkeypatch.setenv(autotune.CACHE_ENV, str(path))
    from_file = autotune.tune(mesh, FREQS, clock=clock)
    assert from_file.cached and from_file.best == first.best and len(mesh.calls) == n_calls
    data = json.loads(path.read_text())
    assert data[first.key]["batch"] == first.best.batch
    # another problem shape is a different key
    other = FakeMesh(clock, batch_cost(6), n_vertices=60)
    assert not autotune.tune(other, FREQS, clock=clock).cached
    # use_cache=False always searches
    assert not autotune.tune(mesh, FREQS, clock=clock, use_cache=False).cached


def test_result_dict_is_json():
    clock = FakeClock()
    res = autotune.tune(FakeMesh(clock, batch_cost(6)), FREQS, clock=clock)
    d = json.loads(json.dumps(res.to_dict()))
    assert d["best"]["batch"] == res.best.batch and len(d["trials"]) == len(res.trials)


def test_job_tunes_on_the_whole_sweep(tmp_path):
    """The job loop hands the whole sweep to the engine's tuner before it asks for its
    chunk size, so the tuner scores batches on every frequency of the job (not on the
    first chunk) and the chunks that follow are the winner's batch."""
    meshes = pkg_module("meshes")
    job_mod = pkg_module("job")
    mesh = meshes.sphere_with_cap(0.1, 1, 40.0)
    path = tmp_path / "s.msh"
    meshes.write_gmsh22(path, mesh.vertices * 1000.0, mesh.faces, mesh.tags)
    seen = {}

    class Engine:
        def __init__(self, **kw):
            self.batch = None

        def prepare(self, vertices, faces, drives, points, *a, **k):
            self.nv, self.n_rhs, self.n_points = len(vertices), len(drives), len(points)

        def tune_sweep(self, freqs, sound_speed, rho):
            seen["tuned"] = np.asarray(freqs).copy()
            self.batch = 5

        def preferred_chunk(self, n):
            seen["chunk_asked_after_tune"] = "tuned" in seen
            return self.batch

        def solve(self, freqs, c, rho):
            seen.setdefault("calls", []).append(len(freqs))
            n = len(freqs)

            class R:
                pressure = np.ones((n, self.n_rhs, self.nv), complex)
                field = np.ones((n, self.n_rhs, self.n_points), complex)
                stats = {}

            return R()

        def close(self):
            pass

    freqs = np.geomspace(100, 3000, 12)
    cfg = {"mesh_file": str(path), "scale_factor": 0.001, "step_size": 90.0,
           "radiators": [{"name": "cap", "tag": 2, "channel": "main"}], "channels": [{"name": "main"}]}
    job = job_mod.ExteriorJob({"config": cfg, "frequencies_hz": freqs.tolist()}, engine_factory=lambda **kw: Engine())
    out = list(job.results())
    assert len(out) == 12
    assert np.allclose(seen["tuned"], freqs.astype(np.float32))
    assert seen["chunk_asked_after_tune"] and seen["calls"] == [5, 5, 2]
