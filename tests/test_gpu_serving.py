"""Serving scheduler on the GPU: results identical alone and under a concurrent
mix (bitwise for jobs that run on their own; within 1e-8, the refinement level
of the mixed form, for small jobs that share launches with others), and a
seeded Poisson stream checked against the oracle."""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
serving = pkg_module("serving")
meshes = pkg_module("meshes")


def job_for(mesh, freqs, job_id, chunk=4):
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    pts = np.array([[0.0, 0.0, 2.0], [2.0, 0.0, 0.0], [0.0, 1.2, 1.6], [-1.0, -1.0, 1.0]])
    return serving.ServingJob(vertices=mesh.vertices, faces=mesh.faces, drive=drive, points=pts,
                              freqs_hz=np.asarray(freqs, dtype=float), chunk=chunk, job_id=job_id)


def test_results_identical_alone_and_in_a_mix(native):
    probe_mesh = meshes.seeded_piston_mesh(2000, 11)
    freqs = [300.0, 900.0, 2500.0, 4100.0, 6000.0]
    with serving.ServingScheduler(max_running=1, group_faces=0) as sch:
        alone = sch.submit(job_for(probe_mesh, freqs, "alone"))
        assert sch.drain(300)
    assert alone.status == "completed", alone.error
    with serving.ServingScheduler(max_running=4, group_faces=0) as sch:
        others = [sch.submit(job_for(meshes.seeded_piston_mesh(n, s), np.geomspace(200, 5000, k), f"o{s}"))
                  for n, s, k in ((5000, 1, 9), (1000, 2, 3), (3000, 3, 7), (8000, 4, 5), (1500, 5, 12))]
        mixed = sch.submit(job_for(probe_mesh, freqs, "mixed"))
        assert sch.drain(600)
    assert all(j.status == "completed" for j in others + [mixed]), [j.error for j in others + [mixed]]
    assert np.array_equal(alone.pressure, mixed.pressure)
    assert np.array_equal(alone.field, mixed.field)


def test_small_jobs_sharing_launches_match_alone(native):
    """Five small jobs of similar size queued behind a large one share one worker's launches
    (bem_solve_jobs); each result equals the same job run alone to 1e-8."""
    small = [(meshes.seeded_piston_mesh(1000 + 40 * s, 20 + s), np.geomspace(300, 4000, 3 + s)) for s in range(5)]
    alone = []
    with serving.ServingScheduler(max_running=1, group_faces=0) as sch:
        for i, (m, f) in enumerate(small):
            alone.append(sch.submit(job_for(m, f, f"alone{i}")))
        assert sch.drain(300)
    with serving.ServingScheduler(max_running=1, policy="fifo") as sch:
        sch.submit(job_for(meshes.seeded_piston_mesh(8000, 3), np.geomspace(200, 3000, 4), "large"))
        grouped = [sch.submit(job_for(m, f, f"g{i}")) for i, (m, f) in enumerate(small)]
        assert sch.drain(300)
    assert all(j.status == "completed" for j in alone + grouped), [j.error for j in alone + grouped]
    assert max(j.group_size for j in grouped) > 1
    for a, g in zip(alone, grouped):
        assert np.linalg.norm(g.pressure - a.pressure) <= 1e-8 * np.linalg.norm(a.pressure)
        assert np.linalg.norm(g.field - a.field) <= 1e-8 * np.linalg.norm(a.field)


def test_poisson_stream_completes_and_matches_oracle(native):
    from oracle import oracle

    stream = serving.poisson_jobs(8, 20.0, seed=4, sizes=(1000, 2000), max_freqs=6, n_far=50)
    with serving.ServingScheduler(max_running=3) as sch:
        jobs = serving.replay(sch, stream, timeout_s=600)
    assert all(j.status == "completed" for j in jobs), [j.error for j in jobs]
    summary = serving.latency_summary(jobs)
    assert summary["jobs"] == 8 and summary["p50_ms"] <= summary["p99_ms"]
    j = min(jobs, key=lambda x: x.n_faces)
    mesh = meshes.BoundaryMesh(j.vertices, j.faces, np.where(j.drive[0] != 0, meshes.RADIATOR_TAG, 1).astype(np.int32))
    i = len(j.freqs_hz) // 2
    omega = 2 * np.pi * j.freqs_hz[i]
    ref = oracle.solve_frequency(mesh, omega / j.sound_speed, j.drive[0] * 1j * j.rho * omega, j.points)
    assert np.linalg.norm(j.field[i, 0] - ref.field[:, 0]) / np.linalg.norm(ref.field[:, 0]) < 1e-5
