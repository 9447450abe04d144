#!/usr/bin/env python
"""Benchmark of the GB300 exterior Helmholtz BEM hot path.

Workload (the mixed-precision configuration): closed box 0.3 x 0.2 x 0.25 m,
~10,000 triangles, circular piston (r = 5 cm) on the front face, 64
log-spaced frequencies 200 Hz - 12 kHz, far field at 2 x 73 polar points plus
2000 Fibonacci-sphere points at 2 m.  One step = one batch of frequencies
solved end to end (assembly, LU factorisation with FP64 iterative refinement,
field evaluation).  Metric: frequency solves/s.

Arms:
  default           this repository's CUDA path (one GPU per rank, frequencies
                    sharded across ranks: weak scaling, no collective on the
                    data path)
  --impl reference  the reference's algorithm on the host cores: the FP32 CPU
                    restatement of the BEAT CPU engine (the Julia engine itself
                    cannot run on these machines), one frequency per step
"""

from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "frequency solves/s @10k tris (mixed vs FP64, ≤1e-5 err); p50/p99 latency"
UNIT = "frequency-solves/s"
SOUND_SPEED = 343.0
RHO = 1.205


def pkg(name: str):
    return importlib.import_module("boundary-lab_gb300." + name)


def workload(faces: int = 10000):
    meshes = pkg("meshes")
    request = pkg("request")
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), faces, 0.05, "+z")
    _, horizontal, vertical, _ = request.polar_observation_points({"step_size": 5.0, "distance": 2.0})
    sphere = request.fibonacci_sphere(2000, 2.0)
    points = np.vstack([horizontal, vertical, sphere])
    freqs = np.logspace(np.log10(200.0), np.log10(12000.0), 64)
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    return mesh, points, freqs, drive


def describe(mesh, points, freqs) -> str:
    return (f"closed box 0.3x0.2x0.25 m, {mesh.n_faces} triangles ({mesh.n_vertices} P1 dofs), circular piston r=5 cm "
            f"on +z ({int((mesh.tags == 2).sum())} faces); {len(freqs)} log-spaced freqs 200 Hz-12 kHz; "
            f"{len(points)} observation points (2x73 polar + 2000 Fibonacci at 2 m)")


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        return False

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def cpu_oracle_step(mesh, points, freq, drive, threads: int) -> float:
    """One frequency of the reference algorithm in FP32 on the host (assembly, BM system, LU, field)."""
    from oracle import oracle

    t0 = time.perf_counter()
    omega = 2 * np.pi * freq
    q = (drive[0] * (1j * RHO * omega)).astype(np.complex64)
    oracle.solve_frequency(mesh, omega / SOUND_SPEED, q, points, precision="f32", threads=threads)
    return time.perf_counter() - t0


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, points, freqs, drive = workload(args.faces)
    threads = os.cpu_count() or 1
    from oracle.build import build_oracle

    build_oracle()
    # The host path has nothing to warm up beyond one small solve (page-in of the
    # library and of OpenBLAS); timed steps are capped at 6 full-size frequencies so
    # the run stays within a few minutes whatever --steps asks for.
    small_mesh, small_points, _, small_drive = workload(600)
    for _ in range(args.warmup):
        cpu_oracle_step(small_mesh, small_points[:64], 500.0, small_drive, threads)
    timed = min(args.steps, 6)
    sel = [freqs[(i * 13) % len(freqs)] for i in range(timed)]
    times = [cpu_oracle_step(mesh, points, f, drive, threads) for f in sel]
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": describe(mesh, points, freqs), "step": "1 frequency (bounded sample)",
                   "timed_steps": len(times), "warmup": "one small solve per warm-up step"},
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "1 frequency of the 10k-triangle box per step: FP32 restatement of BEAT CPU assembly "
                      "(colored OpenMP), BM system, LAPACK cgetrf/cgetrs (scipy OpenBLAS), field",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--faces", type=int, default=10000)
    ap.add_argument("--fp64-freqs", type=int, default=2, help="frequencies timed in the plain FP64 form")
    ap.add_argument("--cpu-baseline", type=int, default=1, help="frequencies timed on the host for cpu_baseline")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-extras", action="store_true", help="skip FP64 form, e2e and CPU baseline (profiling runs)")
    ap.add_argument("--serving-jobs", type=int, default=40, help="jobs in the seeded Poisson serving stream (0: skip)")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="serving arrivals per second")
    ap.add_argument("--serving-running", type=int, default=4, help="concurrent jobs on the GPU")
    ap.add_argument("--lu-gemm", type=int, default=0, choices=[0, 1, 2],
                    help="LU trailing update: 0 automatic, 1 cuBLAS cgemm, 2 tcgen05 3xTF32")
    args = ap.parse_args()
    if args.warmup < 3 and not args.no_extras:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    native = pkg("native")
    native.load()
    mesh, points, freqs, drive = workload(args.faces)
    B = args.batch
    ctx = native.Context(local_rank)
    m = ctx.upload_mesh(mesh.vertices, mesh.faces)
    m.set_excitation(drive)
    m.set_observation_points(points)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=f"cuda:{local_rank}")
    p_dev = torch.empty((B, 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
    u_dev = torch.empty((B, 1, len(points)), dtype=torch.complex128, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    opts = dict(precision=native.BEM_PRECISION_MIXED, sound_speed=SOUND_SPEED, rho=RHO, batch=B, refine_tol=1e-10,
                max_refine=8, lu_gemm=args.lu_gemm)

    sharding = pkg("sharding")

    def step_freqs(step: int):
        # weak scaling: rank r takes batch (step * world + r) of the sweep
        return freqs[sharding.step_batch(step, rank, world, B, len(freqs))]

    for s in range(args.warmup):
        m.solve_device(step_freqs(s), p_dev.data_ptr(), u_dev.data_ptr(), **opts)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev_start = torch.cuda.Event(enable_timing=True)
    ev_end = torch.cuda.Event(enable_timing=True)
    step_events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats_list = []
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev_start.record(stream)
            for s in range(args.steps):
                flush.fill_(float(s))  # write 256 MiB (> 129 MB L2) between steps
                step_events[s][0].record(stream)
                stats_list.append(m.solve_device(step_freqs(args.warmup + s), p_dev.data_ptr(), u_dev.data_ptr(),
                                                 profile=1, **opts))
                step_events[s][1].record(stream)
            ev_end.record(stream)
        torch.cuda.synchronize()
    elapsed = ev_start.elapsed_time(ev_end) / 1e3
    if dist:
        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    solved = args.steps * B * world
    value = solved / elapsed
    step_ms = [a.elapsed_time(b) for a, b in step_events]
    kernel_s = {k: sum(st["kernel_s"][k] for st in stats_list) for k in stats_list[0]["kernel_s"]}
    per_freq_ms = {k: 1e3 * v / (args.steps * B) for k, v in kernel_s.items()}

    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (compensated) + f64 refinement",
        "data": "synthetic",
        "config": {"workload": describe(mesh, points, freqs), "form": "mixed", "batch": B,
                   "l2": "256 MiB buffer written before every timed step (> 129 MB L2)",
                   "parallelism": f"replicas x{world}, frequencies sharded"},
        "clocks": clocks.summary(),
        "stage_ms_per_freq": per_freq_ms,
        "step_ms": step_ms,
        "refine_steps_max": max(st["max_refine_steps"] for st in stats_list),
        "lu_trailing_update": {1: "cublas cgemm", 2: "tcgen05 3xTF32"}.get(stats_list[0]["lu_gemm_used"]),
        "rel_residual_max": max(st["max_rel_residual"] for st in stats_list),
    }

    # dominant kernel roofline: regular-pair assembly, FP32 pipe
    st0 = stats_list[0]
    regular_qpairs = st0["regular_pairs"] * 36
    flops_per_qpair = 101  # counted from regular_f32_kernel (FMA = 2 flop), see the design doc
    reg_s = kernel_s["regular"] / (args.steps * B)
    achieved = regular_qpairs * flops_per_qpair / reg_s / 1e12 if reg_s > 0 else None
    clock = result["clocks"]["sm_mhz"] or 1920.0
    fp32_peak = 152 * 128 * 2 * clock * 1e6 / 1e12
    result["roofline"] = {
        "kernel": "regular_f32_kernel (regular face-pair assembly)",
        "bound": "fp32",
        "achieved": achieved,
        "peak": fp32_peak,
        "unit": "TFLOP/s",
        "frac": (achieved / fp32_peak) if achieved else None,
        # DRAM bytes per launch from one ncu capture of this kernel at this workload
        # (dram__bytes_read.sum + dram__bytes_write.sum, current source); the
        # algorithmic bytes are the extended-row output, 3 x N_f x ldR x 8 B = 1.360e9
        "traffic": 1.3146e9 if args.faces == 10000 else None,
        "peak_source": "152 SMs x 128 FP32 lanes x 2 flop x median SM clock sampled during the run "
                       "(MEASURED_PEAKS.json has no FP32 figure)",
        "work_per_launch": f"{regular_qpairs:.4g} q-pairs x {flops_per_qpair} flop",
    }

    if not args.no_extras and rank == 0:
        # plain FP64 form on a subset, and the mixed-form error against it
        sel = freqs[[10, 50, 30, 60][: args.fp64_freqs]]
        ev_a, ev_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p64 = torch.empty((len(sel), 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
        u64 = torch.empty((len(sel), 1, len(points)), dtype=torch.complex128, device="cuda")
        with torch.cuda.stream(stream):
            ev_a.record(stream)
            st64 = m.solve_device(sel, p64.data_ptr(), u64.data_ptr(), precision=native.BEM_PRECISION_FP64,
                                  sound_speed=SOUND_SPEED, rho=RHO, batch=len(sel), profile=1)
            ev_b.record(stream)
        torch.cuda.synchronize()
        t64 = ev_a.elapsed_time(ev_b) / 1e3
        pm = torch.empty_like(p64)
        um = torch.empty_like(u64)
        m.solve_device(sel, pm.data_ptr(), um.data_ptr(), **{**opts, "batch": len(sel)})
        torch.cuda.synchronize()
        errs = [float(torch.linalg.norm(um[i] - u64[i]) / torch.linalg.norm(u64[i])) for i in range(len(sel))]
        perr = [float(torch.linalg.norm(pm[i] - p64[i]) / torch.linalg.norm(p64[i])) for i in range(len(sel))]
        v64 = len(sel) / t64
        result["fp64_form"] = {"value": v64, "unit": UNIT, "freqs_hz": [float(f) for f in sel],
                               "stage_ms_per_freq": {k: 1e3 * v / len(sel) for k, v in st64["kernel_s"].items()}}
        result["speedup_vs_fp64"] = value / world / v64
        result["max_rel_far_field_err_vs_fp64"] = max(errs)
        result["max_rel_surface_pressure_err_vs_fp64"] = max(perr)

        # end to end through the C ABI with host buffers: upload mesh + caches, solve a batch, copy results back
        e2e_times = []
        h2d = mesh.vertices.nbytes + mesh.faces.astype(np.int32).nbytes + drive.nbytes + points.nbytes + B * 8
        d2h = B * (mesh.n_vertices + len(points)) * 16
        for s in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m2 = ctx.upload_mesh(mesh.vertices, mesh.faces)
            m2.set_excitation(drive)
            m2.set_observation_points(points)
            m2.solve(step_freqs(s), **opts)
            m2.release()
            e2e_times.append(time.perf_counter() - t0)
        result["e2e"] = {"value": B / statistics.median(e2e_times), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                         "d2h_bytes_per_step": int(d2h),
                         "what": "per step: bem_upload_mesh (plan + FP64 singular moments) + excitation + points from "
                                 "host arrays, bem_solve_frequencies of one batch with host output buffers"}
        # CPU baseline: the reference algorithm (FP32 restatement) on the host cores, bounded sample
        if args.cpu_baseline > 0:
            threads = os.cpu_count() or 1
            from oracle.build import build_oracle

            build_oracle()
            ts = [cpu_oracle_step(mesh, points, freqs[32 + i], drive, threads) for i in range(args.cpu_baseline)]
            result["cpu_baseline"] = {
                "value": len(ts) / sum(ts), "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"{len(ts)} frequency of the same workload: FP32 restatement of BEAT CPU assembly "
                          "(colored OpenMP), BM system, LAPACK cgetrf/cgetrs, field",
            }
        # serving stream: seeded Poisson arrivals of mixed-size jobs, latency per job
        if args.serving_jobs > 0:
            result["serving"] = serving_run(args, local_rank)
    # gpu_launches: our kernels per timed step.  Per batch of B frequencies with
    # P = ceil(n/64) panels and R refinement steps: 6 assembly kernels per
    # frequency; LU 6P - 4 (panel, swap, trsm, operand split x2, tcgen05 update)
    # or 3P - 1 with the cuBLAS update; permutation, FP64 copy, 5 (R + 1) solve /
    # residual kernels, 2 field kernels.
    nv = mesh.n_vertices
    panels = (nv + 63) // 64
    refine = result["refine_steps_max"]
    lu = 6 * panels - 4 if stats_list[0]["lu_gemm_used"] == 2 else 3 * panels - 1
    per_batch = 6 * B + lu + 2 + 5 * (refine + 1) + 2
    result["gpu_launches"] = per_batch * args.steps
    m.release()
    ctx.close()
    if rank == 0:
        print(json.dumps(result))
    if dist:
        dist.destroy_process_group()


def serving_run(args, device: int) -> dict:
    """The serving stream (seeded Poisson arrivals, sizes 1k-15k triangles, 1-32
    frequencies each) replayed twice on the same GPU: with the GB300 scheduler
    (concurrent jobs, smallest-work-first with aging) and one job at a time in
    arrival order, the reference server's per-GPU policy."""
    serving = pkg("serving")
    out = {"stream": f"{args.serving_jobs} jobs, Poisson {args.serving_rate:g}/s (seed 0), sizes uniform over "
                     "{1k, 2k, 5k, 10k, 15k} triangles (box or cube-sphere, seeded piston), 1-32 log-spaced "
                     "freqs in 100 Hz-8 kHz, 2x73 polar + 1000 Fibonacci points; latency = arrival to last "
                     "result, mixed form"}
    for name, running, policy in (("gb300_scheduler", args.serving_running, "sjf"), ("one_job_at_a_time_fifo", 1, "fifo")):
        stream = serving.poisson_jobs(args.serving_jobs, args.serving_rate, seed=0)
        with serving.ServingScheduler(device, max_running=running, policy=policy) as sch:
            jobs = serving.replay(sch, stream, timeout_s=900)
        out[name] = {"max_running": running, "policy": policy, **serving.latency_summary(jobs)}
    return out


if __name__ == "__main__":
    main()
