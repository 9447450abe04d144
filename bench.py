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
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "frequency solves/s @10k tris (mixed vs FP64, ≤1e-5 err); p50/p99 latency"
UNIT = "frequency-solves/s"
SOUND_SPEED = 343.0
RHO = 1.205
# regular_f32_kernel DRAM bytes per frequency on box10k (ncu, profiles/regular_f32_kernel_box10k.md)
REGULAR_DRAM_BYTES_PER_FREQ = 1.3964e9  # (152.0 MB read + 5,433.6 MB written) / 4 frequencies


def pkg(name: str):
    return importlib.import_module("boundary-lab_gb300." + name)


# The synthetic workloads of the benchmark, by name: mesh, observation points,
# frequencies, form.  "box10k" is the headline configuration (mixed form).
WORKLOADS = {
    "sphere1280": dict(mesh="sphere1280", f=(100.0, 3000.0, 16), polar=False, n_far=1000, form="fp64",
                       text="rigid sphere r=0.1 m, icosphere {nf} triangles ({nv} dofs), unit-velocity cap (polar "
                            "angle < 30 deg, {nr} faces); 16 log-spaced freqs 100 Hz-3 kHz; FP64 form; 1000 "
                            "Fibonacci points at 2 m"),
    "box5k": dict(mesh="box5k", f=(50.0, 10000.0, 200), polar=False, n_far=2000, form="mixed",
                  text="closed box 0.3x0.2x0.25 m, {nf} triangles ({nv} dofs), circular piston r=5 cm on +z ({nr} "
                       "faces); 200 log-spaced freqs 50 Hz-10 kHz; 2000 Fibonacci points at 2 m"),
    "box10k": dict(mesh="box10k", f=(200.0, 12000.0, 64), polar=True, n_far=2000, form="mixed",
                   text="closed box 0.3x0.2x0.25 m, {nf} triangles ({nv} P1 dofs), circular piston r=5 cm on +z "
                        "({nr} faces); 64 log-spaced freqs 200 Hz-12 kHz; {npt} observation points (2x73 polar + "
                        "2000 Fibonacci at 2 m)"),
    "box1k": dict(mesh="box1k", f=(100.0, 8000.0, 16), polar=True, n_far=1000, form="mixed",
                  text="closed box 0.3x0.2x0.25 m, {nf} triangles ({nv} dofs), circular piston r=5 cm on +z ({nr} "
                       "faces); 16 log-spaced freqs 100 Hz-8 kHz; {npt} observation points (2x73 polar + 1000 "
                       "Fibonacci at 2 m): the small jobs of the serving stream"),
    "box2k": dict(mesh="box2k", f=(100.0, 8000.0, 16), polar=True, n_far=1000, form="mixed",
                  text="closed box 0.3x0.2x0.25 m, {nf} triangles ({nv} dofs), circular piston r=5 cm on +z ({nr} "
                       "faces); 16 log-spaced freqs 100 Hz-8 kHz; {npt} observation points (2x73 polar + 1000 "
                       "Fibonacci at 2 m): the small jobs of the serving stream"),
    "horn20k": dict(mesh="horn20k", f=(500.0, 16000.0, 32), polar=False, n_far=5000, form="mixed",
                    text="exponential horn (throat r=2.5 cm, mouth r=15 cm, length 20 cm) in a 0.5x0.4x0.4 m box, "
                         "{nf} triangles ({nv} dofs), driven throat disc ({nr} faces); 32 log-spaced freqs "
                         "500 Hz-16 kHz; 5000 Fibonacci points at 2 m"),
}


def workload(name: str = "box10k", faces: int | None = None):
    """(mesh, points, freqs, drive, spec) of a named workload; ``faces`` re-meshes the box."""
    meshes = pkg("meshes")
    request = pkg("request")
    spec = WORKLOADS[name]
    if faces is not None and name.startswith("box"):
        mesh = meshes.box_with_piston((0.3, 0.2, 0.25), faces, 0.05, "+z")
    elif name in ("box1k", "box2k"):
        mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 1000 if name == "box1k" else 2000, 0.05, "+z")
    else:
        mesh = meshes.config_mesh(spec["mesh"])
    parts = []
    if spec["polar"]:
        _, horizontal, vertical, _ = request.polar_observation_points({"step_size": 5.0, "distance": 2.0})
        parts += [horizontal, vertical]
    parts.append(request.fibonacci_sphere(spec["n_far"], 2.0))
    points = np.vstack(parts)
    lo, hi, n = spec["f"]
    freqs = np.logspace(np.log10(lo), np.log10(hi), n)
    drive = (mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :]
    return mesh, points, freqs, drive, spec


def describe(mesh, points, spec) -> str:
    return spec["text"].format(nf=mesh.n_faces, nv=mesh.n_vertices, nr=int((mesh.tags == 2).sum()), npt=len(points))


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self._first = threading.Event()
        self._reader = None

    def _read(self) -> None:
        for ln in self.proc.stdout:
            if ln.strip():
                self.lines.append(ln)
                self._first.set()
        self._first.set()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        self._reader = threading.Thread(target=self._read, daemon=True)
        self._reader.start()
        # nvidia-smi's first start on a box initialises NVML, which stalls this
        # process's CUDA calls for a few hundred ms: start timing after its first sample
        self._first.wait(timeout=15)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            if self._reader is not None:
                self._reader.join(timeout=5)
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


def cpu_oracle_step(mesh, points, freq, drive, threads: int, precision: str = "f32", regular_order: int = 4):
    """One frequency of the reference algorithm on the host (assembly, BM system, LU,
    field): FP32 as the reference's engine computes, or FP64.  Returns (seconds, solution)."""
    from oracle import oracle

    t0 = time.perf_counter()
    omega = 2 * np.pi * freq
    q = drive[0] * (1j * RHO * omega)
    if precision == "f32":
        q = q.astype(np.complex64)
    sol = oracle.solve_frequency(mesh, omega / SOUND_SPEED, q, points, precision=precision, threads=threads,
                                 regular_order=regular_order)
    return time.perf_counter() - t0, sol


def workload_config(args, mesh, points, spec, world: int) -> dict:
    """The ``config`` object both arms print (identical, so the two lines name the same run)."""
    return {"workload": describe(mesh, points, spec), "name": args.workload, "form": spec["form"],
            "l2": "GPU arm: a 256 MiB buffer is written before every timed step (> 129 MB L2); "
                  "host arm: inputs in host memory",
            "parallelism": f"frequencies sharded over {world} rank(s), no collective on the data path"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    mesh, points, freqs, drive, spec = workload(args.workload, args.faces)
    if args.form:
        spec = {**spec, "form": args.form}
    threads = os.cpu_count() or 1
    cpu_prec = "f64" if spec["form"] == "fp64" else "f32"
    from oracle.build import build_oracle

    build_oracle()
    # Warm-up steps: one small solve each (page-in of the library and of OpenBLAS).
    # Timed steps: exactly --steps full-size frequencies of the workload's sweep.
    small_mesh, small_points, _, small_drive, _ = workload("box10k", 600)
    for _ in range(args.warmup):
        cpu_oracle_step(small_mesh, small_points[:64], 500.0, small_drive, threads)
    sel = [freqs[(i * 13) % len(freqs)] for i in range(args.steps)]
    t0 = time.perf_counter()
    times = [cpu_oracle_step(mesh, points, f, drive, threads, cpu_prec)[0] for f in sel]
    total = time.perf_counter() - t0
    value = len(times) / total
    sample = (f"1 full-size frequency of the workload per step ({len(times)} steps): {cpu_prec.upper()} restatement "
              "of BEAT CPU assembly (colored OpenMP), BM system, LAPACK getrf/getrs (scipy OpenBLAS), field")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if cpu_prec == "f64" else "f32",
        "data": "synthetic",
        "config": workload_config(args, mesh, points, spec, world),
        "step": "1 frequency of the sweep on the host cores; warm-up: one small solve per warm-up step",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def launch_ranks(args) -> int:
    """``--gpus N`` started without a launcher: start N ranks with torch.distributed.run
    (one process per GPU, 127.0.0.1 rendezvous) running this script with the same
    arguments, and return their exit status.  Rank 0 prints the JSON line."""
    import socket

    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", str(args.gpus),
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def run_plan(args) -> None:
    """``--plan``: each rank reports the frequency batches it would solve (no GPU work);
    rank 0 gathers them over gloo and prints one JSON line.  Shows the sharding that the
    timed run uses: rank r takes batch (step x world + r) of the sweep."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    spec = WORKLOADS[args.workload]
    lo, hi, n = spec["f"]
    freqs = np.logspace(np.log10(lo), np.log10(hi), n)
    B = min(args.batch or 15, len(freqs))
    lanes = args.lanes if 2 * B <= len(freqs) else 1
    sharding = pkg("sharding")
    mine = [[int(i) for i in np.arange(len(freqs))[sharding.step_batch(s, rank, world, lanes * B, len(freqs))]]
            for s in range(args.warmup + args.steps)]
    gathered = [mine]
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps({"plan": True, "n_gpus": world, "batch": B, "lanes": lanes, "n_freq": len(freqs),
                          "rank_batches": gathered}))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=0,
                    help="frequencies per step; 0: the library's largest batch (bem_auto_batch: the LU's "
                         "cluster panels resident in one wave)")
    ap.add_argument("--workload", default="box10k", choices=sorted(WORKLOADS),
                    help="synthetic workload (box10k: the headline mixed-form configuration)")
    ap.add_argument("--faces", type=int, default=None, help="re-mesh the box workloads to about this many triangles")
    ap.add_argument("--fp64-freqs", type=int, default=0,
                    help="frequencies of the sweep solved in the plain FP64 form for the per-frequency error "
                         "(0: every frequency)")
    ap.add_argument("--cpu-baseline", type=int, default=1, help="frequencies timed on the host for cpu_baseline")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-extras", action="store_true", help="skip FP64 form, e2e and CPU baseline (profiling runs)")
    ap.add_argument("--serving-jobs", type=int, default=40, help="jobs in the seeded Poisson serving stream (0: skip)")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="serving arrivals per second")
    ap.add_argument("--serving-running", type=int, default=4, help="concurrent jobs on the GPU")
    ap.add_argument("--lu-block", type=int, default=0, choices=[0, 32, 64], help="LU panel width (0 automatic)")
    ap.add_argument("--form", default=None, choices=["mixed", "fp64"], help="override the workload's precision form")
    ap.add_argument("--autotune", type=int, default=1, choices=[0, 1],
                    help="time the candidate launch configurations on the workload's sweep before the run "
                         "(autotune.tune) and use the winner's LU panel width and trailing update")
    ap.add_argument("--lanes", type=int, default=2, choices=[1, 2],
                    help="batches per step solved side by side on two streams (bem_solve_options.lanes)")
    ap.add_argument("--lu-gemm", type=int, default=0, choices=[0, 1, 2],
                    help="LU trailing update: 0 automatic, 1 cuBLAS cgemm, 2 tcgen05 3xFP16")
    ap.add_argument("--plan", action="store_true",
                    help="print the frequency batches each rank would solve (no GPU work)")
    args = ap.parse_args()
    if args.warmup < 3 and not args.no_extras:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args))
    if args.plan:
        run_plan(args)
        return
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
    mesh, points, freqs, drive, spec = workload(args.workload, args.faces)
    if args.form:
        spec = {**spec, "form": args.form}
    fp64_workload = spec["form"] == "fp64"
    ctx = native.Context(local_rank)
    m = ctx.upload_mesh(mesh.vertices, mesh.faces)
    m.set_excitation(drive)
    m.set_observation_points(points)
    form = native.BEM_PRECISION_FP64 if fp64_workload else native.BEM_PRECISION_MIXED
    tune_info = None
    if args.autotune and not args.no_extras and args.lu_block == 0 and args.lu_gemm == 0:
        # The tuner scores configurations on the workload's whole sweep (ceil(n_freq / batch)
        # batches); the timed steps keep their one-batch size and take the winner's LU
        # panel width and trailing update.
        try:
            tr = pkg("autotune").tune(m, freqs, precision=form, sound_speed=SOUND_SPEED, rho=RHO, device=local_rank,
                                      use_cache=False)
            args.lu_block, args.lu_gemm = tr.best.lu_block, tr.best.lu_gemm
            tune_info = tr.to_dict()
        except Exception as exc:  # noqa: BLE001 - the run goes on with the library's own choice
            tune_info = {"error": f"{type(exc).__name__}: {exc}"}
    B = min(args.batch if args.batch > 0 else m.auto_batch(0, form), len(freqs))
    lanes = args.lanes if 2 * B <= len(freqs) else 1
    SB = lanes * B  # frequencies per step: one batch per lane
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=f"cuda:{local_rank}")
    p_dev = torch.empty((SB, 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
    u_dev = torch.empty((SB, 1, len(points)), dtype=torch.complex128, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    opts = dict(precision=form, sound_speed=SOUND_SPEED, rho=RHO, batch=B, lanes=lanes, refine_tol=1e-10,
                max_refine=8, lu_gemm=args.lu_gemm, lu_block=args.lu_block)

    sharding = pkg("sharding")

    def step_freqs(step: int):
        # weak scaling: rank r takes batch (step * world + r) of the sweep
        return freqs[sharding.step_batch(step, rank, world, SB, len(freqs))]

    for s in range(args.warmup):
        m.solve_device(step_freqs(s), p_dev.data_ptr(), u_dev.data_ptr(), **opts)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev_start = torch.cuda.Event(enable_timing=True)
    ev_end = torch.cuda.Event(enable_timing=True)
    step_events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    flush.fill_(-1.0)  # first use loads torch's fill kernel (hundreds of ms on a fresh box): not in the timed region
    torch.cuda.synchronize()
    stats_list = []
    host_ms = []
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev_start.record(stream)
            for s in range(args.steps):
                h0 = time.perf_counter()
                flush.fill_(float(s))  # write 256 MiB (> 129 MB L2) between steps
                step_events[s][0].record(stream)
                h1 = time.perf_counter()
                stats_list.append(m.solve_device(step_freqs(args.warmup + s), p_dev.data_ptr(), u_dev.data_ptr(),
                                                 profile=1, **opts))
                h2 = time.perf_counter()
                step_events[s][1].record(stream)
                host_ms.append((1e3 * (h1 - h0), 1e3 * (h2 - h1)))
            ev_end.record(stream)
        torch.cuda.synchronize()
    elapsed = ev_start.elapsed_time(ev_end) / 1e3
    if dist:
        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    solved = args.steps * SB * world
    value = solved / elapsed
    step_ms = [a.elapsed_time(b) for a, b in step_events]
    kernel_s = {k: sum(st["kernel_s"][k] for st in stats_list) for k in stats_list[0]["kernel_s"]}
    # per-lane stage intervals of the timed region, summed over the lanes: with two lanes
    # the stages of one overlap the other's, so each interval includes the other lane's work
    lane_sum_ms = {k: 1e3 * v / (args.steps * SB) for k, v in kernel_s.items()}
    # stage breakdown of one step's frequencies on one lane, after the timed region (nothing
    # overlaps it; a call of the timed calls' size takes the same kernels, e.g. the singular
    # remainder through the Chebyshev moments in calls of at least 12 frequencies)
    st1 = m.solve_device(step_freqs(0), p_dev.data_ptr(), u_dev.data_ptr(), profile=1, **{**opts, "lanes": 1})
    torch.cuda.synchronize()
    nb1 = len(step_freqs(0))
    per_freq_ms = {k: 1e3 * v / nb1 for k, v in st1["kernel_s"].items()}

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
        "dtype": "f64" if fp64_workload else "f32 (compensated) + f64 refinement",
        "data": "synthetic",
        "config": workload_config(args, mesh, points, spec, world),
        "step": (f"{lanes} batches of {B} frequencies of the sweep per rank, side by side on two streams"
                 if lanes > 1 else f"one batch of {B} frequencies of the sweep per rank"),
        "clocks": clocks.summary(),
        "launch": {"batch": B, "lanes": lanes, "lu_block": args.lu_block, "lu_gemm": args.lu_gemm},
        "autotune": tune_info,
        "stage_ms_per_freq": per_freq_ms,  # one step's frequencies on one lane, after the timed region
        "stage_ms_per_freq_lane_sums": lane_sum_ms if lanes > 1 else None,
        "step_ms": step_ms,
        # timed region minus the steps: the L2 flushes and host time between steps
        "between_steps_ms": 1e3 * elapsed - sum(step_ms),
        "host_ms": [[round(a, 3), round(b, 3)] for a, b in host_ms],  # (flush + event, solve call) per step
        "refine_steps_max": max(st["max_refine_steps"] for st in stats_list),
        "lu_trailing_update": {1: "cublas cgemm", 2: "tcgen05 3xFP16"}.get(stats_list[0]["lu_gemm_used"]),
        "rel_residual_max": max(st["max_rel_residual"] for st in stats_list),
    }

    # dominant kernel roofline: regular-pair assembly, FP32 pipe (mixed form)
    st0 = stats_list[0]
    regular_qpairs = st0["regular_pairs"] * 36
    # FP32 flop the regular kernel executed (FMA = 2), counted by the library from the
    # kernel's source for the launch widths it used: per q-pair and frequency
    # 35.67 + 26.83 / w, w = frequencies sharing one launch's geometry (4 at this size:
    # 42.4 flop; 49.1 with pairs of frequencies)
    reg_flop = sum(st["regular_flop"] for st in stats_list)
    flops_per_qpair = reg_flop / (regular_qpairs * args.steps * SB) if regular_qpairs else 0.0
    reg_s = kernel_s["regular"] / (args.steps * SB)  # seconds per frequency
    achieved = reg_flop / kernel_s["regular"] / 1e12 if kernel_s["regular"] > 0 else None
    clock = result["clocks"]["sm_mhz"] or 1920.0
    n_sm = torch.cuda.get_device_properties(local_rank).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * clock * 1e6 / 1e12
    result["roofline"] = {
        "kernel": "regular_f32_kernel (regular face-pair assembly)",
        "bound": "fp32",
        "achieved": achieved,
        "peak": fp32_peak,
        "unit": "TFLOP/s",
        "frac": (achieved / fp32_peak) if achieved else None,
        # DRAM bytes per frequency from one ncu capture of this kernel at this workload
        # (dram__bytes_read.sum + dram__bytes_write.sum, current source); the algorithmic
        # bytes are the extended-row output, 3 x N_f x ldR x 8 B = 1.360e9 per frequency
        "traffic": REGULAR_DRAM_BYTES_PER_FREQ if args.workload == "box10k" and args.faces in (None, 10000) else None,
        "peak_source": f"{n_sm} SMs (device query) x 128 FP32 lanes x 2 flop x median SM clock sampled during the run "
                       "(MEASURED_PEAKS.json has no FP32 figure)",
        "work_per_frequency": f"{regular_qpairs:.4g} q-pairs x {flops_per_qpair:.2f} flop",
        "ms_per_frequency": 1e3 * reg_s,
        "timing": ("CUDA events around each regular launch on its lane's stream over the timed region; with "
                   "two lanes the launches share the GPU with the other lane's kernels" if lanes > 1 else
                   "CUDA events around each regular launch over the timed region"),
        # the same kernel on one lane with nothing beside it (one batch after the timed region)
        "one_lane": ({"achieved": st1["regular_flop"] / st1["kernel_s"]["regular"] / 1e12,
                      "frac": st1["regular_flop"] / st1["kernel_s"]["regular"] / 1e12 / fp32_peak,
                      "ms_per_frequency": 1e3 * st1["kernel_s"]["regular"] / nb1}
                     if st1["kernel_s"]["regular"] > 0 else None),
        # the same time against the reference's own arithmetic per q-pair (about 160 flop:
        # S, D, K' and H integrands formed separately, BeatEngineCpuAssembly.jl:316-346),
        # context only: this kernel folds them and shares the geometry across frequencies
        "reference_flop_equivalent_frac": (regular_qpairs * 160 / reg_s / 1e12 / fp32_peak) if reg_s > 0 else None,
    }

    if fp64_workload:
        result["roofline"] = None
        result["roofline_note"] = "FP64 workload: the regular assembly runs regular_f64_kernel on the FP64 pipe"

    if not args.no_extras and rank == 0 and fp64_workload:
        # the FP64 GPU form against the FP64 CPU oracle on one frequency
        from oracle.build import build_oracle

        build_oracle()
        f_chk = freqs[len(freqs) // 2]
        p_g, u_g, _ = m.solve(np.array([f_chk]), **{**opts, "batch": 1})
        _, ref = cpu_oracle_step(mesh, points, f_chk, drive, os.cpu_count() or 1, "f64")
        result["max_rel_far_field_err_vs_cpu_fp64"] = float(
            np.linalg.norm(u_g[0, 0] - ref.field[:, 0]) / np.linalg.norm(ref.field[:, 0]))
        result["max_rel_surface_pressure_err_vs_cpu_fp64"] = float(
            np.linalg.norm(p_g[0, 0] - ref.pressure[:, 0]) / np.linalg.norm(ref.pressure[:, 0]))
    if not args.no_extras and rank == 0 and not fp64_workload:
        result.update(accuracy_sweep(m, freqs, mesh, points, opts, args, stream, value / world))

    if not args.no_extras and rank == 0:
        # end to end through the C ABI with host buffers: upload mesh + caches, solve a batch, copy results back
        e2e_times = []
        h2d = mesh.vertices.nbytes + mesh.faces.astype(np.int32).nbytes + drive.nbytes + points.nbytes + SB * 8
        d2h = SB * (mesh.n_vertices + len(points)) * 16
        for s in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m2 = ctx.upload_mesh(mesh.vertices, mesh.faces)
            m2.set_excitation(drive)
            m2.set_observation_points(points)
            m2.solve(step_freqs(s), **opts)
            m2.release()
            e2e_times.append(time.perf_counter() - t0)
        result["e2e"] = {"value": SB / statistics.median(e2e_times), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                         "d2h_bytes_per_step": int(d2h),
                         "what": "per step: bem_upload_mesh (plan + singular moments) + excitation + points from "
                                 "host arrays, bem_solve_frequencies of the step's frequencies (one batch per lane) "
                                 "with host output buffers"}
        # CPU baseline: the reference algorithm (FP32 restatement) on the host cores, bounded sample
        if args.cpu_baseline > 0:
            threads = os.cpu_count() or 1
            from oracle.build import build_oracle

            build_oracle()
            cpu_prec = "f64" if fp64_workload else "f32"
            ts = [cpu_oracle_step(mesh, points, freqs[(len(freqs) // 2 + i) % len(freqs)], drive, threads,
                                  cpu_prec)[0] for i in range(args.cpu_baseline)]
            result["cpu_baseline"] = {
                "value": len(ts) / sum(ts), "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"{len(ts)} frequency of the same workload: {cpu_prec.upper()} restatement of BEAT CPU "
                          "assembly (colored OpenMP), BM system, LAPACK getrf/getrs, field",
            }
            # the reference CPU backend's own default rule: wavelength-driven regular order
            # (kh = k sqrt(p90 face area): order 1 up to kh 0, order 2 up to kh 2, else 4)
            se = pkg("system_exterior")
            f_w = freqs[len(freqs) // 2]
            sel = se.exterior_quadrature_selection({}, mesh, float(f_w), SOUND_SPEED, 4, "cpu")
            tw = cpu_oracle_step(mesh, points, f_w, drive, threads, cpu_prec, regular_order=sel.order)[0]
            result["cpu_baseline_wavelength_rule"] = {
                "value": 1.0 / tw, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"1 frequency ({f_w:.0f} Hz) with the reference CPU default regular rule "
                          f"(wavelength mode, order {sel.order}; the GPU path and cpu_baseline use the fixed "
                          "order-4 rule of the CUDA backend)",
            }
        # serving stream: seeded Poisson arrivals of mixed-size jobs, latency per job
        if args.serving_jobs > 0 and args.workload == "box10k":
            result["serving"] = serving_run(args, local_rank)
            result["small_jobs"] = small_jobs_run(local_rank)
        # retained-trace field (the bem_field operation): one request per call, host traces
        if args.workload == "box10k":
            result["retained_field"] = retained_field_run(mesh, local_rank)
    # gpu_launches: this library's kernels launched in the timed region, counted by
    # the library itself per call (bem_solve_stats.kernel_launches)
    result["gpu_launches"] = int(sum(st["kernel_launches"] for st in stats_list))
    m.release()
    ctx.close()
    if rank == 0:
        print(json.dumps(result))
    if dist:
        dist.destroy_process_group()


def accuracy_sweep(m, freqs, mesh, points, opts, args, stream, mixed_rate: float) -> dict:
    """The plain FP64 GPU form on the sweep's frequencies (every one by default) and the
    mixed form's relative error against it, per frequency: far field and surface
    pressure.  The mixed form is solved twice: in one call over all the frequencies with
    the timed steps' options (batch, lanes: the production path, e.g. the singular
    remainder through the Chebyshev moments), whose errors are the record, and one
    frequency per call (the point-by-point singular kernel), which also gives the
    refinement steps and final relative residual of each frequency.  The FP64 form runs
    in batches of at most 16 and is timed with CUDA events on the library's stream."""
    import torch

    native = pkg("native")
    n_f = len(freqs)
    n_sel = n_f if args.fp64_freqs <= 0 else min(args.fp64_freqs, n_f)
    sel = freqs[np.unique(np.linspace(0, n_f - 1, n_sel).round().astype(int))]
    chunk = min(16, len(sel))
    p64 = torch.empty((len(sel), 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
    u64 = torch.empty((len(sel), 1, len(points)), dtype=torch.complex128, device="cuda")
    fp64 = dict(precision=native.BEM_PRECISION_FP64, sound_speed=SOUND_SPEED, rho=RHO)
    # warm-up: the FP64 form's first call loads its kernels (cuBLAS zgemm, FP64 kernels) lazily
    m.solve_device(sel[:1], p64.data_ptr(), u64.data_ptr(), batch=1, **fp64)
    torch.cuda.synchronize()
    ev_a, ev_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kernel_s: dict = {}
    with torch.cuda.stream(stream):
        ev_a.record(stream)
        for i in range(0, len(sel), chunk):
            st = m.solve_device(sel[i:i + chunk], p64[i].data_ptr(), u64[i].data_ptr(), batch=min(chunk, len(sel) - i),
                                profile=1, **fp64)
            for k, v in st["kernel_s"].items():
                kernel_s[k] = kernel_s.get(k, 0.0) + v
        ev_b.record(stream)
    torch.cuda.synchronize()
    t64 = ev_a.elapsed_time(ev_b) / 1e3
    pw = torch.empty((len(sel), 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
    uw = torch.empty((len(sel), 1, len(points)), dtype=torch.complex128, device="cuda")
    stw = m.solve_device(sel, pw.data_ptr(), uw.data_ptr(), **opts)
    torch.cuda.synchronize()
    errs = [float(torch.linalg.norm(uw[i] - u64[i]) / torch.linalg.norm(u64[i])) for i in range(len(sel))]
    perr = [float(torch.linalg.norm(pw[i] - p64[i]) / torch.linalg.norm(p64[i])) for i in range(len(sel))]
    pm = torch.empty((1, 1, mesh.n_vertices), dtype=torch.complex128, device="cuda")
    um = torch.empty((1, 1, len(points)), dtype=torch.complex128, device="cuda")
    errs1, perr1, steps, resid = [], [], [], []
    for i, f in enumerate(sel):
        st = m.solve_device([f], pm.data_ptr(), um.data_ptr(), **{**opts, "batch": 1})
        torch.cuda.synchronize()
        errs1.append(float(torch.linalg.norm(um[0] - u64[i]) / torch.linalg.norm(u64[i])))
        perr1.append(float(torch.linalg.norm(pm[0] - p64[i]) / torch.linalg.norm(p64[i])))
        steps.append(int(st["max_refine_steps"]))
        resid.append(float(st["max_rel_residual"]))
    v64 = len(sel) / t64
    return {
        "fp64_form": {"value": v64, "unit": UNIT, "freqs_hz": [float(f) for f in sel],
                      "stage_ms_per_freq": {k: 1e3 * v / len(sel) for k, v in kernel_s.items()},
                      "far_field_err_per_freq": errs, "surface_pressure_err_per_freq": perr,
                      "sweep_call": {"refine_steps_max": int(stw["max_refine_steps"]),
                                     "rel_residual_max": float(stw["max_rel_residual"]),
                                     "singular_cheb_freqs": int(stw["singular_cheb_freqs"])},
                      "far_field_err_per_freq_single_calls": errs1,
                      "surface_pressure_err_per_freq_single_calls": perr1,
                      "mixed_refine_steps_per_freq": steps, "mixed_rel_residual_per_freq": resid},
        "speedup_vs_fp64": mixed_rate / v64,
        "max_rel_far_field_err_vs_fp64": max(errs),
        "max_rel_surface_pressure_err_vs_fp64": max(perr),
    }


def retained_field_run(mesh, device: int, n_points: int = 5000, calls: int = 8) -> dict:
    """The exterior field of retained boundary traces (coupled_field.evaluate_bem_field,
    the reference's bem_field operation) on this mesh: 5,000 Fibonacci points at 2 m,
    seeded complex64 traces, 2,500 Hz; the first call uploads the domain (excluded)."""
    cf = pkg("coupled_field")
    rng = np.random.default_rng(11)
    p = (rng.normal(size=mesh.n_vertices) + 1j * rng.normal(size=mesh.n_vertices)).astype(np.complex64)
    q = (rng.normal(size=mesh.n_faces) + 1j * rng.normal(size=mesh.n_faces)).astype(np.complex64)
    i = np.arange(n_points)
    z = 1.0 - (2.0 * i + 1.0) / n_points
    phi = i * np.pi * (3.0 - np.sqrt(5.0))
    rr = np.sqrt(1.0 - z * z)
    pts = 2.0 * np.stack([rr * np.cos(phi), rr * np.sin(phi), z], axis=1)
    ev = cf.FieldEvaluator(device)
    req = cf.BemFieldEvaluationRequest("bench", pts, mesh.vertices, mesh.faces, p, q, 2500.0, SOUND_SPEED)
    try:
        cf.evaluate_bem_field(req, evaluator=ev)  # domain upload + warm-up
        t0 = time.perf_counter()
        for _ in range(calls):
            cf.evaluate_bem_field(req, evaluator=ev)
        dt = (time.perf_counter() - t0) / calls
    finally:
        ev.release()
    pairs = n_points * mesh.n_faces * 3  # (point, source) Green evaluations, 3-point rule
    return {"what": "coupled_field.evaluate_bem_field per request (host traces in, host field out, "
                    "C ABI bem_evaluate_field), 3-point rule, mixed form, 2,500 Hz, 5,000 points at 2 m",
            "ms_per_request": dt * 1e3, "points": n_points, "faces": int(mesh.n_faces),
            "green_evaluations_per_s": pairs / dt}


def small_jobs_run(device: int, n_jobs: int = 24, n_freq: int = 8) -> dict:
    """Small jobs submitted at once (seeded boxes and cube-spheres of 900-1,200 triangles,
    8 log-spaced frequencies 300 Hz - 6 kHz each), run three ways on one GPU: one job at a
    time, four jobs at a time on their own streams, and four workers whose small jobs of
    similar size share launches (bem_solve_jobs).  Frequency solves/s from first submit
    to last result, mixed form."""
    serving = pkg("serving")
    meshes = pkg("meshes")
    request = pkg("request")
    _, horizontal, vertical, _ = request.polar_observation_points({"step_size": 5.0, "distance": 2.0})
    points = np.concatenate([horizontal, vertical, request.fibonacci_sphere(500, 2.0)])
    rng = np.random.default_rng(5)
    specs = [(meshes.seeded_piston_mesh(int(rng.integers(900, 1200)), int(rng.integers(1 << 30))),
              np.geomspace(300.0, 6000.0, n_freq)) for _ in range(n_jobs)]

    def jobs():
        return [serving.ServingJob(vertices=m.vertices, faces=m.faces,
                                   drive=(m.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :],
                                   points=points, freqs_hz=f, chunk=n_freq, job_id=f"small-{i}")
                for i, (m, f) in enumerate(specs)]

    out = {"what": f"{n_jobs} jobs of 900-1,200 triangles x {n_freq} freqs (300 Hz - 6 kHz) submitted at once, "
                   "2x73 polar + 500 Fibonacci points, mixed form; frequency solves/s from first submit to last result"}
    for name, running, group in (("one_at_a_time", 1, 0), ("four_streams", 4, 0), ("shared_launches", 4, 3000)):
        with serving.ServingScheduler(device, max_running=running, policy="fifo", group_faces=group) as sch:
            warm = sch.submit(jobs()[0])  # page in kernels of this worker set
            sch.drain(300)
            t0 = time.perf_counter()
            js = [sch.submit(j) for j in jobs()]
            sch.drain(600)
            wall = time.perf_counter() - t0
        done = [j for j in js if j.status == "completed"]
        out[name] = {"max_running": running, "frequency_solves_per_s": len(done) * n_freq / wall, "wall_s": wall,
                     "jobs_in_shared_launches": sum(j.group_size > 1 for j in done),
                     "failed": [j.error for j in js if j.status != "completed"][:2], "warm_status": warm.status}
    return out


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
