"""Throughput benchmark of the type-2 NUFFT exec path on GB300.

Workload (one "step" = one execute of the plan):
  2D type 2 on a radial MRI-like trajectory: 1024 x 1024 modes, 512
  golden-angle spokes (theta_k = k * pi * (3 - sqrt 5)) x 2048 samples with
  radius linearly spaced in [-pi, pi) (M = 1,048,576), Fourier coefficients
  iid complex N(0,1), FP32, tol 1e-6, seeded synthetic data.

Metric: nonuniform points per second of execute(), with the relative l2
error against the FP64 oracle (direct sum on random targets) reported beside
it.  `value` times execute() on device-resident inputs with CUDA events on the
plan's stream (L2 flushed with a 256 MB write between steps, outside the
timed events); `e2e` times the same public call with the coefficients copied
from pinned host memory and the result copied back inside each step.

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, FP64, all host cores, scipy FFT) on the same workload.

Multi-GPU: replicas -- each rank runs the workload on its own GPU; no data
moves between ranks; value = sum of points / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_MODES = (1024, 1024)
SPOKES, SAMPLES = 512, 2048
TOL = 1e-6
METRIC = "NU pts/s exec at rel-l2 err<=tol vs FP64 oracle"
UNIT = "NU pts/s"
WORKLOAD = ("2D type-2 NUFFT, radial trajectory 512 golden-angle spokes x 2048 samples "
            "(M=1048576), 1024x1024 modes, FP32, tol 1e-6, ntransf 1")


def radial_points():
    k = np.arange(SPOKES)
    theta = k * np.pi * (3.0 - math.sqrt(5.0))
    r = np.linspace(-np.pi, np.pi, SAMPLES, endpoint=False)
    x = (r[None, :] * np.cos(theta)[:, None]).ravel()
    y = (r[None, :] * np.sin(theta)[:, None]).ravel()
    return x.astype(np.float32), y.astype(np.float32)


def coefficients(seed=7):
    rng = np.random.default_rng(seed)
    shape = N_MODES[::-1]
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.idx), "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(key: str):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh).get(key)
    return None


# --------------------------------------------------------------------------
def cpu_pipeline_rate(x, y, fk, steps=2, warmup=0):
    """Oracle (FP64 C restatement + scipy FFT, all host cores) on the full
    workload; returns (pts/s, cores, seconds per step)."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    O.set_num_threads(cores)
    plan = O.OraclePlan(2, N_MODES, -1, TOL, True)
    plan.fft_workers = cores
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    fk128 = fk.astype(np.complex128)
    for _ in range(warmup):
        plan.execute(x64, y64, None, data=fk128)
    t0 = time.perf_counter()
    for _ in range(steps):
        plan.execute(x64, y64, None, data=fk128)
    dt = (time.perf_counter() - t0) / steps
    return x.size / dt, cores, dt


def accuracy(x, y, fk, c_gpu, ntargets=512, seed=3):
    from oracle import oracle as O
    O.set_num_threads(os.cpu_count() or 1)
    idx = np.random.default_rng(seed).choice(x.size, size=ntargets, replace=False)
    ref = O.direct_type2(x.astype(np.float64), y.astype(np.float64), None,
                         fk.astype(np.complex128).ravel(), N_MODES, -1, idx)
    est = c_gpu.ravel()[idx].astype(np.complex128)
    return float(np.linalg.norm(est - ref) / np.linalg.norm(ref)), ntargets


# --------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    x, y = radial_points()
    fk = coefficients()
    rate_steps = []
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    O.set_num_threads(cores)
    plan = O.OraclePlan(2, N_MODES, -1, TOL, True)
    plan.fft_workers = cores
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    fk128 = fk.astype(np.complex128)
    for _ in range(args.warmup):
        plan.execute(x64, y64, None, data=fk128)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        plan.execute(x64, y64, None, data=fk128)
        rate_steps.append(time.perf_counter() - t1)
    total = time.perf_counter() - t0
    value = x.size * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded radial trajectory, CN(0,1) coefficients)",
        "config": {"workload": WORKLOAD, "global_batch": 1, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "full workload per step (FP64 oracle restatement of the "
                                   "reference's type-2 path: amplify, scipy FFT, interp)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    from cufinufft_gb300 import cufinufft
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
    x, y = radial_points()
    fk = coefficients()
    M = x.size
    stream = torch.cuda.Stream(device=dev)
    # the library's 2D x axis is the fastest mode axis; the Python interface
    # takes C-ordered axes (kx = slow, ky = fast)
    plan = cufinufft(2, N_MODES[::-1], eps=TOL, dtype=np.float32, isign=-1)
    plan.set_stream(stream)
    xg = torch.from_numpy(x).to(dev)
    yg = torch.from_numpy(y).to(dev)
    fk_dev = torch.from_numpy(fk).to(dev)
    c_dev = torch.zeros(M, dtype=torch.complex64, device=dev)
    with torch.cuda.stream(stream):
        plan.set_pts(yg, xg)
        plan.execute(c_dev, fk_dev)
    torch.cuda.synchronize()
    info = plan.info()
    c_first = c_dev.cpu().numpy()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    # warm-up
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            plan.execute(c_dev, fk_dev)
    torch.cuda.synchronize()

    # ---- timed: device-resident inputs
    plan.set_timing(True)
    plan.stage_times(reset=True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler(local_rank)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            plan.execute(c_dev, fk_dev)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    stages = plan.stage_times(reset=True)
    plan.set_timing(False)

    # ---- e2e: host buffers, copies inside each step
    fk_host = torch.from_numpy(fk.ravel().copy()).pin_memory()
    c_host = torch.empty(M, dtype=torch.complex64).pin_memory()
    fk_stage = torch.empty_like(fk_dev)
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            fk_stage.view(-1).copy_(fk_host, non_blocking=True)
            plan.execute(c_dev, fk_stage)
            c_host.copy_(c_dev, non_blocking=True)
    torch.cuda.synchronize()
    barrier()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            ev2[i][0].record(stream)
            fk_stage.view(-1).copy_(fk_host, non_blocking=True)
            plan.execute(c_dev, fk_stage)
            c_host.copy_(c_dev, non_blocking=True)
            ev2[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = sum(a.elapsed_time(b) for a, b in ev2)
    assert np.allclose(c_host.numpy(), c_first, rtol=0, atol=1e-3 * np.abs(c_first).max())

    # max over ranks
    times = torch.tensor([dev_ms, e2e_ms], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    dev_ms, e2e_ms = float(times[0]), float(times[1])
    if rank != 0:
        return

    value = world * M * args.steps / (dev_ms / 1e3)
    e2e_value = world * M * args.steps / (e2e_ms / 1e3)
    err, ntg = accuracy(x, y, fk, c_first)

    # roofline of the dominant kernel of ours: the interp kernel
    interp_ms = stages["spreadinterp"] / max(stages["batches"], 1)
    nf1, nf2 = info["nf1"], info["nf2"]
    grid_bytes = nf1 * nf2 * 8           # grid read once (complex64)
    point_bytes = M * (2 * (4 + 4) + 4)  # per point: (first tap int32 + offset f32) x 2 axes + index
    out_bytes = M * 8                    # c written (complex64)
    alg = grid_bytes + point_bytes + out_bytes
    achieved = alg / (interp_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic("interp_gm_2d_f32_radial")
    roof = {"kernel": "k_interp_gm<float,2,7>", "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "algorithmic_bytes": alg, "kernel_ms": interp_ms, "peak_source": peak_kind,
            "stage_ms": {k: v / max(stages["batches"], 1) for k, v in stages.items()
                         if k != "batches"}}

    cpu = None
    if world == 1 and not args.no_cpu:
        rate, cores, dt = cpu_pipeline_rate(x, y, fk, steps=2, warmup=1)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"full workload, 2 executes after 1 warm-up ({dt:.2f} s each), FP64 "
                         "oracle restatement of the reference's type-2 path, scipy FFT"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded radial trajectory, CN(0,1) coefficients)",
        "config": {"workload": WORKLOAD, "global_batch": world, "seq_len": None,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed between steps (256 MB write, outside the timed events)",
                   "method": info["method"], "ns": info["ns"], "nf": [nf1, nf2]},
        "rel_l2_err": err, "rel_l2_targets": ntg, "tol": TOL,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": fk.nbytes,
                "d2h_bytes_per_step": M * 8},
        "gpu_launches": 2 * args.steps,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
