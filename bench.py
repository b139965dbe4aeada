"""Throughput benchmark of the NUFFT exec path on GB300.

Default workload (one "step" = one execute() of the plan):
  2D type 2 on a radial MRI-like trajectory: 1024 x 1024 modes, 512
  golden-angle spokes (theta_k = k * pi * (3 - sqrt 5)) x 2048 samples with
  radius linearly spaced in [-pi, pi) (M = 1,048,576), Fourier coefficients
  iid complex N(0,1), FP32, tol 1e-6, seeded synthetic data.
Other workloads (--workload): radial2d-f64 (the same at FP64, tol 1e-12),
uniform2d (2D type 1, 256^2 modes, M = 1e5 uniform points, FP32, tol 1e-5),
cluster3d (3D type 1, 128^3 modes, M = 3.2e7, half uniform and half in 8
Gaussian clusters of sigma 0.05, FP32, tol 1e-6) and cluster3d-f64 (3D type 2
on the same points, FP64, tol 1e-9).

Metric: nonuniform points per second of execute() at relative l2 error <= tol
against FP64 direct sums on random modes/targets (the error is reported
beside it).  Plans use the library's tolerance-meeting kernel width
(--width-rule tol, the default): the reference's own width rule
ns = ceil(-log10(tol/10)) leaves errors of one to four times tol, so its
throughput is reported beside the headline as `parity_width`, and --width-rule
reference times it instead.  The default run also times, device time only,
the 3D clustered type-1 workload and the uneven 64-plan batch (tuned+batched
against 64 plain plans, and against the same plain plans spreading with the
reference's per-tap shared atomics) under `extra_workloads` (--no-extras
skips them).  `value` times execute() on device-resident inputs with CUDA events
on the plan's stream (L2 flushed with a 256 MB write between steps, outside
the timed events); `e2e` times the same public call with the input copied
from pinned host memory and the output copied back inside each step.

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, in the workload's precision -- FP32 arithmetic for FP32 workloads,
as the reference's FP32 build computes -- all host cores, scipy FFT) on the
same workload.

Multi-GPU: replicas -- each rank runs the workload on its own GPU; no data
moves between ranks; value = sum of points / max time over ranks.
"""
from __future__ import annotations

import argparse
import collections
import ctypes
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

METRIC = "NU pts/s exec at rel-l2 err<=tol vs FP64 oracle"
UNIT = "NU pts/s"


# --------------------------------------------------------------------------
class Workload:
    """A seeded synthetic workload.  ``modes`` is (N1, N2[, N3]) with N1 the
    fastest index (the library's nmodes order); points are returned in the
    library's axis order (x fastest)."""

    def __init__(self, name, ntype, modes, single, tol, desc, ntransf=1, acc_n=512):
        self.name, self.ntype, self.modes = name, ntype, tuple(modes)
        self.dim = len(modes)
        self.single, self.tol, self.desc = single, tol, desc
        self.ntransf = ntransf
        self.acc_n = acc_n
        self.upsampfac = 2.0   # of the timed plan (--upsampfac); the oracle's same-width check follows it
        self._pts = None

    @property
    def rdt(self):
        return np.float32 if self.single else np.float64

    @property
    def cdt(self):
        return np.complex64 if self.single else np.complex128

    def make_points(self):
        raise NotImplementedError

    def points(self):
        if self._pts is None:
            self._pts = [p.astype(self.rdt) for p in self.make_points()]
        return self._pts

    def data(self, seed=7):
        rng = np.random.default_rng(seed)
        if self.ntype == 1:
            M = self.points()[0].size
            shape = (self.ntransf, M)
        else:
            shape = (self.ntransf,) + self.modes[::-1]
        out = np.empty(shape, dtype=self.cdt)
        out.real = rng.standard_normal(shape)
        out.imag = rng.standard_normal(shape)
        return out


class Radial2D(Workload):
    SPOKES, SAMPLES = 512, 2048

    def make_points(self):
        k = np.arange(self.SPOKES)
        theta = k * np.pi * (3.0 - math.sqrt(5.0))
        r = np.linspace(-np.pi, np.pi, self.SAMPLES, endpoint=False)
        x = (r[None, :] * np.cos(theta)[:, None]).ravel()
        y = (r[None, :] * np.sin(theta)[:, None]).ravel()
        return [x, y]


class Uniform(Workload):
    def __init__(self, *a, M=100000, seed=1, **k):
        super().__init__(*a, **k)
        self.M, self.seed = M, seed

    def make_points(self):
        rng = np.random.default_rng(self.seed)
        return [rng.uniform(-np.pi, np.pi, self.M) for _ in range(self.dim)]


class Cluster3D(Workload):
    def __init__(self, *a, M=32_000_000, seed=5, **k):
        super().__init__(*a, **k)
        self.M, self.seed = M, seed

    def make_points(self):
        rng = np.random.default_rng(self.seed)
        half = self.M // 2
        pts = []
        centres = rng.uniform(-np.pi, np.pi, (8, 3))
        which = rng.integers(0, 8, self.M - half)
        for d in range(3):
            u = rng.uniform(-np.pi, np.pi, half).astype(np.float32)
            g = centres[which, d] + 0.05 * rng.standard_normal(self.M - half)
            g = (g + np.pi) % (2 * np.pi) - np.pi           # wrapped into [-pi, pi)
            pts.append(np.concatenate([u, g.astype(np.float32)]))
        return pts


WORKLOADS = {
    "radial2d": lambda: Radial2D(
        "radial2d", 2, (1024, 1024), True, 1e-6,
        "2D type-2 NUFFT, radial trajectory 512 golden-angle spokes x 2048 samples "
        "(M=1048576), 1024x1024 modes, FP32, tol 1e-6, ntransf 1"),
    "radial2d-f64": lambda: Radial2D(
        "radial2d-f64", 2, (1024, 1024), False, 1e-12,
        "2D type-2 NUFFT, radial trajectory 512 golden-angle spokes x 2048 samples "
        "(M=1048576), 1024x1024 modes, FP64, tol 1e-12, ntransf 1", acc_n=256),
    "uniform2d": lambda: Uniform(
        "uniform2d", 1, (256, 256), True, 1e-5,
        "2D type-1 NUFFT, 256x256 modes, M=1e5 iid uniform points, FP32, tol 1e-5, ntransf 1",
        M=100000, acc_n=1000),
    "cluster3d": lambda: Cluster3D(
        "cluster3d", 1, (128, 128, 128), True, 1e-6,
        "3D type-1 NUFFT, 128^3 modes, M=3.2e7 (half uniform, half in 8 Gaussian clusters "
        "sigma 0.05), FP32, tol 1e-6, ntransf 1", acc_n=48),
    "cluster3d-f64": lambda: Cluster3D(
        "cluster3d-f64", 2, (128, 128, 128), False, 1e-9,
        "3D type-2 NUFFT, 128^3 modes, same 3.2e7 clustered points, FP64, tol 1e-9, ntransf 1",
        acc_n=16),
}


# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.samples = []   # (host time, line)
        self.thread = None
        self.first = threading.Event()

    def start(self, wait_s=3.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.idx), "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        self.first.wait(wait_s)

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))
            self.first.set()

    def stop(self, t0: float, t1: float) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.06)  # one more sample after the region
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        inside = [s for s in self.samples if t0 <= s[0] <= t1 + 0.06]
        note = "samples inside the timed region"
        if not inside and self.samples:
            # region shorter than the sampling period: nearest samples
            inside = sorted(self.samples, key=lambda s: abs(s[0] - 0.5 * (t0 + t1)))[:2]
            note = "timed region shorter than the 50 ms sampling period; nearest samples"
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in inside:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[2]))
                smax = max(smax, float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "note": note}


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
def atomic_roofline(taps: int, k_ms: float, single: bool) -> dict:
    """The spread's own ceiling: algorithmic tap updates (M ns^d per
    transform, a complex add each, i.e. two real adds) per second against the
    device's measured shared-memory atomicAdd rate (the library's
    cufinufft_atomic_rate probe, one lane per address).  Dense cells summed in
    registers (cell-run layout) issue fewer atomics than the algorithmic count,
    so `frac` can pass 1 there."""
    from cufinufft_gb300 import _cufinufft as cl
    rates = {}
    for kind, key in ((0, "shared_f32"), (1, "shared_i32"), (2, "global_red_v2_f32"),
                      (3, "shared_u64")):
        r = ctypes.c_double(0.0)
        if cl.atomic_rate(kind, ctypes.byref(r)) != 0:
            raise RuntimeError("cufinufft_atomic_rate failed")
        rates[key] = r.value
    achieved = 2.0 * taps / (k_ms / 1e3)
    peak = rates["shared_f32"] if single else None
    return {"bound": "shared-atomic", "unit": "real adds/s", "achieved": achieved,
            "algorithmic_adds": 2 * taps, "peak": peak,
            "frac": achieved / peak if peak else None,
            "measured_rates": rates,
            "note": "peak = shared FP32 atomicAdd lane-ops/s measured on this device by "
                    "cufinufft_atomic_rate; FP64 plans: no FP32 peak applies"}


def oracle_plan(w: Workload, cores: int, ns=None, timing=False):
    """The oracle's plan for this workload.  timing: the CPU legs (baseline
    and reference arm) run in the workload's own precision -- FP32 arithmetic
    for FP32 workloads, as the reference's FP32 build computes -- while the
    accuracy check stays FP64."""
    from oracle import oracle as O
    O.set_num_threads(cores)
    plan = O.OraclePlan(w.ntype, w.modes, 1 if w.ntype == 1 else -1, w.tol, w.single, ns=ns,
                        upsampfac=w.upsampfac if ns is not None else 2.0,
                        fp32_arith=timing and w.single)
    plan.fft_workers = cores
    return plan


def cpu_step(plan, w: Workload, pts64, data128):
    args = list(pts64) + [None] * (3 - w.dim)
    return plan.execute(*args, data=data128, ntr=w.ntransf)


def cpu_sample(w: Workload, budget_s=20.0):
    """Bounded CPU sample of the workload: full execs while one fits the
    budget, else a subset of the points (spread/interp scale with M)."""
    cores = os.cpu_count() or 1
    plan = oracle_plan(w, cores, timing=True)
    pts = [p.astype(np.float64) for p in w.points()]
    data = w.data().astype(np.complex128)
    M = pts[0].size
    frac = 1.0
    if M > 4_000_000:
        frac = 4_000_000 / M  # sample of the points; the FFT stays full size
        n = int(M * frac)
        pts = [p[:n] for p in pts]
        if w.ntype == 1:
            data = data[:, :n]
    Ms = pts[0].size
    t0 = time.perf_counter()
    cpu_step(plan, w, pts, data)
    dt = time.perf_counter() - t0
    reps = max(1, min(5, int(budget_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        cpu_step(plan, w, pts, data)
    dt = (time.perf_counter() - t0) / reps
    sample = (f"{reps} execs of {'the full workload' if frac == 1.0 else f'{Ms} of {M} points'}"
              f" ({dt:.3f} s each), oracle restatement of the reference's path in "
              f"{'FP32' if w.single else 'FP64'} arithmetic, scipy FFT")
    return Ms * w.ntransf / dt, cores, sample


def accuracy(w: Workload, out_first: np.ndarray, seed=3, oracle_same_width=True, ns=None):
    """rel-l2 error of the first transform against FP64 direct sums on a
    seeded subset of modes/targets, and (oracle_same_width) the oracle's own
    error at kernel width ns on the same subset."""
    from oracle import oracle as O
    O.set_num_threads(os.cpu_count() or 1)
    pts = [p.astype(np.float64) for p in w.points()] + [None] * (3 - w.dim)
    data = w.data()[0].astype(np.complex128)
    rng = np.random.default_rng(seed)
    if w.ntype == 1:
        n = int(np.prod(w.modes))
        idx = rng.choice(n, size=min(n, w.acc_n), replace=False)
        ref = O.direct_type1(*pts, data, w.modes, 1, idx)
    else:
        M = pts[0].size
        idx = rng.choice(M, size=min(M, w.acc_n), replace=False)
        ref = O.direct_type2(*pts, data.ravel(), w.modes, -1, idx)
    est = out_first.ravel()[idx].astype(np.complex128)
    err = float(np.linalg.norm(est - ref) / np.linalg.norm(ref))
    # the same transform by the oracle (FP64 arithmetic, the reference's kernel
    # width and shape for this tol) at the same modes/targets: the error the
    # reference's parameter rule itself leaves, beside ours
    oracle_err = None
    if oracle_same_width and pts[0].size <= 4_000_000:
        plan = oracle_plan(w, os.cpu_count() or 1, ns=ns)
        full = cpu_step(plan, w, [p for p in pts if p is not None], w.data().astype(np.complex128))
        o = np.asarray(full)[0].ravel()[idx]
        oracle_err = float(np.linalg.norm(o - ref) / np.linalg.norm(ref))
    return err, int(idx.size), oracle_err


# --------------------------------------------------------------------------
# Replicas: every rank runs the whole workload on its own GPU; nothing moves
# between ranks except the timings.
def reduce_max(vals, dist, device):
    """Max over the ranks of each value in `vals` (floats); no-op on one rank."""
    import torch
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    if dist is not None and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def replica_rate(world, units, steps, ms):
    """Whole-job rate: `world` replicas each did `units` per step for `steps`
    steps, and the slowest took `ms` in total."""
    return world * units * steps / (ms / 1e3)


# --------------------------------------------------------------------------
def run_reference(args, w: Workload, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    plan = oracle_plan(w, cores, timing=True)
    pts = [p.astype(np.float64) for p in w.points()]
    data = w.data().astype(np.complex128)
    M = pts[0].size
    if M > 4_000_000:  # bounded sample so the run ends within minutes
        n = 4_000_000
        pts = [p[:n] for p in pts]
        if w.ntype == 1:
            data = data[:, :n]
    Ms = pts[0].size
    for _ in range(min(args.warmup, 3)):
        cpu_step(plan, w, pts, data)
    # every step is a full execute of the sample; the run stops after
    # args.steps steps or 120 s, whichever comes first
    t0 = time.perf_counter()
    steps = 0
    while steps < args.steps:
        cpu_step(plan, w, pts, data)
        steps += 1
        if time.perf_counter() - t0 > 120.0:
            break
    total = time.perf_counter() - t0
    args.steps = steps
    value = Ms * w.ntransf * steps / total
    sample = ("full workload per step" if Ms == M else f"{Ms} of {M} points per step (full-size FFT)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if w.single else "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": w.desc, "global_batch": 1, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample + f"; oracle restatement of the reference's path in "
                                            f"{'FP32' if w.single else 'FP64'} arithmetic "
                                            "(spread/interp + deconvolve in C/OpenMP, scipy FFT)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _make_plan(w: Workload, dev, stream, opts):
    import torch

    from cufinufft_gb300 import cufinufft
    plan = cufinufft(w.ntype, w.modes[::-1], n_trans=w.ntransf, eps=w.tol, dtype=w.rdt,
                     isign=1 if w.ntype == 1 else -1, **opts)
    plan.set_stream(stream)
    return plan


def _io_tensors(w: Workload, data_dev, M, dev):
    import torch
    ctorch = torch.complex64 if w.single else torch.complex128
    if w.ntype == 1:
        out = torch.zeros((w.ntransf,) + w.modes[::-1], dtype=ctorch, device=dev)
        return data_dev, out, (data_dev, out)
    out = torch.zeros((w.ntransf, M), dtype=ctorch, device=dev)
    return data_dev, out, (out, data_dev)


def _time_device(plan, args_ce, steps, stream, flush):
    """Device time (ms) of `steps` executes, L2 flushed before each (outside
    the events)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            plan.execute(*args_ce)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev)


def _tuned_plan(w: Workload, dev, stream, opts, pts_dev, args_ce, flush, tuned: bool):
    """The plan to time.  Tuned: the learned selector's layout (gpu_method 0)
    against the library autotuner's best layout class on a second plan over
    the same points; a few flushed executes of each decide which is kept.
    Returns (plan, autotuner entry if it won else None, selector's plan info)."""
    import torch
    plan = _make_plan(w, dev, stream, opts)
    with torch.cuda.stream(stream):
        plan.set_pts(*pts_dev[::-1])  # the Python interface takes C-ordered axes
    torch.cuda.synchronize()
    selector_info = plan.info()
    tune = None
    if tuned:
        alt = _make_plan(w, dev, stream, opts)
        with torch.cuda.stream(stream):
            alt.set_pts(*pts_dev[::-1])
        torch.cuda.synchronize()
        best = alt.autotune()[0]
        # always timed against each other: plan info does not report the
        # subproblem cap, so equal method and bins can still be two classes
        k = 3
        for p in (plan, alt):
            _time_device(p, args_ce, 1, stream, flush)
        t_sel = _time_device(plan, args_ce, k, stream, flush)
        t_alt = _time_device(alt, args_ce, k, stream, flush)
        if t_alt < t_sel:
            plan, alt = alt, plan
            tune = best
        del alt
    return plan, tune, selector_info


def _tuned_opts(args, w: Workload):
    # tuned form: the library chooses the method (gpu_method 0) unless given
    opts = {"gpu_method": args.method}
    if args.upsampfac is not None:
        opts["upsampfac"] = args.upsampfac
    if args.kerevalmeth is not None:
        opts["gpu_kerevalmeth"] = args.kerevalmeth
    elif args.method == 0 and not w.single:
        # tuned FP64: the fitted piecewise-polynomial kernel (Horner) instead
        # of exp(beta sqrt(1 - c x^2)) in FP64 -- same error against the
        # oracle, a third less interpolation time on GB300's FP64 units
        opts["gpu_kerevalmeth"] = 1
    return opts


def run_ours(args, w: Workload, rank, world, local_rank, extra=False):
    """Times the workload and returns its JSON line (rank 0; None on other
    ranks).  `extra`: a second workload of the default run, device time only
    (no e2e, clocks or CPU leg), returned as a smaller record."""
    import torch
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
    pts = w.points()
    M = pts[0].size
    data = w.data()
    opts = dict(_tuned_opts(args, w), width_rule=args.width_rule)
    stream = torch.cuda.Stream(device=dev)
    pts_dev = [torch.from_numpy(p).to(dev) for p in pts]
    data_dev = torch.from_numpy(data).to(dev)
    inp, out, args_ce = _io_tensors(w, data_dev, M, dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    plan, tune, selector_info = _tuned_plan(w, dev, stream, opts, pts_dev, args_ce, flush,
                                            args.method == 0 and args.layout is None)
    if args.layout is not None:
        # a fixed layout for the timed plan (profiling a given kernel)
        lm, lx, ly, lz, lc = (int(v) for v in args.layout.split(","))
        plan.set_layout(lm, (lx, ly, lz)[:w.dim], lc)
    with torch.cuda.stream(stream):
        plan.execute(*args_ce)
    torch.cuda.synchronize()
    info = plan.info()
    out_first = out.cpu().numpy()

    def barrier():
        if dist is not None:
            dist.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            plan.execute(*args_ce)
    torch.cuda.synchronize()

    # ---- timed: device-resident inputs (each execute replays the plan's
    # CUDA graph of its launches)
    clocks = None if extra else ClockSampler(local_rank)
    if clocks:
        clocks.start()
    barrier()
    torch.cuda.synchronize()
    t_start = time.time()
    dev_ms = _time_device(plan, args_ce, args.steps, stream, flush)
    t_end = time.time()
    barrier()
    clk = clocks.stop(t_start, t_end) if clocks else None

    # ---- stage times (roofline): the same executes with the library's stage
    # events on, which launches the kernels directly, over a second timed pass
    stage_steps = max(3, min(args.steps, 500))
    plan.set_timing(True)
    plan.stage_times(reset=True)
    stage_pass_ms = _time_device(plan, args_ce, stage_steps, stream, flush)
    stages = plan.stage_times(reset=True)
    plan.set_timing(False)

    # ---- plain form: the reference's default options (method, bins, exp
    # kernel) at the same kernel width, same inputs
    plain_ms = None
    if not args.no_plain:
        plain = _make_plan(w, dev, stream, {"width_rule": args.width_rule})
        with torch.cuda.stream(stream):
            plain.set_pts(*pts_dev[::-1])
            for _ in range(args.warmup):
                plain.execute(*args_ce)
        torch.cuda.synchronize()
        plain_steps = max(3, min(args.steps, 200))
        plain_ms = _time_device(plain, args_ce, plain_steps, stream, flush) / plain_steps
        plain_info = plain.info()
        del plain

    # ---- parity form: the tuned form at the reference's own kernel width
    # (its results are the reference algorithm's, parameter for parameter)
    parity = None
    if args.width_rule == "tol" and not args.no_plain:
        ppl, ptune, _ = _tuned_plan(w, dev, stream, dict(opts, width_rule="reference"), pts_dev,
                                    args_ce, flush, args.method == 0)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                ppl.execute(*args_ce)
        torch.cuda.synchronize()
        par_out = out.cpu().numpy()
        psteps = max(3, min(args.steps, 200))
        par_ms = _time_device(ppl, args_ce, psteps, stream, flush) / psteps
        pinfo = ppl.info()
        parity = {"value": M * w.ntransf / (par_ms / 1e3), "ms_per_step": par_ms,
                  "ns": pinfo["ns"], "method": pinfo["method"],
                  "bins": [pinfo["binsizex"], pinfo["binsizey"], pinfo["binsizez"]][:w.dim],
                  "note": "same tuned form at the reference's kernel width "
                          "(ns = ceil(-log10(tol/10))), which leaves errors above tol"}
        del ppl

    if extra:
        units = M * w.ntransf
        err, nacc, _ = accuracy(w, out_first, oracle_same_width=False) if not args.no_accuracy \
            else (None, 0, None)
        perr = accuracy(w, par_out, oracle_same_width=False)[0] \
            if (parity is not None and not args.no_accuracy) else None
        if parity is not None:
            parity["rel_l2_err"] = perr
        return {"workload": w.desc, "value": units / (dev_ms / args.steps / 1e3),
                "ms_per_step": dev_ms / args.steps, "steps": args.steps,
                "dtype": "f32" if w.single else "f64", "ns": info["ns"],
                "width_rule": args.width_rule, "method": info["method"],
                "bins": [info["binsizex"], info["binsizey"], info["binsizez"]][:w.dim],
                "cell_order": info["cell_order"], "kerevalmeth": info["kerevalmeth"],
                "layout_from": None if args.method != 0 else (
                    "autotuner" if tune is not None else "selector"),
                "rel_l2_err": err, "rel_l2_points": nacc, "tol": w.tol,
                "plain": None if plain_ms is None else {
                    "value": units / (plain_ms / 1e3), "ms_per_step": plain_ms,
                    "method": plain_info["method"],
                    "note": "reference default options at the same kernel width"},
                "parity_width": parity,
                "stage_ms": {k: v / max(stages["batches"], 1) for k, v in stages.items()
                             if k != "batches"},
                "l2": "flushed between steps (256 MB write, outside the timed events)",
                "timing": "device time of execute() (CUDA events on the plan stream), inputs "
                          "resident"}

    # ---- e2e: host buffers through the public call; every step copies its
    # input from pinned host memory and its output back.  Two plans on two
    # streams alternate so one step's copies overlap the other's compute.
    inp_host = torch.from_numpy(data.copy()).pin_memory()
    out_host = torch.empty((2,) + tuple(out.shape), dtype=out.dtype).pin_memory()
    streams = [stream, torch.cuda.Stream(device=dev)]
    plans = [plan, _make_plan(w, dev, streams[1], opts)]
    with torch.cuda.stream(streams[1]):
        plans[1].set_pts(*pts_dev[::-1])
    if tune is not None:
        plans[1].set_layout(tune["method"], (tune["binsizex"], tune["binsizey"], tune["binsizez"]),
                            tune["maxsubprobsize"])
    stage_in = [torch.empty_like(inp) for _ in range(2)]
    stage_out = [torch.empty_like(out) for _ in range(2)]

    def ce(k):
        return (stage_in[k], stage_out[k]) if w.ntype == 1 else (stage_out[k], stage_in[k])

    def e2e_serial(steps):
        # per step: [events] H2D -> execute -> D2H [events]; L2 flushed
        # between steps outside the events
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        st = streams[0]
        with torch.cuda.stream(st):
            for i in range(steps):
                flush.fill_(float(i))
                ev[i][0].record(st)
                stage_in[0].copy_(inp_host, non_blocking=True)
                plans[0].execute(*ce(0))
                out_host[0].copy_(stage_out[0], non_blocking=True)
                ev[i][1].record(st)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev)

    def e2e_pipelined(steps):
        # a continuous stream of transforms: two plans alternate, so one
        # step's copies overlap the other's compute (no flush in between)
        done = [torch.cuda.Event() for _ in range(2)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(streams[0])
        streams[1].wait_event(t0)
        for i in range(steps):
            k = i % 2
            st = streams[k]
            with torch.cuda.stream(st):
                stage_in[k].copy_(inp_host, non_blocking=True)
                plans[k].execute(*ce(k))
                out_host[k].copy_(stage_out[k], non_blocking=True)
                done[k].record(st)
        streams[0].wait_event(done[1])
        t1.record(streams[0])
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)

    e2e_serial(min(args.warmup, 20))
    e2e_pipelined(max(2, min(args.warmup, 20)))
    barrier()
    e2e_ms = e2e_serial(args.steps)
    e2e_pipe_ms = e2e_pipelined(args.steps)
    barrier()
    # the same transform: equal up to the order of FP32/FP64 atomic additions,
    # which the deconvolution amplifies at low upsampling factors
    for k in range(2):
        dif = np.linalg.norm((out_host[k].numpy() - out_first).ravel())
        if dif > (10 * w.tol + 1e-5) * np.linalg.norm(out_first.ravel()):
            raise RuntimeError("e2e output differs from the device-resident run")

    dev_ms, e2e_ms, e2e_pipe_ms = reduce_max([dev_ms, e2e_ms, e2e_pipe_ms], dist, dev)
    if rank != 0:
        return

    units = M * w.ntransf
    value = replica_rate(world, units, args.steps, dev_ms)
    e2e_value = replica_rate(world, units, args.steps, e2e_ms)
    err, nacc, oracle_err = accuracy(w, out_first, ns=info["ns"]) if not args.no_accuracy \
        else (None, 0, None)
    if parity is not None:
        parity["rel_l2_err"] = accuracy(w, par_out, oracle_same_width=False)[0] \
            if not args.no_accuracy else None

    # roofline of the dominant kernel of ours: spread (type 1) / interp (type 2)
    s = 4 if w.single else 8
    nb = max(stages["batches"], 1)
    k_ms = stages["spreadinterp"] / nb
    nf = [info["nf1"], info["nf2"], info["nf3"]]
    Nf = nf[0] * nf[1] * nf[2]
    grid_bytes = Nf * 2 * s * w.ntransf           # grid read (interp) / written (spread) once
    point_bytes = M * (w.dim * (4 + s) + 4)       # sorted points: first tap + offset per axis, index
    data_bytes = M * 2 * s * w.ntransf            # strengths read / values written
    alg = grid_bytes + point_bytes + data_bytes
    achieved = alg / (k_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    kname = ("spread" if w.ntype == 1 else "interp") + ("_sm" if info["method"] == 2 else "_gm")
    tkey = f"{kname}_{w.name}"
    roof = {"kernel": f"k_{kname}<{'float' if w.single else 'double'},{w.dim},{info['ns']}>",
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": committed_traffic(tkey),
            "algorithmic_bytes": alg, "kernel_ms": k_ms,
            "kernel_ms_source": f"library stage events over a second timed pass of {stage_steps} "
                                f"executes launched directly ({stage_pass_ms / stage_steps:.4f} ms "
                                f"per execute there)",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
            "stage_ms": {k: v / nb for k, v in stages.items() if k != "batches"}}
    if w.ntype == 1:
        roof["atomic"] = atomic_roofline(M * info["ns"] ** w.dim * w.ntransf, k_ms, w.single)

    cpu = None
    if world == 1 and not args.no_cpu:
        rate, cores, sample = cpu_sample(w)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if w.single else "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": w.desc, "name": w.name, "global_batch": world, "seq_len": None,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed between steps (256 MB write, outside the timed events)",
                   "form": "tuned (gpu_method 0: the learned selector's layout, or the library "
                           "autotuner's best of its twelve layout classes when that executes "
                           "faster on this plan's points)" if args.method == 0
                   else f"gpu_method {args.method}",
                   "method": info["method"], "ns": info["ns"], "nf": nf[:w.dim],
                   "bins": [info["binsizex"], info["binsizey"], info["binsizez"]][:w.dim],
                   "kerevalmeth": info["kerevalmeth"],
                   "layout_from": None if args.method != 0 else (
                       "autotuner" if tune is not None else "selector"),
                   "selector_pick": None if args.method != 0 else {
                       "method": selector_info["method"],
                       "bins": [selector_info["binsizex"], selector_info["binsizey"],
                                selector_info["binsizez"]][:w.dim]}},
        "rel_l2_err": err, "rel_l2_points": nacc, "tol": w.tol,
        "rel_l2_err_oracle_same_width": oracle_err,
        "width_rule": args.width_rule,
        "parity_width": parity,
        "plain": None if plain_ms is None else {
            "value": units / (plain_ms / 1e3), "ms_per_step": plain_ms,
            "method": plain_info["method"], "ns": plain_info["ns"],
            "note": "reference default options (type 1: gpu_method 2, type 2: gpu_method 1; "
                    "bins, exp kernel) at the same kernel width"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(data.nbytes),
                "d2h_bytes_per_step": int(out.numel() * out.element_size()),
                "ms_per_step": e2e_ms / args.steps,
                "note": "public Python/C-ABI execute with the input copied from pinned host "
                        "memory and the output copied back inside each step's events; L2 "
                        "flushed between steps",
                "pipelined": {"value": replica_rate(world, units, args.steps, e2e_pipe_ms),
                              "ms_per_step": e2e_pipe_ms / args.steps,
                              "note": "same calls as a continuous stream: two plans on two "
                                      "streams alternate so one step's copies overlap the "
                                      "other's compute; no L2 flush between steps"}},
        "gpu_launches": 2 * int(math.ceil(w.ntransf / max(info["maxbatchsize"], 1))) * args.steps,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s_timed": t_end - t_start,
    }
    return line


class Batch64:
    """Config 4: 64 independent 2D type-1 FP32 plans, seeded: N per plan
    log-uniform in 64^2..512^2 (square), M log-uniform in 1e4..2e6, uniform or
    one Gaussian cluster (sigma uniform in [0.02, 1]) around a random centre,
    ntransf uniform in 1..16, tol 1e-5, strengths iid complex N(0,1)."""

    name = "batch64"
    desc = ("uneven batch of 64 2D type-1 FP32 plans: N log-uniform 64^2..512^2, M log-uniform "
            "1e4..2e6 (uniform or Gaussian-clustered, sigma 0.02..1), ntransf 1..16, tol 1e-5")
    tol = 1e-5

    def __init__(self, nplans=64, seed=11):
        rng = np.random.default_rng(seed)
        self.specs = []
        for i in range(nplans):
            n = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
            M = int(round(math.exp(rng.uniform(math.log(1e4), math.log(2e6)))))
            ntr = int(rng.integers(1, 17))
            if rng.uniform() < 0.5:
                pts = [rng.uniform(-np.pi, np.pi, M) for _ in range(2)]
                kind = "uniform"
            else:
                sig = rng.uniform(0.02, 1.0)
                ctr = rng.uniform(-np.pi, np.pi, 2)
                pts = [(ctr[d] + sig * rng.standard_normal(M) + np.pi) % (2 * np.pi) - np.pi
                       for d in range(2)]
                kind = f"cluster sigma {sig:.2f}"
            c = np.empty((ntr, M), dtype=np.complex64)
            c.real = rng.standard_normal((ntr, M))
            c.imag = rng.standard_normal((ntr, M))
            self.specs.append({"modes": (n, n), "M": M, "ntr": ntr, "kind": kind,
                               "pts": [p.astype(np.float32) for p in pts], "c": c})


def run_batch64(args, rank, world, local_rank, extra=False):
    """Config 4: tuned+batched against 64 plain plans; prints its JSON line
    (returns it instead when `extra`)."""
    import torch

    from cufinufft_gb300 import cufinufft, cufinufft_batch
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    wl = Batch64()
    specs = wl.specs
    stream = torch.cuda.Stream(device=dev)
    units = sum(s["M"] * s["ntr"] for s in specs)

    def build(opts, whole_batch=False):
        # whole_batch: all of a plan's transforms in one pass (maxbatchsize =
        # ntransf) instead of the reference's default min(ntransf, 8)
        plans, cs, fks, pts_keep = [], [], [], []
        for s in specs:
            p = cufinufft(1, s["modes"][::-1], n_trans=s["ntr"], eps=wl.tol, dtype=np.float32,
                          maxbatchsize=s["ntr"] if whole_batch else 0,
                          width_rule=args.width_rule, **opts)
            p.set_stream(stream)
            pd = [torch.from_numpy(x).to(dev) for x in s["pts"]]
            with torch.cuda.stream(stream):
                p.set_pts(*pd[::-1])
            pts_keep.append(pd)
            plans.append(p)
            cs.append(torch.from_numpy(s["c"]).to(dev))
            fks.append(torch.zeros((s["ntr"],) + s["modes"][::-1], dtype=torch.complex64,
                                   device=dev))
        torch.cuda.synchronize()
        return plans, cs, fks, pts_keep

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                ev[i][0].record(stream)
            fn()
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / steps

    # plain: the reference's default options, the 64 plans one after another
    plain, cs, fks, keep1 = build({})

    def run_plain():
        with torch.cuda.stream(stream):
            for p, c, f in zip(plain, cs, fks):
                p.execute(c, f)

    # twice: kernels launched directly, as the reference launches them
    # (CUFINUFFT_GRAPH=0), and with each execute replaying its plan's graph
    saved_env = os.environ.get("CUFINUFFT_GRAPH")
    os.environ["CUFINUFFT_GRAPH"] = "0"
    try:
        for _ in range(args.warmup):
            run_plain()
        plain_ms = timed(run_plain, args.steps)
    finally:
        if saved_env is None:
            os.environ.pop("CUFINUFFT_GRAPH", None)
        else:
            os.environ["CUFINUFFT_GRAPH"] = saved_env
    for _ in range(args.warmup):
        run_plain()
    plain_graph_ms = timed(run_plain, args.steps)
    out_plain = [f.cpu().numpy() for f in fks[:8]]
    # and with the reference's subproblem algorithm for method 2 -- per-tap
    # shared-memory atomicAdd into one tile per subproblem -- in place of the
    # library's private-tile kernel (CUFINUFFT_SPREAD_PRIV=0), launched directly
    saved_env = {k: os.environ.get(k) for k in ("CUFINUFFT_GRAPH", "CUFINUFFT_SPREAD_PRIV")}
    os.environ["CUFINUFFT_GRAPH"] = "0"
    os.environ["CUFINUFFT_SPREAD_PRIV"] = "0"
    try:
        for _ in range(args.warmup):
            run_plain()
        plain_atomic_ms = timed(run_plain, args.steps)
    finally:
        for k, v in saved_env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    del plain

    # batched with the library's default choice (gpu_method 0), one graph
    # replay of multi-plan kernels
    tuned, cs2, fks2, keep2 = build({"gpu_method": 0}, whole_batch=True)
    batch = cufinufft_batch(tuned)

    def run_batch_default():
        torch.cuda.current_stream().wait_stream(stream)
        batch.execute(cs2, fks2)
        stream.wait_stream(torch.cuda.default_stream())

    for _ in range(args.warmup):
        run_batch_default()
    default_ms = timed(run_batch_default, max(3, args.steps // 2))
    del batch

    # tuned + batched: every plan autotuned (method, bins, subproblem cap timed
    # on its own points); the batch keeps whichever of the two layouts --
    # library default or per-plan tuned -- ran faster in its warm-up
    t_tune = time.perf_counter()
    chosen = collections.Counter()
    saved = [p.info() for p in tuned]
    for p in tuned:
        e = p.autotune()[0]
        chosen[(e["method"], e["binsizex"], e["maxsubprobsize"] if e["method"] == 2 else 0)] += 1
    batch = cufinufft_batch(tuned)

    def run_tuned():
        torch.cuda.current_stream().wait_stream(stream)
        batch.execute(cs2, fks2)
        stream.wait_stream(torch.cuda.default_stream())

    for _ in range(args.warmup):
        run_tuned()
    tuned_warm_ms = timed(run_tuned, max(3, args.steps // 2))
    policy = "per-plan autotuned layouts"
    if tuned_warm_ms > default_ms:
        del batch
        for p, inf in zip(tuned, saved):
            p.set_layout(inf["method"], (inf["binsizex"], inf["binsizey"], inf["binsizez"]),
                         inf.get("maxsubprobsize", 1024) if inf["method"] == 2 else 1024)
        batch = cufinufft_batch(tuned)
        policy = "library default layouts (faster than per-plan tuned in the warm-up)"
    tune_s = time.perf_counter() - t_tune

    def run_batch():
        # the batch orders itself after the legacy default stream; make the
        # flush on `stream` visible to it by ending on the legacy stream
        torch.cuda.current_stream().wait_stream(stream)
        batch.execute(cs2, fks2)
        stream.wait_stream(torch.cuda.default_stream())

    for _ in range(args.warmup):
        run_batch()
    clocks = None if extra else ClockSampler(local_rank)
    if clocks:
        clocks.start()
    t0 = time.time()
    batch_ms = timed(run_batch, args.steps)
    t1 = time.time()
    clk = clocks.stop(t0, t1) if clocks else None
    out_batch = [f.cpu().numpy() for f in fks2[:8]]
    agree = max(float(np.linalg.norm(a - b) / max(np.linalg.norm(a), 1e-30))
                for a, b in zip(out_plain, out_batch))

    # accuracy of the batched results against FP64 direct sums
    err = None
    if not args.no_accuracy:
        from oracle import oracle as O
        O.set_num_threads(os.cpu_count() or 1)
        rng = np.random.default_rng(3)
        errs = []
        for s, fk in list(zip(specs, out_batch))[:8]:
            n = s["modes"][0] * s["modes"][1]
            idx = rng.choice(n, size=64, replace=False)
            ref = O.direct_type1(s["pts"][0].astype(np.float64), s["pts"][1].astype(np.float64),
                                 None, s["c"][0].astype(np.complex128), s["modes"], 1, idx)
            est = fk[0].ravel()[idx]
            errs.append(float(np.linalg.norm(est - ref) / np.linalg.norm(ref)))
        err = max(errs)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": units / (batch_ms / 1e3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": wl.desc, "name": wl.name, "plans": len(specs),
                   "nu_point_transforms": units,
                   "l2": "flushed between steps (256 MB write, outside the timed events)",
                   "form": "tuned+batched: every plan autotuned, one CUDA-graph replay of "
                           "all plans' executes on parallel branches"},
        "plain": {"value": units / (plain_ms / 1e3), "ms_per_step": plain_ms,
                  "note": "the 64 plans with the reference's default options, executed one "
                          "after another on one stream, kernels launched directly as the "
                          "reference launches them (CUFINUFFT_GRAPH=0)",
                  "graph_replay_ms_per_step": plain_graph_ms},
        "plain_shared_atomic": {
            "ms_per_step": plain_atomic_ms,
            "note": "the same 64 plain plans, launched directly, with method-2 spreading by "
                    "per-tap shared-memory atomicAdd into one tile per subproblem (the "
                    "reference's subproblem algorithm, src/2d/spreadinterp2d.cu "
                    "Spread_2d_Subprob) instead of the library's private-tile kernel"},
        "speedup_vs_plain": plain_ms / batch_ms,
        "speedup_vs_plain_graph_replay": plain_graph_ms / batch_ms,
        "speedup_vs_plain_shared_atomic": plain_atomic_ms / batch_ms,
        "batched_default_ms": default_ms, "batched_tuned_warmup_ms": tuned_warm_ms,
        "autotune": {"seconds": tune_s, "policy": policy,
                     "per_plan_choice": {f"method {m} bins {b}" + (f" maxsub {c}" if c else ""): n
                                         for (m, b, c), n in chosen.items()}},
        "max_rel_diff_batched_vs_plain": agree,
        "rel_l2_err": err, "tol": wl.tol, "width_rule": args.width_rule,
        "rel_l2_note": "worst over the first 8 plans, 64 random modes each, vs FP64 direct sums",
        "clocks": clk,
    }
    if extra:
        return line
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch64"], default="radial2d")
    ap.add_argument("--method", type=int, default=0,
                    help="gpu_method for the timed plan (0 = chosen by the library)")
    ap.add_argument("--kerevalmeth", type=int, default=None)
    ap.add_argument("--upsampfac", type=float, default=None,
                    help="upsampling factor of the timed plan (the reference's opts.upsampfac: "
                         "2.0 by default, 1.25 the low-upsampling grid)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the direct-sum check")
    ap.add_argument("--no-plain", action="store_true", help="skip the default-options plan")
    ap.add_argument("--width-rule", choices=["tol", "reference"], default="tol",
                    help="kernel width: 'tol' meets rel-l2 <= tol (the metric's gate), "
                         "'reference' is the reference's ns = ceil(-log10(tol/10))")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: skip the 3D cluster and uneven-batch lines")
    ap.add_argument("--layout", default=None,
                    help="method,bx,by,bz,maxsub: a fixed layout for the timed plan instead of the "
                         "tuned one (set_layout; method 5 = cell-run spread)")
    ap.add_argument("--points", type=int, default=None,
                    help="number of points of the uniform / clustered workloads (smaller cases "
                         "for profiling; the default is the workload's own)")
    args = ap.parse_args()
    if args.impl == "ours":
        args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", 0))
    if args.workload == "batch64":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "batch64 is timed against the plain per-plan form on the GPU"}))
            return
        run_batch64(args, rank, int(os.environ.get("WORLD_SIZE", 1)),
                    int(os.environ.get("LOCAL_RANK", 0)))
        return
    w = WORKLOADS[args.workload]()
    if args.upsampfac is not None:
        w.upsampfac = args.upsampfac
    if args.points is not None:
        if not hasattr(w, "M"):
            raise SystemExit("--points applies to the uniform and clustered workloads")
        # a smaller case of the same workload (profiling captures)
        w.M = int(args.points)
        w.desc = w.desc + f" (reduced to M={w.M})"
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, w, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        line = run_ours(args, w, rank, world, local_rank)
        if line is not None and world == 1 and args.workload == "radial2d" and not args.no_extras:
            # the other headline configurations, device time only, in the same
            # record: the 3D clustered type 1 and the uneven 64-plan batch
            # (tuned+batched against plain plans)
            import argparse as _ap
            xa = _ap.Namespace(**vars(args))
            xa.steps = max(3, min(args.steps, 10))
            xa.warmup = 3
            t0 = time.time()
            extras = {"cluster3d": run_ours(xa, WORKLOADS["cluster3d"](), rank, world, local_rank,
                                            extra=True),
                      "batch64": run_batch64(xa, rank, world, local_rank, extra=True)}
            extras["wall_s"] = time.time() - t0
            line["extra_workloads"] = extras
        if line is not None:
            print(json.dumps(line), flush=True)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
