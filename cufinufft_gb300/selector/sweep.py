"""Exhaustive timing sweep for the learned selector (runs on a GPU).

For each seeded workload (workloads.spec) this makes a plan, sets its points,
records the plan's features and times all twelve layout classes with the
library's autotuner (cufinufft[f]_autotune), then writes
    features [n][14], times_ms [n][12] (-2: class not runnable), specs (json)
to an .npz file.

    python -m cufinufft_gb300.selector.sweep --n 2000 --out sweep.npz
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def run(n: int, out: str, start: int = 0, device: int = 0, log_every: int = 50,
        max_seconds: float = None) -> None:
    import torch

    from cufinufft_gb300 import cufinufft
    from cufinufft_gb300.selector import workloads as W
    dev = torch.device("cuda", device)
    torch.cuda.set_device(dev)
    feats, times, specs = [], [], []
    t0 = time.time()
    for i in range(start, start + n):
        s = W.spec(i)
        dt = np.float32 if s["single"] else np.float64
        pts = W.points(s, dev)
        try:
            plan = cufinufft(s["type"], tuple(s["modes"])[::-1], eps=s["tol"], dtype=dt,
                             gpu_method=1)
            plan.set_pts(*pts[::-1])
            f = plan.features()
            entries = plan.autotune()
        except RuntimeError as exc:
            print(f"workload {i} skipped: {exc}", flush=True)
            continue
        ms = [e["ms"] for e in entries[1:13]]
        feats.append(list(f))
        times.append(ms)
        specs.append(s)
        del plan, pts
        if max_seconds is not None and time.time() - t0 > max_seconds:
            print(f"stopping after {i - start + 1} workloads (time limit)", flush=True)
            break
        if (i - start + 1) % log_every == 0:
            torch.cuda.empty_cache()
            print(f"{i - start + 1}/{n} workloads, {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(out, features=np.array(feats, dtype=np.float32),
                        times_ms=np.array(times, dtype=np.float32),
                        specs=np.array(json.dumps(specs)))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2000)
    ap.add_argument("--start", type=int, default=0)
    ap.add_argument("--out", default="sweep.npz")
    ap.add_argument("--max-seconds", type=float, default=None)
    a = ap.parse_args()
    run(a.n, a.out, a.start, max_seconds=a.max_seconds)
