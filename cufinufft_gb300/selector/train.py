"""Train the learned layout selector on a timing sweep (runs on a GPU).

Inputs: the .npz written by selector/sweep.py (features [n][14], times_ms
[n][12], -2 where a class cannot run).  Targets are log2(t_k / t_min) per
workload, masked where a class did not run.  Workloads 0..n_train-1 train,
the rest are held out.  Features are standardised with the training set's
mean and standard deviation.  Training is full-batch Adam on the library's
own CUDA kernels (cufinufft_mlp_grad / cufinufft_mlp_adam); evaluation uses
cufinufft_mlp_forward.  Writes cufinufft_gb300/csrc/selector_weights.h and a
JSON report of held-out regret against the exhaustive sweep and against the
reference's default layout.

    python -m cufinufft_gb300.selector.train --data sweep.npz --report report.json
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "csrc", "selector_weights.h")


def targets(times):
    t = np.asarray(times, dtype=np.float64)
    ok = t > 0
    tmin = np.where(ok, t, np.inf).min(axis=1, keepdims=True)
    y = np.where(ok, np.log2(np.where(ok, t, 1.0) / tmin), 0.0)
    return y.astype(np.float32), ok.astype(np.float32)


def standardise(feats, n_train):
    mu = feats[:n_train].mean(axis=0)
    sd = feats[:n_train].std(axis=0)
    sd = np.where(sd < 1e-3, 1.0, sd)
    return mu.astype(np.float32), sd.astype(np.float32)


def init_params(seed):
    from cufinufft_gb300._cufinufft import MLP_CLASSES as K
    from cufinufft_gb300._cufinufft import MLP_FEATURES as F
    from cufinufft_gb300._cufinufft import MLP_HIDDEN as H
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((F, H), (H, H), (H, K)):
        lim = np.sqrt(6.0 / fan_in)
        parts += [rng.uniform(-lim, lim, fan_out * fan_in), np.zeros(fan_out)]
    return np.concatenate(parts).astype(np.float32)


def regret(pred, times, choose_cls=None):
    """Mean and worst relative slowdown of the chosen classes against the
    fastest, and the time-weighted total ratio."""
    t = np.asarray(times, dtype=np.float64)
    ok = t > 0
    if choose_cls is None:
        choose_cls = np.argmin(np.where(ok, pred, np.inf), axis=1)
    tmin = np.where(ok, t, np.inf).min(axis=1)
    tc = t[np.arange(len(t)), choose_cls]
    r = tc / tmin - 1.0
    return {"mean": float(r.mean()), "median": float(np.median(r)), "max": float(r.max()),
            "total_ratio": float(tc.sum() / tmin.sum()),
            "exact": float(np.mean(r == 0))}


def default_classes(specs, times):
    """The reference's default layout: type 1 method 2 (class 6: medium bins,
    cap 1024), type 2 method 1 (class 1: medium bins)."""
    t = np.asarray(times)
    c = np.array([6 if s["type"] == 1 else 1 for s in specs])
    return np.where(t[np.arange(len(t)), c] > 0, c, 1)    # tile too large: method 1


def train(feats, times, n_train, steps=6000, lr=3e-3, seed=0, device=0):
    import torch

    from cufinufft_gb300 import _cufinufft as L
    dev = torch.device("cuda", device)
    T, Mk = targets(times)
    mu, sd = standardise(feats, n_train)
    X = (feats - mu) / sd
    Xd = torch.from_numpy(X[:n_train].copy()).to(dev)
    Td = torch.from_numpy(T[:n_train].copy()).to(dev)
    Md = torch.from_numpy(Mk[:n_train].copy()).to(dev)
    P = torch.from_numpy(init_params(seed)).to(dev)
    G = torch.zeros_like(P)
    m1 = torch.zeros_like(P)
    m2 = torch.zeros_like(P)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    B = n_train
    work = torch.zeros(B * (4 * L.MLP_HIDDEN + 2 * L.MLP_CLASSES), dtype=torch.float32, device=dev)
    msum = float(Mk[:n_train].sum())
    s = torch.cuda.current_stream(dev).cuda_stream
    hist = []
    for step in range(1, steps + 1):
        cur_lr = lr * (0.1 ** (step / steps))      # exponential decay to lr/10
        assert L.mlp_grad(P.data_ptr(), Xd.data_ptr(), Td.data_ptr(), Md.data_ptr(), B, msum,
                          G.data_ptr(), loss.data_ptr(), work.data_ptr(), s) == 0
        assert L.mlp_adam(P.data_ptr(), G.data_ptr(), m1.data_ptr(), m2.data_ptr(), step, cur_lr,
                          s) == 0
        if step % 500 == 0 or step == 1:
            hist.append((step, float(loss.item())))
    return P.cpu().numpy(), mu, sd, hist


def predict(params, mu, sd, feats, device=0):
    import torch

    from cufinufft_gb300 import _cufinufft as L
    dev = torch.device("cuda", device)
    X = torch.from_numpy(((feats - mu) / sd).astype(np.float32)).to(dev)
    P = torch.from_numpy(np.asarray(params, dtype=np.float32)).to(dev)
    B = X.shape[0]
    Y = torch.zeros(B, L.MLP_CLASSES, dtype=torch.float32, device=dev)
    work = torch.zeros(B * 2 * L.MLP_HIDDEN, dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    assert L.mlp_forward(P.data_ptr(), X.data_ptr(), B, Y.data_ptr(), work.data_ptr(), s) == 0
    return Y.cpu().numpy()


def write_header(params, mu, sd, path=HEADER, note=""):
    def fmt(a):
        return ", ".join("%.9g" % float(x) for x in a)
    lines = [
        "// selector_weights.h -- trained parameters of the learned layout selector.",
        "// Written by cufinufft_gb300/selector/train.py; kSelectorTrained = 0 means no",
        "// trained network is compiled in and gpu_method 0 keeps the built-in rule.",
    ]
    if note:
        lines.append("// " + note)
    lines += ["#pragma once", "", "namespace cfg {", "constexpr int kSelectorTrained = 1;",
              "constexpr float kSelMean[14] = {%s};" % fmt(mu),
              "constexpr float kSelStd[14] = {%s};" % fmt(sd),
              "constexpr float kSelParams[%d] = {" % len(params)]
    for i in range(0, len(params), 8):
        lines.append("    " + fmt(params[i:i + 8]) + ",")
    lines += ["};", "}  // namespace cfg", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--data", required=True)
    ap.add_argument("--n-train", type=int, default=1600)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--report", default=None)
    ap.add_argument("--header", default=HEADER)
    a = ap.parse_args()
    d = np.load(a.data)
    feats, times = d["features"], d["times_ms"]
    specs = json.loads(str(d["specs"]))
    params, mu, sd, hist = train(feats, times, a.n_train, a.steps, a.lr, a.seed)
    pred = predict(params, mu, sd, feats)
    tr, ho = slice(0, a.n_train), slice(a.n_train, len(feats))
    dflt = default_classes(specs, times)
    rep = {"n_train": a.n_train, "n_heldout": len(feats) - a.n_train, "steps": a.steps,
           "loss": hist,
           "train": regret(pred[tr], times[tr]),
           "heldout": regret(pred[ho], times[ho]),
           "heldout_default_layout": regret(None, times[ho], dflt[ho])}
    print(json.dumps(rep, indent=1))
    write_header(params, mu, sd, a.header,
                 note="Trained on %d workloads; held-out mean regret %.3f (default layout %.3f)."
                 % (a.n_train, rep["heldout"]["mean"], rep["heldout_default_layout"]["mean"]))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
