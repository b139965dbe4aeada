"""CPU checks of the layout selector's FP64 network oracle (finite
differences, Adam) and of the committed selector against its committed
timing sweep: held-out regret against the exhaustive sweep and against the
reference's default layout."""
import json
import os

import numpy as np
import pytest

from oracle import mlp_oracle as MO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "cufinufft_gb300", "csrc", "selector_weights.h")
SWEEP = os.path.join(ROOT, "cufinufft_gb300", "selector", "sweep_gb300.npz")


def _rand_problem(seed, B=23):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.4, MO.NPARAM)
    X = rng.normal(0, 1, (B, MO.F))
    T = rng.normal(0, 1, (B, MO.K))
    Mk = (rng.random((B, MO.K)) < 0.8).astype(np.float64)
    return p, X, T, Mk


def test_oracle_gradient_finite_differences():
    p, X, T, Mk = _rand_problem(1)
    _, g = MO.loss_and_grad(p, X, T, Mk)
    rng = np.random.default_rng(2)
    for j in rng.choice(MO.NPARAM, 60, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[j] += h
        pm[j] -= h
        fd = (MO.loss_and_grad(pp, X, T, Mk)[0] - MO.loss_and_grad(pm, X, T, Mk)[0]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-6 * max(1.0, abs(fd)), (j, fd, g[j])


def test_oracle_adam_descends():
    p, X, T, Mk = _rand_problem(3)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    l0 = MO.loss_and_grad(p, X, T, Mk)[0]
    for step in range(1, 201):
        _, g = MO.loss_and_grad(p, X, T, Mk)
        p, m, v = MO.adam(p, g, m, v, step, 1e-2)
    assert MO.loss_and_grad(p, X, T, Mk)[0] < 0.5 * l0


def _committed():
    trained, mu, sd, params = MO.read_weights_header(HEADER)
    if not trained or not os.path.exists(SWEEP):
        pytest.skip("no trained selector committed")
    d = np.load(SWEEP)
    return mu, sd, params, d["features"], d["times_ms"], json.loads(str(d["specs"]))


def _regret(times, cls):
    t = times.astype(np.float64)
    ok = t > 0
    tmin = np.where(ok, t, np.inf).min(axis=1)
    tc = t[np.arange(len(t)), cls]
    return tc / tmin - 1.0, tc.sum() / tmin.sum()


def test_committed_selector_regret_heldout():
    """Held-out workloads (the last 400 of the committed sweep): mean regret of
    the selector's choice against the exhaustive sweep's fastest class <= 10%,
    and lower total time than the reference's default layout."""
    mu, sd, params, feats, times, specs = _committed()
    assert len(params) == MO.NPARAM
    ho = slice(len(feats) - 400, len(feats))
    X = (feats[ho] - mu) / sd
    Y, _ = MO.forward(params, X)
    t = times[ho]
    ok = t > 0
    cls = np.argmin(np.where(ok, Y, np.inf), axis=1)
    r_sel, tot_sel = _regret(t, cls)
    dflt = np.array([6 if s["type"] == 1 else 1 for s in specs[ho]])
    dflt = np.where(t[np.arange(len(t)), dflt] > 0, dflt, 1)
    r_def, tot_def = _regret(t, dflt)
    assert r_sel.mean() <= 0.10, r_sel.mean()
    assert tot_sel < tot_def, (tot_sel, tot_def)
    assert r_sel.mean() < r_def.mean(), (r_sel.mean(), r_def.mean())
