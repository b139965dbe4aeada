"""The selector's CUDA network kernels against the FP64 oracle
(forward, masked-MSE gradient, Adam), and gpu_method 0 switching a plan to
the class the committed network predicts."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rand(seed, B):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, MO.NPARAM).astype(np.float32)
    X = rng.normal(0, 1, (B, MO.F)).astype(np.float32)
    T = rng.normal(0, 1, (B, MO.K)).astype(np.float32)
    Mk = (rng.random((B, MO.K)) < 0.8).astype(np.float32)
    return p, X, T, Mk


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("B", [1, 37, 1600])
def test_mlp_forward(B):
    import torch

    from cufinufft_gb300 import _cufinufft as L
    p, X, _, _ = _rand(B, B)
    Y = torch.zeros(B, MO.K, dtype=torch.float32, device="cuda")
    work = torch.zeros(B * 2 * MO.H, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    P, Xd = _dev(p), _dev(X)
    assert L.mlp_forward(P.data_ptr(), Xd.data_ptr(), B, Y.data_ptr(), work.data_ptr(), s) == 0
    ref, _ = MO.forward(p, X)
    np.testing.assert_allclose(Y.cpu().numpy(), ref, rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("B", [5, 300])
def test_mlp_grad(B):
    import torch

    from cufinufft_gb300 import _cufinufft as L
    p, X, T, Mk = _rand(10 + B, B)
    G = torch.zeros(MO.NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    work = torch.zeros(B * (4 * MO.H + 2 * MO.K), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    P, Xd, Td, Md = _dev(p), _dev(X), _dev(T), _dev(Mk)
    assert L.mlp_grad(P.data_ptr(), Xd.data_ptr(), Td.data_ptr(), Md.data_ptr(), B,
                      float(Mk.sum()), G.data_ptr(), loss.data_ptr(), work.data_ptr(), s) == 0
    l_ref, g_ref = MO.loss_and_grad(p, X, T, Mk)
    g = G.cpu().numpy().astype(np.float64)
    assert abs(loss.item() - l_ref) <= 1e-4 * abs(l_ref)
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)


def test_mlp_adam():
    import torch

    from cufinufft_gb300 import _cufinufft as L
    rng = np.random.default_rng(5)
    p = rng.normal(0, 1, MO.NPARAM).astype(np.float32)
    m = np.zeros(MO.NPARAM)
    v = np.zeros(MO.NPARAM)
    P, M1, M2 = _dev(p), _dev(np.zeros(MO.NPARAM, np.float32)), _dev(np.zeros(MO.NPARAM, np.float32))
    pr = p.astype(np.float64)
    s = torch.cuda.current_stream().cuda_stream
    for step in range(1, 6):
        g = rng.normal(0, 1, MO.NPARAM).astype(np.float32)
        Gd = _dev(g)
        assert L.mlp_adam(P.data_ptr(), Gd.data_ptr(), M1.data_ptr(), M2.data_ptr(), step, 1e-2, s) == 0
        pr, m, v = MO.adam(pr, g.astype(np.float64), m, v, step, 1e-2)
    np.testing.assert_allclose(P.cpu().numpy(), pr, rtol=1e-5, atol=1e-6)


def test_mlp_rejects_bad_args():
    from cufinufft_gb300 import _cufinufft as L
    assert L.mlp_forward(None, None, 1, None, None, None) == 13
    assert L.mlp_grad(None, None, None, None, 1, 1.0, None, None, None, None) == 13
    assert L.mlp_adam(None, None, None, None, 1, 1e-3, None) == 13


def test_training_reduces_loss():
    """A few hundred Adam steps on the CUDA kernels fit a synthetic target."""
    from cufinufft_gb300.selector import train as TR
    rng = np.random.default_rng(8)
    feats = rng.normal(0, 1, (400, MO.F)).astype(np.float32)
    w = rng.normal(0, 1, (MO.F, MO.K))
    times = np.exp(0.3 * np.tanh(feats @ w)).astype(np.float32)
    params, mu, sd, hist = TR.train(feats, times, 400, steps=600, lr=3e-3)
    assert hist[-1][1] < 0.3 * hist[0][1], hist


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_auto_method_uses_selector(seed):
    """gpu_method 0: the plan ends on the layout class whose predicted time
    (oracle forward of the committed network on the plan's features) is
    smallest among the classes the plan can run."""
    import torch

    from cufinufft_gb300 import cufinufft
    trained, mu, sd, params = MO.read_weights_header(
        os.path.join(ROOT, "cufinufft_gb300", "csrc", "selector_weights.h"))
    if not trained:
        pytest.skip("no trained selector compiled in")
    rng = np.random.default_rng(seed)
    dim = 1 + seed % 3
    single = seed % 2 == 0
    dt = np.float32 if single else np.float64
    modes = tuple(int(rng.integers(40, 200 if dim < 3 else 60)) for _ in range(dim))
    M = int(rng.integers(20000, 200000))
    ntype = 1 + (seed // 2) % 2
    pts = [rng.uniform(-np.pi, np.pi if seed != 1 else -2.5, M).astype(dt) for _ in range(dim)]
    plan = cufinufft(ntype, modes[::-1], eps=1e-5 if single else 1e-9, dtype=dt, gpu_method=0)
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    f = plan.features()
    info = plan.info()
    Y, _ = MO.forward(params, ((f - mu) / sd)[None, :])
    Y = Y[0]
    # classes the plan can run: probe them through the same API
    runnable = []
    for k in range(MO.K):
        try:
            plan.set_layout_class(k)
            runnable.append(k)
        except RuntimeError:
            pass
    best = min(runnable, key=lambda k: Y[k])
    keys = ("method", "binsizex", "binsizey", "binsizez")
    layouts = []
    for k in runnable:           # near-ties (FP32 device vs FP64 oracle) accept either
        if Y[k] <= Y[best] + 1e-3:
            plan.set_layout_class(k)
            layouts.append(tuple(plan.info()[key] for key in keys))
    assert tuple(info[key] for key in keys) in layouts, (info, layouts, best)
