"""Batches of uneven plans (an extension): the batched execution must give
each plan's own result (same algorithm, only the order of floating-point
atomics differs), for type 1 and type 2, FP32 and FP64, across repeated
executes with changing buffers."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _plans(ntype, single, dim, seed, nplans=7):
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(seed)
    dt = np.float32 if single else np.float64
    tol = 1e-5 if single else 1e-9
    plans, inputs = [], []
    for i in range(nplans):
        n = int(rng.integers(8, 40 if dim == 3 else 90))
        modes = tuple(int(n + rng.integers(0, 9)) for _ in range(dim))
        M = 0 if i == 2 else int(rng.integers(50, 3000))
        ntr = int(rng.integers(1, 5))
        lo, hi = (-np.pi, np.pi) if i % 2 else (0.3, 0.9)  # uniform or clustered
        pts = [rng.uniform(lo, hi, M).astype(dt) for _ in range(dim)]
        plan = cufinufft(ntype, modes[::-1], n_trans=ntr, eps=tol, dtype=dt,
                         gpu_method=int(rng.integers(1, 3)))
        plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
        if ntype == 1:
            data = NC.strengths(rng, M, ntr)
        else:
            data = NC.coeffs(rng, modes, ntr)
        data = data.astype(np.complex64 if single else np.complex128)
        plans.append(plan)
        inputs.append((modes, M, ntr, pts, data))
    return plans, inputs


def _run_single(plan, ntype, modes, M, ntr, data):
    import torch
    d = torch.from_numpy(data).cuda()
    if ntype == 1:
        out = torch.zeros((ntr,) + modes[::-1], dtype=d.dtype, device="cuda")
        plan.execute(d, out)
    else:
        out = torch.zeros((ntr, M), dtype=d.dtype, device="cuda")
        plan.execute(out, d)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("mode", ["tables", "plans"])
@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_batch_matches_each_plan(monkeypatch, mode, single, ntype, dim):
    """Both batch forms: multi-plan kernels over descriptor tables, and a
    graph of every plan's own execute (captured again when the arrays
    change, as they do on every repetition here)."""
    import torch

    from cufinufft_gb300 import cufinufft_batch
    monkeypatch.setenv("CUFINUFFT_BATCH", mode)
    plans, inputs = _plans(ntype, single, dim, seed=100 * dim + ntype)
    refs = [_run_single(p, ntype, *inp[:3], inp[4]) for p, inp in zip(plans, inputs)]
    batch = cufinufft_batch(plans)
    bound = 2e-6 if single else 1e-12
    for rep in range(3):
        cs, fks = [], []
        for (modes, M, ntr, pts, data) in inputs:
            d = torch.from_numpy(data).cuda()
            if ntype == 1:
                cs.append(d)
                fks.append(torch.full((ntr,) + modes[::-1], 7.0, dtype=d.dtype, device="cuda"))
            else:
                fks.append(d)
                cs.append(torch.full((ntr, M), 7.0, dtype=d.dtype, device="cuda"))
        batch.execute(cs, fks)
        torch.cuda.synchronize()
        outs = fks if ntype == 1 else cs
        for i, (o, r) in enumerate(zip(outs, refs)):
            o = o.cpu().numpy()
            if r.size == 0 or np.linalg.norm(r) == 0:
                assert np.all(o == 0), (rep, i)
                continue
            err = np.linalg.norm(o.ravel() - r.ravel()) / np.linalg.norm(r.ravel())
            assert err < bound, (rep, i, err)
    del batch


def test_batch_against_oracle():
    """One batch of 2D type-1 FP32 plans checked against the FP64 oracle."""
    import torch

    from cufinufft_gb300 import cufinufft_batch
    plans, inputs = _plans(1, True, 2, seed=77, nplans=5)
    batch = cufinufft_batch(plans)
    cs, fks = [], []
    for (modes, M, ntr, pts, data) in inputs:
        cs.append(torch.from_numpy(data).cuda())
        fks.append(torch.zeros((ntr,) + modes[::-1], dtype=torch.complex64, device="cuda"))
    batch.execute(cs, fks)
    torch.cuda.synchronize()
    for (modes, M, ntr, pts, data), fk in zip(inputs, fks):
        if M == 0:
            continue
        ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts],
                              data.astype(np.complex128), 1e-5, True, ntr=ntr)
        out = fk.cpu().numpy()
        err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
        assert err < 2e-5, err


def test_batch_rejects_mixed_plans():
    import torch

    from cufinufft_gb300 import cufinufft, cufinufft_batch
    a = cufinufft(1, (16, 16), eps=1e-5, dtype=np.float32)
    b = cufinufft(2, (16, 16), eps=1e-5, dtype=np.float32)
    x = torch.zeros(10, dtype=torch.float32, device="cuda")
    a.set_pts(x, x)
    b.set_pts(x, x)
    with pytest.raises(RuntimeError):
        cufinufft_batch([a, b])           # type 1 and type 2 mixed
    c = cufinufft(1, (16, 16), eps=1e-5, dtype=np.float32)
    with pytest.raises(RuntimeError):
        cufinufft_batch([a, c])           # c has no points yet


def test_batch_with_cell_run_plans():
    """Plans switched to the cell-run layout (method 5) run in the batch
    through the multi-plan cell-run kernel and give their own results."""
    import torch

    from cufinufft_gb300 import cufinufft_batch
    plans, inputs = _plans(1, True, 2, seed=91, nplans=6)
    for i, p in enumerate(plans):
        if i % 2 == 0 and inputs[i][1] > 0:
            p.set_layout(5, (16, 16), 1024)
            assert p.info()["cell_order"] == 1
    refs = [_run_single(p, 1, *inp[:3], inp[4]) for p, inp in zip(plans, inputs)]
    batch = cufinufft_batch(plans)
    cs, fks = [], []
    for (modes, M, ntr, pts, data) in inputs:
        d = torch.from_numpy(data).cuda()
        cs.append(d)
        fks.append(torch.zeros((ntr,) + modes[::-1], dtype=d.dtype, device="cuda"))
    batch.execute(cs, fks)
    torch.cuda.synchronize()
    for i, (o, r) in enumerate(zip(fks, refs)):
        o = o.cpu().numpy()
        if np.linalg.norm(r) == 0:
            assert np.all(o == 0)
            continue
        err = np.linalg.norm(o.ravel() - r.ravel()) / np.linalg.norm(r.ravel())
        assert err < 2e-6, (i, err)
