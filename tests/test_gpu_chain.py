"""FP64 plans at tol >= 1e-6 run their spread/interp, FFT and deconvolution
chain in FP32 (plan info chain_fp32 = 1): the points are folded and placed in
FP64, the kernel's Fourier-series factors evaluated in FP64, c and fk
converted at the boundary.  The reference's FP64 build computes everything in
FP64 (CUFINUFFT_FP64_CHAIN=1 restores that here).

Checks: the chained plan meets tol against FP64 direct sums (tolerance-
meeting width) and agrees with the oracle at the same width within FP32
rounding (2e-5, the bound of FP32 plans); below 1e-6 and with the switch
set, plans stay FP64 (1e-10 against the oracle); the stages repeat, layouts
switch, stage times are read, and a batch of chained plans equals each
plan's own execute."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

CASES = [
    # dim, type, modes, M, tol
    (1, 2, (300,), 5000, 1e-6),
    (2, 1, (50, 40), 8000, 1e-6),
    (2, 2, (64, 48), 8000, 1e-5),
    (3, 1, (16, 18, 14), 8000, 1e-6),
    (3, 2, (16, 18, 14), 8000, 1e-3),
]


@pytest.mark.parametrize("dim,ntype,modes,M,tol", CASES)
def test_chain_meets_tol_and_matches_oracle(dim, ntype, modes, M, tol):
    rng = np.random.default_rng(40 + dim + ntype)
    pts = NC.points(rng, dim, M, lo=-3 * np.pi, hi=3 * np.pi, edges=False)
    data = NC.strengths(rng, M) if ntype == 1 else NC.coeffs(rng, modes)
    out, info = NC.run_gpu(ntype, modes, pts, data, tol, False, width_rule="tol")
    assert info["chain_fp32"] == 1 and info["width_rule"] == 1
    idx = rng.choice(out.size, size=min(out.size, 400), replace=False)
    d = NC.direct(ntype, modes, pts, data, 1 if ntype == 1 else -1, idx)
    err = np.linalg.norm(out.ravel()[idx] - d) / np.linalg.norm(d)
    assert err <= tol, (err, tol)
    ref = NC.oracle_nufft(ntype, modes, pts, data, tol, False, ns=info["ns"])
    same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert same < 2e-5, same


def test_fp64_kept_below_threshold_and_on_request(monkeypatch):
    rng = np.random.default_rng(5)
    modes = (40, 36)
    pts = NC.points(rng, 2, 4000, edges=False)
    c = NC.strengths(rng, 4000)
    out, info = NC.run_gpu(1, modes, pts, c, 1e-7, False)
    assert info["chain_fp32"] == 0
    monkeypatch.setenv("CUFINUFFT_FP64_CHAIN", "1")
    out, info = NC.run_gpu(1, modes, pts, c, 1e-6, False)
    assert info["chain_fp32"] == 0
    ref = NC.oracle_nufft(1, modes, pts, c, 1e-6, False)
    same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert same < 1e-10, same


@pytest.mark.parametrize("method,sort", [(1, 0), (1, 1), (2, 1)])
def test_chain_methods_stages_and_layouts(method, sort):
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(11 + method + sort)
    modes = (48, 40)
    tol = 1e-6
    plan = cufinufft(1, modes[::-1], n_trans=3, eps=tol, dtype=np.float64, gpu_method=method,
                     gpu_sort=sort, maxbatchsize=2)
    for M in (5000, 1200):   # setpts again with another M
        pts = NC.points(rng, 2, M, edges=False)
        c = NC.strengths(rng, M, 3)
        plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
        cd = torch.from_numpy(c).cuda()
        fk = torch.zeros((3,) + modes[::-1], dtype=torch.complex128, device="cuda")
        ref = NC.oracle_nufft(1, modes, pts, c, tol, False, ntr=3, ns=plan.info()["ns"])
        for rep in range(2):  # executes repeat
            plan.execute(cd, fk)
            torch.cuda.synchronize()
            out = fk.cpu().numpy()
            same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
            assert same < 2e-5, (M, rep, same)
    assert plan.info()["chain_fp32"] == 1 and plan.info()["M"] == 1200
    # layouts move the chain's work schedule, not its results
    plan.set_layout(2, (16, 16), 256)
    assert plan.info()["method"] == 2 and plan.info()["binsizex"] == 16
    plan.execute(cd, fk)
    torch.cuda.synchronize()
    assert np.linalg.norm(fk.cpu().numpy().ravel() - ref.ravel()) / np.linalg.norm(ref.ravel()) < 2e-5
    plan.autotune()
    plan.set_timing(True)
    plan.execute(cd, fk)
    st = plan.stage_times(reset=True)
    plan.set_timing(False)
    assert st["batches"] == 2 and st["spreadinterp"] > 0 and st["fft"] > 0
    torch.cuda.synchronize()
    assert np.linalg.norm(fk.cpu().numpy().ravel() - ref.ravel()) / np.linalg.norm(ref.ravel()) < 2e-5


def test_chain_batch_matches_plans():
    import torch

    from cufinufft_gb300 import cufinufft, cufinufft_batch
    rng = np.random.default_rng(77)
    plans, cs, fks, keep, refs = [], [], [], [], []
    for i, (modes, M, ntr) in enumerate((((40, 32), 3000, 2), ((24, 30), 6000, 1),
                                          ((50, 50), 800, 3))):
        p = cufinufft(2, modes[::-1], n_trans=ntr, eps=1e-6, dtype=np.float64)
        pts = NC.points(rng, 2, M, edges=False)
        pd = [torch.from_numpy(x).cuda() for x in pts]
        p.set_pts(*pd[::-1])
        fk = NC.coeffs(rng, modes, ntr)
        c = torch.zeros((ntr, M), dtype=torch.complex128, device="cuda")
        p.execute(c, torch.from_numpy(fk).cuda())
        torch.cuda.synchronize()
        refs.append(c.cpu().numpy())
        plans.append(p)
        keep.append(pd)
        fks.append(torch.from_numpy(fk).cuda())
        cs.append(torch.zeros_like(c))
        assert p.info()["chain_fp32"] == 1
    b = cufinufft_batch(plans)
    b.execute(cs, fks)
    torch.cuda.synchronize()
    for c, r in zip(cs, refs):
        assert np.array_equal(c.cpu().numpy(), r)
    del b
