"""Private-tile 2D spreading (k_spread_sm_priv, the default for 2D subproblem
spreading): each warp of the block adds its share of the points into its own
copy of the tile with plain shared loads and stores; the copies are summed
once.  Checked against the atomic warp-cooperative kernel
(CUFINUFFT_SPREAD_PRIV=0; equal up to the order of additions: 1e-6 FP32,
1e-13 FP64 relative l2) and against the oracle (2e-5 FP32, 1e-10 FP64), over
kernel widths 2..16, bin shapes, wrapping tiles, batches with a partial last
batch, the cell-run layout's sparse tails and clustered points with full
1024-point subproblems."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel()))


CASES = [
    # modes, M, single, tol, bins, ntr
    ((64, 60), 30000, True, 1e-6, (32, 32), 1),
    ((64, 60), 30000, True, 1e-6, (16, 16), 2, "tol"),   # ns 8: full-lane rows
    ((64, 60), 30000, True, 1e-2, (16, 16), 3),
    ((90, 70), 40000, True, 1e-4, (64, 64), 2),
    ((50, 70), 20000, True, 1e-5, (24, 40), 1),
    ((48, 40), 10000, True, 1e-8, (16, 16), 2),     # FP32 ns 9 (its cap at sigma 2): two pairs of y rows
    ((48, 40), 10000, False, 1e-12, (32, 32), 2),
    ((48, 40), 10000, False, 1e-9, (16, 16), 1),
    ((40, 40), 8000, False, 1e-15, (8, 8), 1),
]


@pytest.mark.parametrize("case", CASES)
def test_priv_spread(monkeypatch, case):
    modes, M, single, tol, bins, ntr = case[:6]
    rule = case[6] if len(case) > 6 else None
    rng = np.random.default_rng(int(1e6 * tol) % 89 + M)
    dt = np.float32 if single else np.float64
    pts = NC.points(rng, 2, M, lo=-3 * np.pi, hi=3 * np.pi, dtype=dt, edges=False)
    c = NC.strengths(rng, M, ntr)
    kw = dict(ntr=ntr, gpu_method=2, gpu_binsizex=bins[0], gpu_binsizey=bins[1], maxbatchsize=2)
    if rule:
        kw["width_rule"] = rule
    monkeypatch.setenv("CUFINUFFT_SPREAD_PRIV", "0")
    ref_wc, _ = NC.run_gpu(1, modes, pts, c, tol, single, **kw)
    monkeypatch.delenv("CUFINUFFT_SPREAD_PRIV")
    out, info = NC.run_gpu(1, modes, pts, c, tol, single, **kw)
    assert _rel(out, ref_wc) < (1e-6 if single else 1e-13), info
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, tol, single, ntr=ntr,
                          gpu_method=2, ns=info["ns"])
    assert _rel(out, ref) < (2e-5 if single else 1e-10), info


def _run_cellrun(pts, c, modes, tol):
    import torch

    from cufinufft_gb300 import cufinufft
    plan = cufinufft(1, modes[::-1], eps=tol, dtype=np.float32, gpu_method=2)
    dev = [torch.from_numpy(p).cuda() for p in pts]
    plan.set_pts(*dev[::-1])
    plan.set_layout(5, (32, 32), 1024)
    cd = torch.from_numpy(c.astype(np.complex64)).cuda()
    fk = torch.zeros((1,) + modes[::-1], dtype=torch.complex64, device="cuda")
    plan.execute(cd, fk)
    torch.cuda.synchronize()
    info = plan.info()
    assert info["cell_order"] == 1
    return fk.cpu().numpy(), info


def test_priv_spread_cellrun_layout(monkeypatch):
    """Cell-run layout in 2D: dense prefixes by the cell-run kernel, every
    sparse tail by the private-tile kernel."""
    rng = np.random.default_rng(19)
    M, modes = 60000, (96, 80)
    half = M // 2
    u = [rng.uniform(-np.pi, np.pi, half) for _ in range(2)]
    g = [(0.7 + 0.03 * rng.standard_normal(M - half) + np.pi) % (2 * np.pi) - np.pi
         for _ in range(2)]
    pts = [np.concatenate([a, b]).astype(np.float32) for a, b in zip(u, g)]
    c = NC.strengths(rng, M)
    monkeypatch.setenv("CUFINUFFT_SPREAD_PRIV", "0")
    ref_wc, _ = _run_cellrun(pts, c, modes, 1e-5)
    monkeypatch.delenv("CUFINUFFT_SPREAD_PRIV")
    out, info = _run_cellrun(pts, c, modes, 1e-5)
    assert _rel(out, ref_wc) < 5e-6, info   # dense cells: long FP32 sums in another order
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, 1e-5, True,
                          gpu_method=2)
    assert _rel(out, ref) < 2e-5, info


def test_priv_spread_clustered_full_subproblems(monkeypatch):
    rng = np.random.default_rng(6)
    M, modes = 80000, (64, 64)
    centres = np.array([[3.1, -3.1], [-1.0, 2.0], [0.0, -3.14]])
    which = rng.integers(0, 3, M)
    pts = [((centres[which, d] + 0.2 * rng.standard_normal(M) + np.pi) % (2 * np.pi) - np.pi)
           .astype(np.float32) for d in range(2)]
    c = NC.strengths(rng, M)
    kw = dict(gpu_method=2, gpu_binsizex=32, gpu_binsizey=32)
    monkeypatch.setenv("CUFINUFFT_SPREAD_PRIV", "0")
    ref_wc, _ = NC.run_gpu(1, modes, pts, c, 1e-5, True, **kw)
    monkeypatch.delenv("CUFINUFFT_SPREAD_PRIV")
    out, info = NC.run_gpu(1, modes, pts, c, 1e-5, True, **kw)
    assert M > 500 * info["nsubprob"]   # mostly full 1024-point subproblems
    assert _rel(out, ref_wc) < 5e-6
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, 1e-5, True,
                          gpu_method=2)
    assert _rel(out, ref) < 2e-5


def test_priv_falls_back_when_it_does_not_fit():
    """FP64 at ns 16 with 64^2 bins: four private copies of the tile exceed
    shared memory, so the launch takes the atomic kernel -- results against
    the oracle."""
    rng = np.random.default_rng(32)
    modes, M = (80, 72), 20000
    pts = NC.points(rng, 2, M, dtype=np.float64, edges=False)
    c = NC.strengths(rng, M)
    out, info = NC.run_gpu(1, modes, pts, c, 1e-15, False, gpu_method=2, gpu_binsizex=64,
                           gpu_binsizey=64)
    assert info["ns"] == 16
    ref = NC.oracle_nufft(1, modes, pts, c, 1e-15, False, gpu_method=2)
    assert _rel(out, ref) < 1e-10, info
