"""Slab-owned 3D spreading (k_spread_sm_slab, the default for 3D subproblem
spreading): each warp owns the tile planes of one residue mod ns and adds its
taps with plain shared loads and stores.  Checked against the atomic
warp-cooperative kernel (CUFINUFFT_SPREAD_SLAB=0; equal up to the order of
additions: 1e-6 FP32, 1e-13 FP64 relative l2) and against the oracle (2e-5
FP32, 1e-10 FP64), over kernel widths 2..16, bin shapes, wrapping tiles,
batches with a partial last batch, the cell-run layout's sparse subproblems
and clustered points with full 1024-point subproblems."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel()))


CASES = [
    # modes, M, single, tol, method, bins, ntr
    ((24, 20, 18), 20000, True, 1e-6, 2, (16, 16, 2), 1),
    ((24, 20, 18), 20000, True, 1e-6, 2, (8, 8, 8), 2, "tol"),   # ns 8: full-lane rows
    ((24, 20, 18), 20000, True, 1e-2, 2, (8, 8, 8), 3),
    ((30, 28, 26), 30000, True, 1e-4, 2, (16, 16, 4), 2),
    ((16, 18, 20), 8000, True, 1e-8, 2, (8, 8, 8), 2),      # FP32 ns 9 (its cap at sigma 2): two pairs of y rows
    ((16, 18, 20), 8000, False, 1e-12, 2, (8, 8, 8), 2),
    ((16, 18, 20), 8000, False, 1e-9, 2, (16, 16, 2), 1),
    ((16, 18, 20), 8000, False, 1e-15, 2, (4, 4, 4), 1),
]


@pytest.mark.parametrize("case", CASES)
def test_slab_spread(monkeypatch, case):
    modes, M, single, tol, method, bins, ntr = case[:7]
    rule = case[7] if len(case) > 7 else None
    rng = np.random.default_rng(int(1e6 * tol) % 97 + M)
    dt = np.float32 if single else np.float64
    pts = NC.points(rng, 3, M, lo=-3 * np.pi, hi=3 * np.pi, dtype=dt, edges=False)
    c = NC.strengths(rng, M, ntr)
    kw = dict(ntr=ntr, gpu_method=method, gpu_binsizex=bins[0], gpu_binsizey=bins[1],
              gpu_binsizez=bins[2], maxbatchsize=2)
    if rule:
        kw["width_rule"] = rule
    monkeypatch.setenv("CUFINUFFT_SPREAD_SLAB", "0")
    ref_wc, _ = NC.run_gpu(1, modes, pts, c, tol, single, **kw)
    monkeypatch.delenv("CUFINUFFT_SPREAD_SLAB")
    out, info = NC.run_gpu(1, modes, pts, c, tol, single, **kw)
    assert _rel(out, ref_wc) < (1e-6 if single else 1e-13), info
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, tol, single, ntr=ntr,
                          gpu_method=2, ns=info["ns"])
    assert _rel(out, ref) < (2e-5 if single else 1e-10), info


def _run_cellrun(pts, c, modes, tol):
    """Type 1 FP32 under the cell-run layout (dense subproblems by the
    cell-run kernel, sparse ones by the slab or atomic kernel)."""
    import torch

    from cufinufft_gb300 import cufinufft
    plan = cufinufft(1, modes[::-1], eps=tol, dtype=np.float32, gpu_method=2)
    dev = [torch.from_numpy(p).cuda() for p in pts]
    plan.set_pts(*dev[::-1])
    plan.set_layout(5, (16, 16, 2), 1024)
    cd = torch.from_numpy(c.astype(np.complex64)).cuda()
    fk = torch.zeros((1,) + modes[::-1], dtype=torch.complex64, device="cuda")
    plan.execute(cd, fk)
    torch.cuda.synchronize()
    info = plan.info()
    assert info["cell_order"] == 1
    return fk.cpu().numpy(), info


def test_slab_spread_cellrun_layout(monkeypatch):
    """Cell-run layout: the slab kernel takes the sparse subproblems and the
    cell-run kernel the dense ones."""
    rng = np.random.default_rng(17)
    M, modes = 40000, (32, 30, 28)
    half = M // 2
    u = [rng.uniform(-np.pi, np.pi, half) for _ in range(3)]
    g = [(0.5 + 0.05 * rng.standard_normal(M - half) + np.pi) % (2 * np.pi) - np.pi
         for _ in range(3)]
    pts = [np.concatenate([a, b]).astype(np.float32) for a, b in zip(u, g)]
    c = NC.strengths(rng, M)
    monkeypatch.setenv("CUFINUFFT_SPREAD_SLAB", "0")
    ref_wc, _ = _run_cellrun(pts, c, modes, 1e-5)
    monkeypatch.delenv("CUFINUFFT_SPREAD_SLAB")
    out, info = _run_cellrun(pts, c, modes, 1e-5)
    assert _rel(out, ref_wc) < 5e-6, info   # dense cells: long FP32 sums in another order
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, 1e-5, True,
                          gpu_method=2)
    assert _rel(out, ref) < 2e-5, info


def test_slab_spread_clustered_full_subproblems(monkeypatch):
    """Points packed around a few centres: subproblems of 1024 points (16
    chunks of the staging double buffer), tiles across the periodic edge."""
    rng = np.random.default_rng(5)
    M, modes = 60000, (32, 32, 32)
    centres = np.array([[3.1, -3.1, 0.2], [-1.0, 2.0, 3.0], [0.0, 0.0, -3.14]])
    which = rng.integers(0, 3, M)
    pts = [((centres[which, d] + 0.15 * rng.standard_normal(M) + np.pi) % (2 * np.pi) - np.pi)
           .astype(np.float32) for d in range(3)]
    c = NC.strengths(rng, M)
    kw = dict(gpu_method=2, gpu_binsizex=8, gpu_binsizey=8, gpu_binsizez=8)
    monkeypatch.setenv("CUFINUFFT_SPREAD_SLAB", "0")
    ref_wc, _ = NC.run_gpu(1, modes, pts, c, 1e-5, True, **kw)
    monkeypatch.delenv("CUFINUFFT_SPREAD_SLAB")
    out, info = NC.run_gpu(1, modes, pts, c, 1e-5, True, **kw)
    assert M > 500 * info["nsubprob"]   # mostly full 1024-point subproblems
    assert _rel(out, ref_wc) < 5e-6   # dense cells: thousands of FP32 terms in another order
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c, 1e-5, True,
                          gpu_method=2)
    assert _rel(out, ref) < 2e-5


def test_slab_falls_back_when_it_does_not_fit():
    """FP64 at ns 16 with 8^3 bins: the tile fits shared memory but the
    slab kernel's padded tile and staging do not, so the launch takes the
    atomic kernel -- results against the oracle."""
    rng = np.random.default_rng(31)
    modes, M = (20, 18, 16), 6000
    pts = NC.points(rng, 3, M, dtype=np.float64, edges=False)
    c = NC.strengths(rng, M)
    out, info = NC.run_gpu(1, modes, pts, c, 1e-15, False, gpu_method=2, gpu_binsizex=8,
                           gpu_binsizey=8, gpu_binsizez=8)
    assert info["ns"] == 16
    ref = NC.oracle_nufft(1, modes, pts, c, 1e-15, False, gpu_method=2)
    assert _rel(out, ref) < 1e-10, info
