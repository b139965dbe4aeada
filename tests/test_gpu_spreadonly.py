"""Spread/interpolation-only plans (opts.gpu_spreadinterponly = 1): nmodes is
the fine grid itself, execute() spreads the strengths into fk (type 1) or
interpolates fk at the points (type 2), with no FFT and no deconvolution --
the operation the reference's spread/interp tests run
(test/spread2d_test.cu:80, test/interp2d_test.cu:94).  Checked against the
oracle's FP64 spread/interp (src/2d/spreadinterp2d.cu:16-98 and :516-593)
on the same grid, for every method, dimension and precision, batches of
three transforms in batches of two, and after the autotuner re-laid the
points out."""
import numpy as np
import pytest

from tests import nufft_cases as NC
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # (type, grid, method)
    (1, (200,), 1), (1, (200,), 2), (2, (200,), 1),
    (1, (64, 48), 1), (1, (64, 48), 2), (2, (64, 48), 1), (2, (64, 48), 2),
    (1, (32, 28, 24), 1), (1, (32, 28, 24), 2), (2, (32, 28, 24), 1), (2, (32, 28, 24), 2),
]


def _oracle(ntype, grid, pts, data, tol, single, ntr):
    plan = O.OraclePlan(ntype, grid, 1, tol, single, spreadinterponly=True)
    args = list(pts) + [None] * (3 - len(pts))
    if ntype == 1:
        return plan.spread(*args, c=data, ntr=ntr)
    return plan.interp(*args, fw=data, ntr=ntr)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype,grid,method", CASES)
def test_spread_interp_only_against_oracle(single, ntype, grid, method):
    rng = np.random.default_rng(abs(hash((ntype, grid, method, single))) % 2**32)
    M, ntr = 3000, 3
    tol = 1e-5 if single else 1e-10
    # FP64 runs include points on the fold edges.  In FP32 (ns 6) they stay
    # off them: there c = 4/ns^2 rounds up, so a tap at distance 3 - 4e-14
    # (a point just below 3 pi on this grid) makes 1 - c x^2 negative and the
    # reference's formula, which the oracle restates, returns NaN; the
    # library's kernel returns 0 there.
    pts = NC.points(rng, len(grid), M, edges=not single)
    data = NC.strengths(rng, M, ntr) if ntype == 1 else NC.coeffs(rng, grid, ntr)
    out, info = NC.run_gpu(ntype, grid, pts, data, tol, single, ntr=ntr, gpu_method=method,
                           gpu_spreadinterponly=1, maxbatchsize=2)
    assert (info["nf1"], info["nf2"], info["nf3"])[:len(grid)] == tuple(grid)
    ref = _oracle(ntype, grid, pts, data, tol, single, ntr)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < (1e-5 if single else 1e-12), err


def test_grid_smaller_than_two_kernel_widths_is_rejected():
    from cufinufft_gb300 import cufinufft
    with pytest.raises(RuntimeError):
        cufinufft(1, (10, 64), eps=1e-6, dtype=np.float32, gpu_spreadinterponly=1)  # ns 7: 10 < 14


@pytest.mark.parametrize("ntype", [1, 2])
def test_autotuned_spread_only_plan(ntype):
    import torch
    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(21 + ntype)
    grid = (96, 80)
    M = 20000
    pts = NC.points(rng, 2, M, edges=False)
    data = NC.strengths(rng, M) if ntype == 1 else NC.coeffs(rng, grid)
    plan = cufinufft(ntype, grid[::-1], eps=1e-6, dtype=np.float32, gpu_spreadinterponly=1,
                     gpu_method=2)
    dev = [torch.from_numpy(p.astype(np.float32)).cuda() for p in pts]
    plan.set_pts(*dev[::-1])
    entries = plan.autotune()
    assert entries and entries[0]["ms"] > 0
    if ntype == 1:
        c = torch.from_numpy(data.astype(np.complex64)).cuda()
        fk = torch.zeros(grid[::-1], dtype=c.dtype, device="cuda")
        plan.execute(c, fk)
        out = fk.cpu().numpy()
    else:
        fk = torch.from_numpy(np.ascontiguousarray(data.astype(np.complex64)).reshape(grid[::-1])).cuda()
        c = torch.zeros((M,), dtype=fk.dtype, device="cuda")
        plan.execute(c, fk)
        out = c.cpu().numpy()
    torch.cuda.synchronize()
    ref = _oracle(ntype, grid, pts, data, 1e-6, True, 1)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-5, err


@pytest.mark.parametrize("grid,bins,tol", [((64, 60), (16, 16), 1e-5), ((64, 60), (32, 32), 1e-6),
                                           ((32, 30, 28), (8, 8, 8), 1e-6)])
def test_wide_fp32_kernels_on_the_subproblem_spreads(monkeypatch, grid, bins, tol):
    """FP32 reaches widths above 9 only at upsampling factor 1.25 (9..12
    here), where the private-tile (2D) and slab (3D) spreads stage two or
    three pairs of y kernel rows per lane.  On the grid itself (spread-only:
    no deconvolution, which at sigma 1.25 amplifies FP32 rounding) the
    default kernel must match the shared-atomic kernel to FP32 rounding and
    the oracle's spread at the same width."""
    rng = np.random.default_rng(len(grid) * 100 + bins[0])
    M, ntr = 6000, 2
    pts = NC.points(rng, len(grid), M, edges=False)
    c = NC.strengths(rng, M, ntr)
    kw = dict(ntr=ntr, gpu_method=2, gpu_spreadinterponly=1, maxbatchsize=2, upsampfac=1.25,
              width_rule="tol", gpu_binsizex=bins[0], gpu_binsizey=bins[1])
    if len(grid) == 3:
        kw["gpu_binsizez"] = bins[2]
    env = "CUFINUFFT_SPREAD_PRIV" if len(grid) == 2 else "CUFINUFFT_SPREAD_SLAB"
    monkeypatch.setenv(env, "0")
    ref_atomic, _ = NC.run_gpu(1, grid, pts, c, tol, True, **kw)
    monkeypatch.delenv(env)
    out, info = NC.run_gpu(1, grid, pts, c, tol, True, **kw)
    assert info["ns"] >= 9, info["ns"]
    # norms in FP64: the ES kernel is unnormalised (peak e^beta, ~3e9 per axis
    # at ns 12), so 3D grid values reach ~1e29 and their squares overflow FP32
    out = out.astype(np.complex128)
    ref_atomic = ref_atomic.astype(np.complex128)
    err = np.linalg.norm(out.ravel() - ref_atomic.ravel()) / np.linalg.norm(ref_atomic.ravel())
    assert err < 1e-6, (info["ns"], err)
    plan = O.OraclePlan(1, grid, 1, tol, True, spreadinterponly=True, upsampfac=1.25, ns=info["ns"])
    args = list(pts) + [None] * (3 - len(pts))
    ref = plan.spread(*args, c=c, ntr=ntr)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-5, (info["ns"], err)

