"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Two comparisons per case:
  * against the oracle's FP64 restatement of the same algorithm (same ns,
    beta, grid, kernel): FP64 plans agree to 1e-10 relative l2 (exp-sqrt
    kernel) and FP32 plans to 2e-5 -- rounding of the plan precision only;
    with the fitted piecewise-polynomial kernel (kerevalmeth 1) the fit error
    (~1e-ns of the kernel peak) is added, so the bound is tol;
  * against the FP64 direct sum on a subset of modes/targets: at most
    5 x tol, the error of the reference's own width rule (about 1-3 x tol,
    see tests/test_oracle_golden.py), floored at 2e-5 for FP32 plans.
"""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

MODES = {1: (97,), 2: (24, 33), 3: (12, 10, 14)}
TYPE1_METHODS = {1: [(1, 1), (1, 0), (2, 1)], 2: [(1, 1), (1, 0), (2, 1), (3, 1)],
                 3: [(1, 1), (1, 0), (2, 1), (4, 1)]}
TYPE2_METHODS = {1: [(1, 1), (1, 0)], 2: [(1, 1), (1, 0), (2, 1)], 3: [(1, 1), (1, 0), (2, 1)]}


def info_beta(tol, single):
    from oracle import oracle as O
    return O.setup_spreader(tol, single)[2]


def _bounds(single, tol, kerevalmeth):
    same = (2e-5 if single else 1e-10)
    if kerevalmeth == 1:
        same = max(same, tol)
    direct = 5 * max(tol, 2e-5 if single else 0)
    return same, direct


def _case(ntype, dim, method, sort, single, kerevalmeth, tol, M=1500, ntr=1, maxbatch=1, seed=0,
          lo=-3 * np.pi, hi=3 * np.pi, edges=False, **extra):
    rng = np.random.default_rng(seed + 17 * dim + 5 * ntype + 3 * method)
    modes = MODES[dim]
    pts = NC.points(rng, dim, M, lo, hi, dtype=np.float32 if single else np.float64, edges=edges)
    if ntype == 1:
        data = NC.strengths(rng, M, ntr)
    else:
        data = NC.coeffs(rng, modes, ntr)
    if single:
        data = data.astype(np.complex64)
    out, info = NC.run_gpu(ntype, modes, pts, data, tol, single, ntr=ntr, gpu_method=method,
                           gpu_sort=sort, gpu_kerevalmeth=kerevalmeth, maxbatchsize=maxbatch,
                           **extra)
    ref = NC.oracle_nufft(ntype, modes, [p.astype(np.float64) for p in pts],
                          data.astype(np.complex128), tol, single, ntr=ntr, gpu_method=method)
    # an FP64 plan at tol >= 1e-6 runs its chain in FP32 (plan info
    # chain_fp32): FP32 rounding bounds then
    same, dbound = _bounds(single or info.get("chain_fp32", 0) == 1, tol, kerevalmeth)
    if edges:
        # a point exactly on a fold boundary (x = -pi, pi, -3pi) sits where
        # the kernel is cut off at |x| = ns/2; position roundings ~1e-16 of
        # the two implementations pick the tap on either side of the cut,
        # which moves that point's contribution by exp(-beta) of the peak
        same = max(same, 2.0 * np.exp(-info_beta(tol, single)))
    err_same = float(np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel()))
    assert err_same < same, (err_same, info)
    iflag = 1 if ntype == 1 else -1
    n = int(np.prod(modes)) if ntype == 1 else M
    idx = np.random.default_rng(seed).choice(n, size=min(n, 200), replace=False)
    d = NC.direct(ntype, modes, [p.astype(np.float64) for p in pts], data[0].astype(np.complex128),
                  iflag, idx)
    est = out[0].ravel()[idx]
    err_direct = float(np.linalg.norm(est - d) / np.linalg.norm(d))
    assert err_direct < dbound, (err_direct, info)
    return info


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("ms", [0, 1, 2, 3])
def test_type1_methods(single, dim, ms):
    if ms >= len(TYPE1_METHODS[dim]):
        pytest.skip("method not defined for this dim")
    method, sort = TYPE1_METHODS[dim][ms]
    tol = 1e-5 if single else 1e-9
    info = _case(1, dim, method, sort, single, 0, tol)
    assert info["method"] == (1 if method == 1 else 2)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("ms", [0, 1, 2])
def test_type2_methods(single, dim, ms):
    if ms >= len(TYPE2_METHODS[dim]):
        pytest.skip("method not defined for this dim")
    method, sort = TYPE2_METHODS[dim][ms]
    tol = 1e-5 if single else 1e-9
    _case(2, dim, method, sort, single, 0, tol)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_horner_kernel(single, ntype, dim):
    tol = 1e-4 if single else 1e-11
    method = 2 if (ntype == 1 or dim > 1) else 1
    _case(ntype, dim, method, 1, single, 1, tol)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("tol", [1e-2, 1e-3, 1e-6, 1e-12])
def test_tolerance_sweep_2d(single, tol):
    if single and tol < 1e-6:
        tol = 1e-6
    _case(1, 2, 2, 1, single, 0, tol, seed=3)
    _case(2, 2, 1, 1, single, 0, tol, seed=4)


@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_batched_transforms_partial_last_batch(ntype, dim):
    # ntransf = 5 with maxbatchsize = 2: batches of 2, 2, 1
    # (src/2d/cufinufft2d.cu:39-45 batch loop)
    _case(ntype, dim, 2 if ntype == 1 else 1, 1, True, 0, 1e-5, ntr=5, maxbatch=2, seed=11)
    _case(ntype, dim, 2 if ntype == 1 else 1, 1, False, 0, 1e-9, ntr=5, maxbatch=0, seed=12)


def test_small_subproblems_and_odd_bins():
    # python/cufinufft/tests/test_basic.py:90-119 (gpu_sort False, tiny
    # subproblems) plus bin sizes that do not divide the fine grid
    _case(1, 3, 2, 1, True, 0, 1e-3, M=300, gpu_maxsubprobsize=10)
    _case(1, 2, 2, 1, True, 0, 1e-5, M=3000, gpu_binsizex=7, gpu_binsizey=13)
    _case(2, 2, 2, 1, False, 0, 1e-8, M=3000, gpu_binsizex=5, gpu_binsizey=40)
    _case(1, 3, 1, 0, True, 0, 1e-3, M=300)


def test_clustered_points_many_subproblems():
    # every point in a tiny region: one hot bin, many subproblems
    for single in (True, False):
        for ntype in (1, 2):
            _case(ntype, 2, 2, 1, single, 0, 1e-5 if single else 1e-9, M=20000, lo=0.1, hi=0.12,
                  gpu_maxsubprobsize=256)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_fold_boundary_points(single, ntype, dim):
    # points exactly at -3pi, -pi, 0, pi, -2pi and just inside 3pi
    tol = 1e-3 if single else 1e-6
    _case(ntype, dim, 2 if (ntype == 1 or dim > 1) else 1, 1, single, 0, tol, edges=True, seed=21)


def test_points_in_principal_range_only():
    _case(1, 2, 2, 1, True, 0, 1e-6, lo=-np.pi, hi=np.pi)
    _case(2, 3, 1, 1, False, 0, 1e-10, lo=-np.pi, hi=np.pi)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_library_chosen_method(single, ntype, dim):
    # gpu_method 0 (an extension: the reference rejects it) lets the library
    # pick the method; results are the same algorithm's
    tol = 1e-5 if single else 1e-9
    info = _case(ntype, dim, 0, 1, single, 0, tol, seed=31)
    assert info["method"] in (1, 2)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_set_layout_and_autotune_keep_results(single, ntype, dim):
    """Re-sorting the stored points for another method / bin size (and the
    autotuner, which does that for each candidate) leaves the results equal
    to the oracle's."""
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(40 + dim + 3 * ntype)
    tol = 1e-5 if single else 1e-9
    dt = np.float32 if single else np.float64
    modes = MODES[dim]
    M = 2500
    pts = NC.points(rng, dim, M, dtype=dt, edges=False)
    data = NC.strengths(rng, M) if ntype == 1 else NC.coeffs(rng, modes)
    data = data.astype(np.complex64 if single else np.complex128)
    ref = NC.oracle_nufft(ntype, modes, [p.astype(np.float64) for p in pts],
                          data.astype(np.complex128), tol, single)
    plan = cufinufft(ntype, modes[::-1], eps=tol, dtype=dt)
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    d = torch.from_numpy(data).cuda()

    def run():
        if ntype == 1:
            out = torch.zeros((1,) + modes[::-1], dtype=d.dtype, device="cuda")
            plan.execute(d, out)
        else:
            out = torch.zeros((1, M), dtype=d.dtype, device="cuda")
            plan.execute(out, d)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        return float(np.linalg.norm(o.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel()))

    bound = 2e-5 if single else 1e-10
    assert run() < bound
    layouts = [(1, (7,) * dim), (2, (9,) * dim)] if not (ntype == 2 and dim == 1) else [(1, (7,))]
    for method, bins in layouts:
        plan.set_layout(method, bins, maxsubprobsize=100)
        info = plan.info()
        assert info["method"] == method and info["binsizex"] == bins[0]
        assert run() < bound
    entries = plan.autotune()
    tried = [e for e in entries[1:] if e["ms"] >= 0]
    assert tried and entries[0]["ms"] == min(e["ms"] for e in tried)
    info = plan.info()
    assert info["method"] == entries[0]["method"] and info["binsizex"] == entries[0]["binsizex"]
    assert run() < bound
