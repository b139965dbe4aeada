"""The cell-run spread (layout method 5; the reference's gpu_method 3 in 2D):
points sorted by cell inside their bin, dense runs accumulated in registers.
Results must match the plain method-2 spread (same sums, another order of
additions) and the oracle, with dense runs, sparse points and mixed chunks."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _clustered(rng, dim, M, dt, nf_cells):
    """Half the points inside 2-cell boxes around a few centres (long runs on
    one cell), half uniform (short runs)."""
    h = M // 2
    pts = []
    for d in range(dim):
        c = rng.uniform(-np.pi, np.pi, 3)
        w = 2 * np.pi / nf_cells[d] * 1.5
        dense = c[rng.integers(0, 3, h)] + rng.uniform(0, w, h)
        dense = (dense + np.pi) % (2 * np.pi) - np.pi
        pts.append(np.concatenate([dense, rng.uniform(-np.pi, np.pi, M - h)]).astype(dt))
    return pts


def _run(plan_modes, pts, c, tol, single, ntr, layout=None, **opts):
    import torch

    from cufinufft_gb300 import cufinufft
    dt = np.float32 if single else np.float64
    plan = cufinufft(1, plan_modes[::-1], n_trans=ntr, eps=tol, dtype=dt, maxbatchsize=2, **opts)
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    if layout is not None:
        plan.set_layout(*layout)
    cd = torch.from_numpy(c).cuda()
    fk = torch.zeros((ntr,) + plan_modes[::-1], dtype=cd.dtype, device="cuda")
    plan.execute(cd, fk)
    torch.cuda.synchronize()
    info = plan.info()
    return fk.cpu().numpy(), info


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("dim,modes,bins", [(1, (200,), (64, 1, 1)), (2, (60, 48), (16, 16, 1)),
                                             (2, (40, 40), (32, 32, 1)), (3, (24, 20, 16), (8, 8, 8)),
                                             (3, (20, 20, 20), (16, 16, 2))])
def test_cell_run_matches_plain_and_oracle(single, dim, modes, bins):
    rng = np.random.default_rng(dim * 100 + sum(modes))
    dt = np.float32 if single else np.float64
    # FP64 3D at 1e-7 (ns = 8): the cell-run kernel holds at most 512 taps per point
    tol = 1e-5 if single else (1e-7 if dim == 3 else 1e-9)
    M, ntr = 6000, 3
    pts = _clustered(rng, dim, M, dt, [2 * m for m in modes])
    c = NC.strengths(rng, M, ntr).astype(np.complex64 if single else np.complex128)
    ref_plain, _ = _run(modes, pts, c, tol, single, ntr, gpu_method=2)
    out, info = _run(modes, pts, c, tol, single, ntr, layout=(5, bins, 1024), gpu_method=2)
    assert info["cell_order"] == 1 and info["method"] == 2
    bound = 2e-5 if single else 1e-11   # sums of thousands of terms in another order
    err = np.linalg.norm(out.ravel() - ref_plain.ravel()) / np.linalg.norm(ref_plain.ravel())
    assert err < bound, err
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c.astype(np.complex128),
                          tol, single, ntr=ntr)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < (2e-5 if single else 1e-10), err


def test_all_points_in_one_cell():
    """Every chunk dense: one run per warp slice, flushed once."""
    rng = np.random.default_rng(3)
    modes = (32, 32)
    M = 20000
    x = np.full(M, 0.3) + rng.uniform(0, 1e-3, M)
    y = np.full(M, -1.1) + rng.uniform(0, 1e-3, M)
    pts = [x.astype(np.float32), y.astype(np.float32)]
    c = NC.strengths(rng, M, 1).astype(np.complex64)
    out, info = _run(modes, pts, c, 1e-5, True, 1, layout=(5, (16, 16, 1), 1024), gpu_method=2)
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c.astype(np.complex128),
                          1e-5, True)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 2e-5, err


def test_reference_method3_is_cell_run():
    rng = np.random.default_rng(4)
    modes = (50, 40)
    pts = _clustered(rng, 2, 4000, np.float32, [100, 80])
    c = NC.strengths(rng, 4000, 1).astype(np.complex64)
    out, info = _run(modes, pts, c, 1e-5, True, 1, gpu_method=3)
    assert info["cell_order"] == 1
    plain, _ = _run(modes, pts, c, 1e-5, True, 1, gpu_method=2)
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c.astype(np.complex128),
                          1e-5, True)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    err2 = np.linalg.norm(plain.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    # FP32 sums of thousands of terms per cell: compared against the plain
    # method-2 spread's own FP32 error on the same input
    assert err < max(2e-5, 1.5 * err2), (err, err2)


def test_autotune_reports_twelve_classes_and_keeps_results():
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(5)
    modes = (64, 64)
    pts = _clustered(rng, 2, 20000, np.float32, [128, 128])
    c = torch.from_numpy(NC.strengths(rng, 20000, 1).astype(np.complex64)).cuda()
    plan = cufinufft(1, modes[::-1], eps=1e-5, dtype=np.float32, gpu_method=2)
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    fk0 = torch.zeros(modes[::-1], dtype=torch.complex64, device="cuda")
    plan.execute(c, fk0)
    entries = plan.autotune()
    assert len(entries) == 13
    assert [e["method"] for e in entries[10:13]] == [5, 5, 5]
    assert all(e["ms"] > 0 for e in entries[10:13])
    fk1 = torch.zeros_like(fk0)
    plan.execute(c, fk1)
    torch.cuda.synchronize()
    a, b = fk0.cpu().numpy(), fk1.cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 2e-5


def test_cell_run_rejected_for_type2():
    import torch

    from cufinufft_gb300 import cufinufft
    plan = cufinufft(2, (32, 32), eps=1e-5, dtype=np.float32)
    x = torch.zeros(100, dtype=torch.float32, device="cuda")
    plan.set_pts(x, x)
    with pytest.raises(RuntimeError):
        plan.set_layout(5, (16, 16), 1024)


@pytest.mark.parametrize("tol", [1e-3, 1e-5, 1e-6])
@pytest.mark.parametrize("bins", [(8, 8, 8), (16, 16, 2)])
def test_tensor_core_cell_run_matches(monkeypatch, tol, bins):
    """CUFINUFFT_TC_SPREAD=1: the dense runs of 3D FP32 cell-run subproblems
    are summed by tcgen05 MMAs (TF32 split in two, FP32 accumulation) instead
    of CUDA-core FMAs.  The sums are the same to FP32 rounding, so the result
    matches the CUDA-core cell-run kernel and the oracle (2e-5, the FP32
    bound), with multiple transforms and widths 4 to 7 (<= 8 is the kernel's
    limit)."""
    rng = np.random.default_rng(int(-np.log10(tol)) + bins[2])
    modes = (24, 20, 16)
    M, ntr = 20000, 2
    pts = _clustered(rng, 3, M, np.float32, [2 * m for m in modes])
    c = NC.strengths(rng, M, ntr).astype(np.complex64)
    monkeypatch.delenv("CUFINUFFT_TC_SPREAD", raising=False)
    ref_cc, _ = _run(modes, pts, c, tol, True, ntr, layout=(5, bins, 1024), gpu_method=2)
    monkeypatch.setenv("CUFINUFFT_TC_SPREAD", "1")
    out, info = _run(modes, pts, c, tol, True, ntr, layout=(5, bins, 1024), gpu_method=2)
    assert info["cell_order"] == 1
    err = np.linalg.norm(out.ravel() - ref_cc.ravel()) / np.linalg.norm(ref_cc.ravel())
    assert err < 2e-5, err
    ref = NC.oracle_nufft(1, modes, [p.astype(np.float64) for p in pts], c.astype(np.complex128),
                          tol, True, ntr=ntr)
    err_o = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err_o < 2e-5, err_o
