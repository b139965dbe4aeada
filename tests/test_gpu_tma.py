"""Type-2 subproblem interpolation with its tiles moved by tiled bulk
copies (cp.async.bulk.tensor, the default) against the same kernel loading
every tile cell by cell (CUFINUFFT_TMA=0).  Both put the same grid values in
shared memory and run the same arithmetic, so the outputs are bit-identical.
Points reach the grid edges, so wrapping tiles (which keep the per-cell
path inside the same launch) are covered; batches of three transforms with
maxbatchsize 2 cover the transform coordinate of the copies.  (1D type 2
has no subproblem method: src/1d/interp1d_wrapper.cu:100-116 of the reference.)"""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

CASES = [
    # (modes, single, tol, bins)
    ((100, 120), True, 1e-6, None),              # 2D default bins, TX 38
    ((100, 120), False, 1e-9, None),             # 2D FP64, TX 41 (odd is fine for 16-byte cells)
    ((64, 70), True, 1e-5, None),                # ns 6: odd FP32 tile row, widened by one cell
    ((64, 70), True, 1e-6, (31, 16, 1)),         # odd FP32 bin width, per-cell path
    ((24, 30, 20), True, 1e-6, None),            # 3D
    ((24, 30, 20), False, 1e-8, None),           # 3D FP64
]


def _run(monkeypatch, flag, modes, pts, fk, single, tol, bins, ntr):
    monkeypatch.setenv("CUFINUFFT_TMA", flag)
    opts = dict(gpu_method=2, maxbatchsize=2)
    if bins is not None:
        opts.update(gpu_binsizex=bins[0], gpu_binsizey=bins[1], gpu_binsizez=bins[2])
    return NC.run_gpu(2, modes, pts, fk, tol, single, ntr=ntr, **opts)


@pytest.mark.parametrize("modes,single,tol,bins", CASES)
def test_bulk_copy_tiles_match_per_cell_tiles(monkeypatch, modes, single, tol, bins):
    rng = np.random.default_rng(abs(hash((modes, single, tol))) % 2**32)
    ntr = 3
    pts = NC.points(rng, len(modes), 20000)
    fk = NC.coeffs(rng, modes, ntr)
    a, _ = _run(monkeypatch, "1", modes, pts, fk, single, tol, bins, ntr)
    b, _ = _run(monkeypatch, "0", modes, pts, fk, single, tol, bins, ntr)
    assert np.array_equal(a, b)


def test_bulk_copy_tiles_against_oracle(monkeypatch):
    monkeypatch.setenv("CUFINUFFT_TMA", "1")
    rng = np.random.default_rng(5)
    modes = (96, 80)
    pts = NC.points(rng, 2, 6000)
    fk = NC.coeffs(rng, modes)
    out, _ = NC.run_gpu(2, modes, pts, fk, 1e-6, True, gpu_method=2)
    ref = NC.oracle_nufft(2, modes, pts, fk, 1e-6, True)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-5, err


@pytest.mark.parametrize("single", [True, False])
def test_tile_wait_timeout_reported(monkeypatch, single):
    """A tile wait that runs out is recorded, its tile is loaded cell by cell
    (same values, so the result is right), the block waits for the copy
    before it retires, and the next call on the plan returns the CUDA error
    code once.  CUFINUFFT_TMA_WAIT_TEST=1 makes every first wait give up at
    once; the second wait is the normal bounded one, which the copy meets."""
    import torch

    from cufinufft_gb300 import cufinufft
    monkeypatch.setenv("CUFINUFFT_TMA", "1")
    monkeypatch.setenv("CUFINUFFT_TMA_WAIT_TEST", "1")
    rng = np.random.default_rng(8)
    modes = (96, 80)
    dt = np.float32 if single else np.float64
    tol = 1e-6 if single else 1e-9
    pts = NC.points(rng, 2, 6000, dtype=dt)
    fk = NC.coeffs(rng, modes)
    plan = cufinufft(2, modes[::-1], eps=tol, dtype=dt, gpu_method=2)
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    fk_d = torch.from_numpy(fk.astype(plan.complex_dtype)).cuda()
    c_d = torch.zeros((1, pts[0].size), dtype=fk_d.dtype, device="cuda")
    plan.execute(c_d, fk_d)
    torch.cuda.synchronize()
    ref = NC.oracle_nufft(2, modes, [p.astype(np.float64) for p in pts], fk, tol, single)
    out = c_d.cpu().numpy()
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < (1e-5 if single else 1e-10), err
    # the stall is reported by the next call, once
    with pytest.raises(RuntimeError):
        plan.execute(c_d, fk_d)
    monkeypatch.setenv("CUFINUFFT_TMA_WAIT_TEST", "0")
    plan2 = cufinufft(2, modes[::-1], eps=tol, dtype=dt, gpu_method=2)
    plan2.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    plan2.execute(c_d, fk_d)
    torch.cuda.synchronize()
    plan2.execute(c_d, fk_d)  # no stall recorded: no error
    torch.cuda.synchronize()
    assert np.array_equal(c_d.cpu().numpy(), out)
    del plan, plan2
