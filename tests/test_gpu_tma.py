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
