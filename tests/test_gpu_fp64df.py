"""Double-float interpolation for FP64 plans: the subproblem interpolation of
FP64 type-2 plans with FP32-pair arithmetic (tile, kernel rows and tap sums as
hi + lo floats, ~2^-46 relative) instead of FP64 instructions -- the default
for tol >= 1e-13 (CUFINUFFT_FP64_DF=0 keeps FP64 instructions, =1 forces it
at any tol).  It must agree with the FP64 kernel to 1e-13 relative l2 and with
the oracle to the FP64 bound (1e-10; tol for the fitted polynomials), for both
kernel forms, 2D and 3D (the subproblem method; 1D type 2 runs the global
method), widths up to 16."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

CASES = [
    # dim, modes, tol, kerevalmeth
    (2, (64, 48), 1e-12, 1), (2, (64, 48), 1e-12, 0), (2, (50, 70), 1e-9, 1), (2, (40, 40), 1e-15, 1),
    (3, (20, 18, 16), 1e-9, 1), (3, (20, 18, 16), 1e-9, 0), (3, (16, 16, 16), 1e-12, 1),
]


@pytest.mark.parametrize("dim,modes,tol,kmeth", CASES)
def test_fp64_double_float_interp(monkeypatch, dim, modes, tol, kmeth):
    rng = np.random.default_rng(dim * 10 + kmeth + int(-np.log10(tol)))
    M, ntr = 8000, 2
    pts = NC.points(rng, dim, M, lo=-3 * np.pi, hi=3 * np.pi, edges=False)
    fk = NC.coeffs(rng, modes, ntr)
    method = 2
    monkeypatch.setenv("CUFINUFFT_FP64_DF", "0")
    ref64, info64 = NC.run_gpu(2, modes, pts, fk, tol, False, ntr=ntr, gpu_method=method,
                               gpu_kerevalmeth=kmeth, maxbatchsize=2)
    assert info64["fp64_df"] == 0
    if tol >= 1e-13:
        monkeypatch.delenv("CUFINUFFT_FP64_DF", raising=False)   # the default
    else:
        monkeypatch.setenv("CUFINUFFT_FP64_DF", "1")
    out, info = NC.run_gpu(2, modes, pts, fk, tol, False, ntr=ntr, gpu_method=method,
                           gpu_kerevalmeth=kmeth, maxbatchsize=2)
    assert info["chain_fp32"] == 0 and info["method"] == method and info["fp64_df"] == 1
    diff = np.linalg.norm(out.ravel() - ref64.ravel()) / np.linalg.norm(ref64.ravel())
    assert diff < 1e-13, diff
    ref = NC.oracle_nufft(2, modes, pts, fk, tol, False, ntr=ntr)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < (max(1e-10, tol) if kmeth else 1e-10), err


def test_fp64_df_default_off_below_1e13(monkeypatch):
    monkeypatch.delenv("CUFINUFFT_FP64_DF", raising=False)
    rng = np.random.default_rng(5)
    pts = NC.points(rng, 2, 500, edges=False)
    fk = NC.coeffs(rng, (32, 32), 1)
    _, info = NC.run_gpu(2, (32, 32), pts, fk, 1e-14, False, gpu_method=2)
    assert info["fp64_df"] == 0
