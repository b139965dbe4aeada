"""Double-float FFT of FP64 2D grids (fft_df.cu): FP64 plans whose fine grid
sides are powers of two transform the grid in FP32-pair arithmetic instead of
cuFFT's Z2Z (tol >= 1e-13; CUFINUFFT_FP64_DF_FFT=0 keeps cuFFT).  The result
must agree with the cuFFT form to 1e-13 relative l2 and with the oracle to the
FP64 bound, for types 1 and 2, both signs, square and rectangular grids,
batches with a partial last batch; grids that are not powers of two keep
cuFFT."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel()))


CASES = [
    # ntype, modes, tol, iflag, ntr, maxbatch
    (1, (64, 64), 1e-12, 1, 1, 1),
    (2, (64, 64), 1e-12, -1, 1, 1),
    (1, (128, 32), 1e-9, -1, 3, 2),
    (2, (32, 128), 1e-10, 1, 5, 2),
    (2, (512, 512), 1e-12, -1, 1, 1),
    (1, (256, 128), 1e-11, 1, 2, 2),
]


@pytest.mark.parametrize("ntype,modes,tol,iflag,ntr,maxb", CASES)
def test_df_fft_against_cufft(monkeypatch, ntype, modes, tol, iflag, ntr, maxb):
    rng = np.random.default_rng(ntype * 7 + modes[0] + ntr)
    M = 6000
    pts = NC.points(rng, 2, M, edges=False)
    data = NC.strengths(rng, M, ntr) if ntype == 1 else NC.coeffs(rng, modes, ntr)
    kw = dict(ntr=ntr, iflag=iflag, gpu_method=2, maxbatchsize=maxb)
    monkeypatch.setenv("CUFINUFFT_FP64_DF_FFT", "0")
    ref_cufft, info0 = NC.run_gpu(ntype, modes, pts, data, tol, False, **kw)
    assert info0["df_fft"] == 0
    monkeypatch.delenv("CUFINUFFT_FP64_DF_FFT")
    out, info = NC.run_gpu(ntype, modes, pts, data, tol, False, **kw)
    assert info["df_fft"] == 1, info
    assert _rel(out, ref_cufft) < 1e-13, (info["nf1"], info["nf2"])
    ref = NC.oracle_nufft(ntype, modes, pts, data, tol, False, ntr=ntr, iflag=iflag, gpu_method=2)
    assert _rel(out, ref) < 1e-10


def test_df_fft_not_taken_off_its_domain():
    rng = np.random.default_rng(4)
    pts = NC.points(rng, 2, 1000, edges=False)
    fk = NC.coeffs(rng, (50, 70))
    _, info = NC.run_gpu(2, (50, 70), pts, fk, 1e-12, False, gpu_method=2)   # nf 100 x 140
    assert info["df_fft"] == 0
    _, info = NC.run_gpu(2, (64, 64), pts, NC.coeffs(rng, (64, 64)), 1e-14, False, gpu_method=2)
    assert info["df_fft"] == 0   # below the tol gate
    _, info = NC.run_gpu(2, (64, 64), pts, NC.coeffs(rng, (64, 64)), 1e-5, True, gpu_method=2)
    assert info["df_fft"] == 0   # FP32 plan
