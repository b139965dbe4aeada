"""Pruned power-of-two FFT passes (csrc/halffft.cu, CUFINUFFT_FFT=half, for
fine grids whose sides are powers of two in [256, 2048]) against cuFFT over the
whole grid (CUFINUFFT_FFT=cufft) and against the oracle.  Both compute the
same transform; the passes split each 2M-point line into two M-point FFTs
over the mode lines only, so results agree to the plan precision's FFT
rounding: 1e-5 relative l2 (FP32), 1e-12 (FP64).  Cases cover odd and even
mode counts, modes filling the whole half line, both signs, batches with a
partial last batch, and 1D/2D/3D."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

CASES = [
    # modes (N1 fastest), type; fine grids 256 .. 2048 per side
    ((509,), 1), ((509,), 2), ((1024,), 2), ((127,), 1),
    ((127, 128), 1), ((127, 128), 2), ((256, 255), 1), ((256, 255), 2), ((1024, 512), 1),
    ((1024, 512), 2), ((128, 127, 126), 1), ((128, 127, 126), 2),
]


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("modes,ntype", CASES)
def test_half_fft_matches_cufft(monkeypatch, modes, ntype, single):
    rng = np.random.default_rng(sum(modes) + ntype)
    dim = len(modes)
    M = 3000
    tol = 1e-5 if single else 1e-9
    dt = np.float32 if single else np.float64
    cdt = np.complex64 if single else np.complex128
    pts = NC.points(rng, dim, M, dtype=dt, edges=False)
    ntr = 3
    data = (NC.strengths(rng, M, ntr) if ntype == 1 else NC.coeffs(rng, modes, ntr)).astype(cdt)
    iflag = -1 if ntype == 1 else 1   # the opposite signs of the defaults
    monkeypatch.setenv("CUFINUFFT_FFT", "half")
    a, ia = NC.run_gpu(ntype, modes, pts, data, tol, single, ntr=ntr, iflag=iflag, maxbatchsize=2)
    monkeypatch.setenv("CUFINUFFT_FFT", "cufft")
    b, ib = NC.run_gpu(ntype, modes, pts, data, tol, single, ntr=ntr, iflag=iflag, maxbatchsize=2)
    assert ia["half_fft"] == 1 and ib["half_fft"] == 0
    rel = np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel())
    assert rel < (1e-5 if single else 1e-12), rel
    ref = NC.oracle_nufft(ntype, modes, [p.astype(np.float64) for p in pts],
                          data.astype(np.complex128), tol, single, ntr=ntr, iflag=iflag)
    same = np.linalg.norm(a.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert same < (2e-5 if single else 1e-10), same


def test_half_fft_not_taken_for_other_sizes(monkeypatch):
    monkeypatch.setenv("CUFINUFFT_FFT", "half")
    rng = np.random.default_rng(2)
    pts = NC.points(rng, 2, 500, dtype=np.float32)
    c = NC.strengths(rng, 500).astype(np.complex64)
    _, info = NC.run_gpu(1, (50, 70), pts, c, 1e-5, True)   # fine grid 100 x 140
    assert info["half_fft"] == 0
