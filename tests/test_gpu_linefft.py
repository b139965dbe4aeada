"""The pruned line-FFT path (per-axis shared-memory FFTs with the
deconvolution / amplification fused, fftpass.cu; CUFINUFFT_FFT=line)
against the whole-grid cuFFT path (the default), on the same points and inputs: both
compute the same DFT, so they agree to FP rounding.  Covers 1D/2D/3D,
types 1 and 2, FP32 and FP64, power-of-two and 2,3,5-mixed lengths, odd mode
counts, both signs, and a partial last batch."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu

CASES = [
    (1, (50,)), (1, (135,)), (1, (1000,)),      # nf 100, 270, 2000
    (2, (64, 48)), (2, (75, 33)), (2, (192, 256)),
    (3, (16, 12, 10)), (3, (25, 15, 27)),
]


def _run(monkeypatch, backend, ntype, modes, pts, data, tol, single, ntr, iflag, maxbatch):
    monkeypatch.setenv("CUFINUFFT_FFT", backend)
    return NC.run_gpu(ntype, modes, pts, data, tol, single, ntr=ntr, iflag=iflag,
                      maxbatchsize=maxbatch)


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim,modes", CASES)
def test_line_fft_matches_cufft(monkeypatch, single, ntype, dim, modes):
    rng = np.random.default_rng(hash((ntype, modes, single)) % 2**32)
    M = 3000
    ntr = 3
    tol = 1e-5 if single else 1e-11
    iflag = 1 if sum(modes) % 2 else -1
    pts = NC.points(rng, dim, M, edges=False)
    data = NC.strengths(rng, M, ntr) if ntype == 1 else NC.coeffs(rng, modes, ntr)
    a, ia = _run(monkeypatch, "line", ntype, modes, pts, data, tol, single, ntr, iflag, 2)
    b, ib = _run(monkeypatch, "cufft", ntype, modes, pts, data, tol, single, ntr, iflag, 2)
    assert ia["line_fft"] == 1 and ib["line_fft"] == 0
    err = np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel())
    assert err < (2e-6 if single else 1e-13), err


def test_line_fft_against_oracle(monkeypatch):
    """One 2D type-2 FP32 plan with a mixed-radix grid, against the oracle."""
    monkeypatch.setenv("CUFINUFFT_FFT", "line")
    rng = np.random.default_rng(11)
    modes = (135, 96)               # nf 270 x 192
    pts = NC.points(rng, 2, 5000, edges=False)
    fk = NC.coeffs(rng, modes)
    out, info = NC.run_gpu(2, modes, pts, fk, 1e-5, True)
    assert info["line_fft"] == 1 and info["nf1"] == 270
    ref = NC.oracle_nufft(2, modes, pts, fk, 1e-5, True)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 5e-5, err


def test_long_lines_fall_back_to_cufft(monkeypatch):
    monkeypatch.setenv("CUFINUFFT_FFT", "line")
    rng = np.random.default_rng(12)
    pts = NC.points(rng, 1, 2000, edges=False)
    c = NC.strengths(rng, 2000)
    out, info = NC.run_gpu(1, (2500,), pts, c, 1e-9, False)    # FP64: nf 5000 > 4096
    assert info["line_fft"] == 0
    ref = NC.oracle_nufft(1, (2500,), pts, c, 1e-9, False)
    err = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-10, err
