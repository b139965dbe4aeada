"""The allocation-free spreading entry point, checked against the plan path.

cufinufftf_spread2d_noalloc exists for callers that cannot allocate device
memory where they need the transform (frameworks that own all device memory,
real-time loops, memory-budgeted services): it spreads onto a fine grid the
caller provides and keeps its sort scratch in a fixed device array.  This
test calls it through the C ABI twice in a row (different points, so the
second call must not see the first one's scratch) and checks each grid,
carried through the same FFT and deconvolution on the host, against the
type-1 result of the existing makeplan/setpts/execute path, within the FP32
tolerance the other GPU tests use (2e-5 relative l2).  The file is named to
be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_BOUND = 2e-5


def _entry():
    from cufinufft_gb300 import _cufinufft as L
    fn = L.lib.cufinufftf_spread2d_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("modes,span", [
    ((96, 80), 1),    # fine grid 192 x 160: whole 32-cell bins, points in [-pi, pi)
    ((50, 70), 3),    # fine grid 100 x 140: partial last bins (periodic wrap of
                      # their tiles), points in [-3pi, 3pi) (the fold)
])
def test_noalloc_spread_matches_plan_execute_twice(modes, span):
    import torch

    from cufinufft_gb300 import cufinufft
    from oracle import oracle as O

    spread = _entry()
    tol = 1e-5                # modes are (N1, N2), N1 fastest
    stream = torch.cuda.current_stream()
    for call, (M, seed) in enumerate(((20000, 1), (7000, 2))):
        rng = np.random.default_rng(seed + 10 * span)
        x = rng.uniform(-span * np.pi, span * np.pi, M).astype(np.float32)
        y = rng.uniform(-span * np.pi, span * np.pi, M).astype(np.float32)
        c = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
        xg, yg, cg = (torch.from_numpy(a).cuda() for a in (x, y, c))

        # existing path: makeplan / setpts / execute
        plan = cufinufft(1, modes[::-1], eps=tol, dtype=np.float32)
        plan.set_pts(yg, xg)
        fk = torch.zeros(modes[::-1], dtype=torch.complex64, device="cuda")
        plan.execute(cg, fk)
        info = plan.info()
        nf1, nf2 = info["nf1"], info["nf2"]
        torch.cuda.synchronize()
        fk_plan = fk.cpu().numpy()
        del plan

        # allocation-free spreading onto a caller-provided fine grid
        fw = torch.empty((nf2, nf1), dtype=torch.complex64, device="cuda")
        ier = spread(M, xg.data_ptr(), yg.data_ptr(), cg.data_ptr(), nf1, nf2, tol,
                     fw.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert ier == 0, (call, ier)
        torch.cuda.synchronize()

        # the plan's remaining stages on the host: FFT (+i, unnormalised) and
        # division by the kernel's Fourier series
        op = O.OraclePlan(1, modes, +1, tol, True)
        assert op.nf == (nf1, nf2)
        g = np.fft.ifft2(fw.cpu().numpy().astype(np.complex128), norm="forward")
        k1 = np.arange(modes[0]) - modes[0] // 2
        k2 = np.arange(modes[1]) - modes[1] // 2
        sub = g[np.ix_(k2 % nf2, k1 % nf1)]
        fk_noalloc = sub / np.outer(op.ker[1][np.abs(k2)], op.ker[0][np.abs(k1)])
        err = np.linalg.norm(fk_noalloc - fk_plan) / np.linalg.norm(fk_plan)
        assert err < FP32_BOUND, (call, err)


def test_noalloc_rejects_requests_beyond_its_scratch():
    import torch
    spread = _entry()
    x = torch.zeros(8, dtype=torch.float32, device="cuda")
    c = torch.zeros(8, dtype=torch.complex64, device="cuda")
    fw = torch.zeros(64 * 64, dtype=torch.complex64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # more points than the fixed scratch holds (131072)
    assert spread(200000, x.data_ptr(), x.data_ptr(), c.data_ptr(), 64, 64, 1e-5,
                  fw.data_ptr(), s) == 13
    # a fine grid with more than 4096 bins of 32x32 cells (4096 x 4096 has
    # 16384); both requests are refused before any device work is queued
    assert spread(8, x.data_ptr(), x.data_ptr(), c.data_ptr(), 4096, 4096, 1e-5,
                  fw.data_ptr(), s) == 13
