"""Shared helpers for the GPU parity tests: seeded inputs, a run through the
library's Python interface (which calls the C ABI), and the oracle."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def points(rng, dim, M, lo=-np.pi, hi=np.pi, dtype=np.float64, edges=True):
    """Seeded points; with ``edges`` a few land exactly on the fold
    boundaries -3pi, -pi, pi and just below 3pi."""
    pts = [rng.uniform(lo, hi, M) for _ in range(dim)]
    if edges and M >= 8:
        special = np.array([-np.pi, np.pi, -3 * np.pi, np.nextafter(3 * np.pi, 0), 0.0,
                            np.nextafter(-np.pi, 0), np.nextafter(np.pi, 0), -2 * np.pi])
        for p in pts:
            p[:8] = special[rng.permutation(8)]
    return [p.astype(dtype) for p in pts]


def strengths(rng, M, ntr=1, dtype=np.complex128):
    return (rng.standard_normal((ntr, M)) + 1j * rng.standard_normal((ntr, M))).astype(dtype)


def coeffs(rng, modes, ntr=1, dtype=np.complex128):
    shape = (ntr,) + tuple(modes[::-1])
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def run_gpu(ntype, modes, pts, data, tol, single, ntr=1, iflag=None, **opts):
    """Run through cufinufft_gb300.cufinufft with torch CUDA tensors.
    ``modes`` is (N1, N2, N3) with N1 fastest; returns numpy output."""
    import torch

    from cufinufft_gb300 import cufinufft
    dt = np.float32 if single else np.float64
    cdt = np.complex64 if single else np.complex128
    dim = len(modes)
    if iflag is None:
        iflag = 1 if ntype == 1 else -1
    maxbatch = opts.pop("maxbatchsize", 1)
    plan = cufinufft(ntype, tuple(modes[::-1]), n_trans=ntr, eps=tol, isign=iflag, dtype=dt,
                     maxbatchsize=maxbatch, **opts)
    # library x is the fastest axis: the wrapper takes C-ordered axes
    # (kx = slowest ... last = fastest)
    dev = [torch.from_numpy(np.ascontiguousarray(p.astype(dt))).cuda() for p in pts]
    plan.set_pts(*dev[::-1])
    M = pts[0].size
    if ntype == 1:
        c = torch.from_numpy(np.ascontiguousarray(data.astype(cdt))).cuda()
        fk = torch.zeros((ntr,) + tuple(modes[::-1]), dtype=c.dtype, device="cuda")
        plan.execute(c, fk)
        torch.cuda.synchronize()
        out = fk.cpu().numpy()
    else:
        fk = torch.from_numpy(np.ascontiguousarray(data.astype(cdt))).cuda()
        c = torch.zeros((ntr, M), dtype=fk.dtype, device="cuda")
        plan.execute(c, fk)
        torch.cuda.synchronize()
        out = c.cpu().numpy()
    info = plan.info()
    del plan
    return out, info


def oracle_nufft(ntype, modes, pts, data, tol, single, ntr=1, iflag=None, gpu_method=1, **plan_kw):
    """The oracle's transform; ``plan_kw`` passes ``ns`` (a plan's kernel
    width under another width rule) or ``upsampfac`` to the oracle plan."""
    if iflag is None:
        iflag = 1 if ntype == 1 else -1
    plan = O.OraclePlan(ntype, modes, iflag, tol, single, gpu_method=gpu_method, **plan_kw)
    args = list(pts) + [None] * (3 - len(pts))
    return plan.execute(*args, data=data, ntr=ntr)


def direct(ntype, modes, pts, data, iflag, idx):
    """FP64 direct sums at mode (type 1) or target (type 2) indices of the
    first transform."""
    args = list(pts) + [None] * (3 - len(pts))
    if ntype == 1:
        return O.direct_type1(*args, np.asarray(data).reshape(-1)[:pts[0].size], modes, iflag, idx)
    return O.direct_type2(*args, np.asarray(data).reshape(-1)[:int(np.prod(modes))], modes, iflag,
                          idx)
