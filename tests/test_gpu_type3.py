"""Type 3 (nonuniform points to nonuniform frequencies), which the reference
reserves in its interface (src/cufinufft.cu:533-536: makeplan returns 1)
without implementing it.  Checked against FP64 direct sums
f_k = sum_j c_j exp(i sgn s_k . x_j) (oracle/nufft_oracle.c orc_dirft_type3):
the method chains a spread, a type-2 transform and a division by the
kernel's Fourier transform, each within the kernel's accuracy, so the bound
is 5 tol (FP32: floored at 5e-5, the FP32 plans' own floor on these sizes)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _run(dim, M, N, tol, single, ntr=1, iflag=1, xr=(-2.0, 5.0), sr=(-30.0, 12.0), seed=0, **opts):
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(seed + 13 * dim + M)
    dt = np.float32 if single else np.float64
    cdt = np.complex64 if single else np.complex128
    xs = [rng.uniform(*xr, M).astype(dt) for _ in range(dim)]
    ss = [rng.uniform(*sr, N).astype(dt) for _ in range(dim)]
    c = NC.strengths(rng, M, ntr).astype(cdt)
    plan = cufinufft(3, (1,) * dim, n_trans=ntr, eps=tol, isign=iflag, dtype=dt, **opts)
    # C-ordered axes: the last one is x
    plan.set_pts(*[torch.from_numpy(a).cuda() for a in xs[::-1]],
                 **dict(zip("stu", [torch.from_numpy(a).cuda() for a in ss[::-1]])))
    fk = torch.zeros((ntr, N), dtype=torch.complex64 if single else torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(c).cuda(), fk)
    torch.cuda.synchronize()
    out = fk.cpu().numpy()
    info = plan.info()
    del plan
    x64 = [a.astype(np.float64) for a in xs] + [None] * (3 - dim)
    s64 = [a.astype(np.float64) for a in ss] + [None] * (3 - dim)
    errs = []
    for t in range(ntr):
        ref = O.direct_type3(*x64, c[t].astype(np.complex128), *s64, iflag, np.arange(N))
        errs.append(np.linalg.norm(out[t] - ref) / np.linalg.norm(ref))
    return max(errs), info


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_type3_against_direct_sum(dim, single):
    for tol in ((1e-4, 1e-5) if single else (1e-6, 1e-9, 1e-12)):
        M = 4000 if dim < 3 else 2000
        err, info = _run(dim, M, 300, tol, single)
        assert info["type"] == 3
        assert err < 5 * max(tol, 1e-5 if single else 0), (tol, err, info["nf1"])


def test_type3_batch_sign_and_centred_data():
    # ntransf 3 with maxbatch 2, negative sign, data centred on 0 and far off it
    err, _ = _run(2, 3000, 200, 1e-9, False, ntr=3, iflag=-1, maxbatchsize=2)
    assert err < 5e-9, err
    err, _ = _run(2, 3000, 200, 1e-9, False, xr=(-1.0, 1.0), sr=(-50.0, 50.0))
    assert err < 5e-9, err
    err, _ = _run(1, 3000, 200, 1e-9, False, xr=(100.0, 104.0), sr=(500.0, 520.0))
    assert err < 5e-9, err


def test_type3_degenerate_extents_and_empty():
    import torch

    from cufinufft_gb300 import cufinufft
    # all frequencies equal (S = 0) and a single source point (X = 0)
    err, _ = _run(1, 1, 50, 1e-9, False, xr=(0.7, 0.7))
    assert err < 5e-9, err
    err, _ = _run(2, 500, 1, 1e-9, False, sr=(3.0, 3.0))
    assert err < 5e-9, err
    # M = 0: zeros out
    plan = cufinufft(3, (1,), eps=1e-6, dtype=np.float64)
    x = torch.zeros(0, dtype=torch.float64, device="cuda")
    s = torch.linspace(-3, 3, 10, dtype=torch.float64, device="cuda")
    plan.set_pts(x, s=s)
    f = torch.ones((1, 10), dtype=torch.complex128, device="cuda")
    plan.execute(torch.zeros((1, 0), dtype=torch.complex128, device="cuda"), f)
    torch.cuda.synchronize()
    assert np.all(f.cpu().numpy() == 0)
