"""Parity at the benchmark configurations' own sizes (seeded synthetic
inputs with their shapes), through the C ABI, against the oracle:

  * 2D type 1 FP32, 256^2 modes, 1e5 uniform points, tol 1e-5, checked on
    1000 random modes;
  * 2D type 2 on the radial MRI-like trajectory (512 golden-angle spokes x
    2048 samples, 1024^2 modes): FP32 tol 1e-6 with the library-chosen
    layout (learned selector) and with the reference's method 1, FP64 tol
    1e-12, checked on 4096 random targets;
  * 3D clustered points (half uniform, half in 8 Gaussian clusters of sigma
    0.05), 128^3 modes, M reduced to 2e6: type 1 FP32 tol 1e-6 (the selector
    picks the cell-run layout for these points) and type 2 FP64 tol 1e-9;
  * a 16-plan slice of the uneven batch (2D type 1 FP32, tol 1e-5) run as
    one batch.

Each case is run at the reference's kernel width and, where the reference's
width leaves an error above tol, at the tolerance-meeting width.  Bounds:
against FP64 direct sums, <= 3 tol at the reference's width (it leaves 1 to
2 tol on these workloads) and <= tol at the tolerance-meeting width; against
the oracle's transform at the same width (same algorithm), the plan
precision's rounding: 2e-5 (FP32), 1e-10 (FP64 exp kernel), tol (FP64
fitted polynomials).  The reference's own checks are single-mode direct sums
(test/cufinufft2d2_test.cu:182-189)."""
import math

import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def radial(spokes=512, samples=2048):
    k = np.arange(spokes)
    theta = k * np.pi * (3.0 - math.sqrt(5.0))
    r = np.linspace(-np.pi, np.pi, samples, endpoint=False)
    return [(r[None, :] * np.cos(theta)[:, None]).ravel(),
            (r[None, :] * np.sin(theta)[:, None]).ravel()]


def clustered3d(M, seed=5):
    rng = np.random.default_rng(seed)
    half = M // 2
    centres = rng.uniform(-np.pi, np.pi, (8, 3))
    which = rng.integers(0, 8, M - half)
    pts = []
    for d in range(3):
        u = rng.uniform(-np.pi, np.pi, half)
        g = centres[which, d] + 0.05 * rng.standard_normal(M - half)
        g = (g + np.pi) % (2 * np.pi) - np.pi
        pts.append(np.concatenate([u, g]))
    return pts


def _check(ntype, modes, pts, data, tol, single, n_check, rule, direct_bound, seed=3,
           oracle=True, **opts):
    dt = np.float32 if single else np.float64
    cdt = np.complex64 if single else np.complex128
    p_in = [p.astype(dt) for p in pts]
    out, info = NC.run_gpu(ntype, modes, p_in, data.astype(cdt), tol, single, width_rule=rule,
                           **opts)
    p64 = [p.astype(np.float64) for p in p_in]
    rng = np.random.default_rng(seed)
    idx = rng.choice(out.size, size=min(out.size, n_check), replace=False)
    d = NC.direct(ntype, modes, p64, data.astype(np.complex128), 1 if ntype == 1 else -1, idx)
    err = np.linalg.norm(out.ravel()[idx] - d) / np.linalg.norm(d)
    assert err <= direct_bound, (err, direct_bound, info["ns"], info["method"])
    if oracle:
        ref = NC.oracle_nufft(ntype, modes, p64, data.astype(np.complex128), tol, single,
                              ns=info["ns"])
        same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
        kmeth = opts.get("gpu_kerevalmeth", 0)
        bound = 2e-5 if single else (max(1e-10, tol) if kmeth else 1e-10)
        assert same <= bound, (same, bound)
    return err, info


@pytest.mark.parametrize("rule,bound", [("reference", 3.0), ("tol", 1.0)])
def test_uniform2d_type1_fp32(rule, bound):
    rng = np.random.default_rng(1)
    M = 100000
    pts = [rng.uniform(-np.pi, np.pi, M) for _ in range(2)]
    c = NC.strengths(rng, M)
    _check(1, (256, 256), pts, c, 1e-5, True, 1000, rule, bound * 1e-5)


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("rule,bound", [("reference", 3.0), ("tol", 1.0)])
def test_radial2d_type2_fp32(method, rule, bound):
    rng = np.random.default_rng(7)
    fk = NC.coeffs(rng, (1024, 1024))
    err, info = _check(2, (1024, 1024), radial(), fk, 1e-6, True, 4096, rule, bound * 1e-6,
                       gpu_method=method)
    if method == 0:
        assert info["method"] in (1, 2)


@pytest.mark.parametrize("kerevalmeth", [0, 1])
def test_radial2d_type2_fp64(kerevalmeth):
    rng = np.random.default_rng(7)
    fk = NC.coeffs(rng, (1024, 1024))
    _check(2, (1024, 1024), radial(), fk, 1e-12, False, 4096, "tol", 1e-12, gpu_method=0,
           gpu_kerevalmeth=kerevalmeth)


def test_cluster3d_type1_fp32_reference_width():
    rng = np.random.default_rng(9)
    M = 2_000_000
    pts = clustered3d(M)
    c = NC.strengths(rng, M)
    err, info = _check(1, (128, 128, 128), pts, c, 1e-6, True, 1000, "reference", 3e-6,
                       gpu_method=0)
    # the learned selector sends these points to the cell-run layout
    assert info["cell_order"] == 1, info


@pytest.mark.parametrize("layout", [(5, (16, 16, 2), 1024), (2, (16, 16, 2), 1024),
                                    (1, (16, 16, 2), 1024)])
def test_cluster3d_type1_fp32_tol_width(layout):
    """At the tolerance-meeting width the kernel's own error is ~2e-7, and the
    rest is FP32 accumulation: a million clustered points add into a few
    hundred cells.  The cell-run layout sums each run in registers and meets
    1e-6; layouts that add every point with FP32 atomics (shared tiles, or the
    grid in L2) reach the FP32 accumulation floor of ~2e-6 on this input."""
    import torch

    from cufinufft_gb300 import cufinufft
    rng = np.random.default_rng(9)
    M = 2_000_000
    modes = (128, 128, 128)
    pts = [p.astype(np.float32) for p in clustered3d(M)]
    c = NC.strengths(rng, M).astype(np.complex64)
    plan = cufinufft(1, modes[::-1], eps=1e-6, dtype=np.float32, width_rule="tol")
    plan.set_pts(*[torch.from_numpy(p).cuda() for p in pts[::-1]])
    plan.set_layout(*layout)
    fk = torch.zeros(modes[::-1], dtype=torch.complex64, device="cuda")
    plan.execute(torch.from_numpy(c).cuda(), fk)
    torch.cuda.synchronize()
    out = fk.cpu().numpy().ravel()
    idx = np.random.default_rng(3).choice(out.size, size=1000, replace=False)
    p64 = [p.astype(np.float64) for p in pts]
    d = NC.direct(1, modes, p64, c.astype(np.complex128), 1, idx)
    err = np.linalg.norm(out[idx] - d) / np.linalg.norm(d)
    bound = 1e-6 if layout[0] == 5 else 3e-6
    assert err <= bound, (layout, err)


def test_cluster3d_type2_fp64():
    rng = np.random.default_rng(9)
    pts = clustered3d(2_000_000)
    fk = NC.coeffs(rng, (128, 128, 128))
    _check(2, (128, 128, 128), pts, fk, 1e-9, False, 1024, "tol", 1e-9, gpu_method=0,
           gpu_kerevalmeth=1)


def test_batch64_slice_against_direct_sums():
    """The first 16 plans of the seeded uneven batch, run as one batch after
    per-plan autotuning, each checked on 64 random modes of its first
    transform; the smaller plans also against the oracle's transform."""
    import torch

    from bench import Batch64
    from cufinufft_gb300 import cufinufft, cufinufft_batch
    specs = Batch64().specs[:16]
    tol = 1e-5
    plans, cs, fks, keep = [], [], [], []
    for s in specs:
        p = cufinufft(1, s["modes"][::-1], n_trans=s["ntr"], eps=tol, dtype=np.float32,
                      maxbatchsize=s["ntr"], gpu_method=0, width_rule="tol")
        pd = [torch.from_numpy(x).cuda() for x in s["pts"]]
        p.set_pts(*pd[::-1])
        p.autotune()
        keep.append(pd)
        plans.append(p)
        cs.append(torch.from_numpy(s["c"]).cuda())
        fks.append(torch.zeros((s["ntr"],) + s["modes"][::-1], dtype=torch.complex64,
                               device="cuda"))
    batch = cufinufft_batch(plans)
    batch.execute(cs, fks)
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    for i, (s, fk) in enumerate(zip(specs, fks)):
        out = fk.cpu().numpy()
        p64 = [x.astype(np.float64) for x in s["pts"]]
        n = s["modes"][0] * s["modes"][1]
        idx = rng.choice(n, size=64, replace=False)
        d = NC.direct(1, s["modes"], p64, s["c"][0].astype(np.complex128), 1, idx)
        err = np.linalg.norm(out[0].ravel()[idx] - d) / np.linalg.norm(d)
        assert err <= tol, (i, err, s["kind"])
        if s["M"] * s["ntr"] <= 2_000_000:
            ns = plans[i].info()["ns"]
            ref = NC.oracle_nufft(1, s["modes"], p64, s["c"].astype(np.complex128), tol, True,
                                  ntr=s["ntr"], ns=ns)
            same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
            assert same <= 2e-5, (i, same)
    del batch
