"""Executes replayed as CUDA graphs (the default when stage timing is off)
against direct launches (CUFINUFFT_GRAPH=0): the same kernels on the same
inputs, so type 2 (no atomics) is bit-identical and type 1 agrees to FP32
rounding of the reduction order.  Covers replay with the same arrays,
capture again with new arrays, and new points / a new layout after a capture
(the plan must not replay a graph that holds its old arrays)."""
import numpy as np
import pytest

from tests import nufft_cases as NC

pytestmark = pytest.mark.gpu


def _plan(monkeypatch, graph, ntype, modes, pts, single, **opts):
    import torch

    from cufinufft_gb300 import cufinufft
    monkeypatch.setenv("CUFINUFFT_GRAPH", graph)
    dt = np.float32 if single else np.float64
    plan = cufinufft(ntype, modes[::-1], eps=1e-6 if single else 1e-10, dtype=dt, **opts)
    plan.set_pts(*[torch.from_numpy(p.astype(dt)).cuda() for p in pts[::-1]])
    return plan


def _exec(plan, ntype, modes, M, data, single):
    import torch
    cdt = torch.complex64 if single else torch.complex128
    d = torch.from_numpy(data.astype(np.complex64 if single else np.complex128)).cuda()
    if ntype == 1:
        out = torch.zeros((1,) + modes[::-1], dtype=cdt, device="cuda")
        plan.execute(d, out)
    else:
        out = torch.zeros((1, M), dtype=cdt, device="cuda")
        plan.execute(out, d)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _same(a, b, ntype, single):
    if ntype == 2:
        assert np.array_equal(a, b)
    else:
        err = np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b.ravel())
        assert err < (1e-6 if single else 1e-13), err


@pytest.mark.parametrize("single", [True, False], ids=["f32", "f64"])
@pytest.mark.parametrize("ntype", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_graph_replay_matches_direct(monkeypatch, single, ntype, dim):
    rng = np.random.default_rng(7 * dim + ntype)
    modes = (40, 36) if dim == 2 else (16, 12, 10)
    M = 5000
    pts = NC.points(rng, dim, M)
    data = NC.strengths(rng, M) if ntype == 1 else NC.coeffs(rng, modes)
    ref = _exec(_plan(monkeypatch, "0", ntype, modes, pts, single, gpu_method=2 if ntype == 2 else 1),
                ntype, modes, M, data, single)
    plan = _plan(monkeypatch, "1", ntype, modes, pts, single, gpu_method=2 if ntype == 2 else 1)
    for _ in range(3):  # capture, then replays; every call allocates new arrays (capture again)
        _same(_exec(plan, ntype, modes, M, data, single), ref, ntype, single)


def test_graph_replays_same_arrays_and_sees_new_points(monkeypatch):
    import torch
    rng = np.random.default_rng(31)
    modes, M = (48, 40), 6000
    pts = NC.points(rng, 2, M)
    fk = NC.coeffs(rng, modes).astype(np.complex64)
    plan = _plan(monkeypatch, "1", 2, modes, pts, True, gpu_method=2)
    d = torch.from_numpy(fk).cuda()
    out = torch.zeros((1, M), dtype=torch.complex64, device="cuda")
    plan.execute(out, d)
    torch.cuda.synchronize()
    first = out.cpu().numpy()
    out.zero_()
    plan.execute(out, d)  # same arrays: replay
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), first)
    # new points, same arrays: the replayed graph must not hold the old layout
    pts2 = NC.points(rng, 2, M)
    plan.set_pts(*[torch.from_numpy(p.astype(np.float32)).cuda() for p in pts2[::-1]])
    out.zero_()
    plan.execute(out, d)
    torch.cuda.synchronize()
    ref = NC.oracle_nufft(2, modes, pts2, fk.astype(np.complex128), 1e-6, True)
    err = np.linalg.norm(out.cpu().numpy().ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-5, err
    # another layout, same arrays and points
    plan.set_layout(2, (16, 16), 256)
    out.zero_()
    plan.execute(out, d)
    torch.cuda.synchronize()
    err = np.linalg.norm(out.cpu().numpy().ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert err < 1e-5, err
