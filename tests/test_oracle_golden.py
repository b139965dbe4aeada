"""The CPU oracle pinned against the reference's own host code.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from
the reference's contrib/ helpers compiled from source (oracle/_ref).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def params():
    with open(os.path.join(GOLD, "spreader_params.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="module")
def vectors():
    return dict(np.load(os.path.join(GOLD, "reference_vectors.npz")))


def test_setup_spreader_matches_reference(params):
    # contrib/spreadinterp.cpp:6-67, both the FP32 and FP64 builds, bit-exact
    for case in params["setup_spreader"]:
        ier, ns, beta, c = O.setup_spreader(case["tol"], case["prec"] == "f")
        assert (ier, ns) == (case["ier"], case["ns"]), case
        assert beta == case["beta"] and c == case["c"], case


def test_set_nf_matches_reference(params):
    # contrib/common.cpp:24-37 and contrib/utils.cpp:3-22, exact integers
    for case in params["set_nf_type12"]:
        _, ns, _, _ = O.setup_spreader(case["tol"], case["prec"] == "f")
        nf = O.set_nf_type12(case["ms"], ns, case["method"], case["bs"])
        assert nf == case["nf"], case


def test_fseries_matches_reference(vectors):
    # contrib/common.cpp:39-124.  FP64: the reference's phase-winding sum and
    # the oracle's direct cosine sum agree to 1e-9 relative (the winding's own
    # rounding reaches ~6e-11 at k=nf/2).  The FP32 build rounds its phase
    # rates to float, so only 1e-2 relative is asked of it.
    n = 0
    for key, ref in vectors.items():
        if not (key.startswith("d_nf") or key.startswith("f_nf")):
            continue
        prec, nfs, tols = key.split("_")
        nf = int(nfs[2:])
        tol = float(tols[3:])
        _, ns, beta, c = O.setup_spreader(tol, prec == "f")
        mine = O.fseries(nf, ns, beta, c)
        rtol = 1e-9 if prec == "d" else 1e-2
        np.testing.assert_allclose(mine, ref, rtol=rtol, atol=0, err_msg=key)
        n += 1
    assert n >= 20


def test_es_kernel_matches_reference(vectors):
    for single, tol, x, ref in vectors["evaluate_kernel"]:
        _, ns, beta, c = O.setup_spreader(tol, bool(single))
        mine = O.es_kernel(x, ns, beta, c)
        if single:
            # the FP32 build forms c*x*x in float before the FP64 exp/sqrt
            xf = np.float32(x)
            cx2 = np.float32(np.float32(c) * xf) * xf
            if abs(xf) < ns / 2:
                mine = float(np.float32(np.exp(beta * np.sqrt(1.0 - float(cx2)))))
        assert mine == pytest.approx(ref, rel=1e-7 if single else 1e-15, abs=0)


def test_direct_sums_match_reference_dirft2d(vectors):
    # contrib/dirft2d.cpp:7-64 (FP64 build) on seeded inputs
    M, ms, mt = (int(v) for v in vectors["dirft2d_shape"])
    x, y = vectors["dirft2d_x"], vectors["dirft2d_y"]
    c = vectors["dirft2d_c"].view(np.complex128)
    fk = vectors["dirft2d_fk"].view(np.complex128)
    for iflag in (1, -1):
        f1 = O.direct_type1(x, y, None, c, (ms, mt), iflag, np.arange(ms * mt))
        np.testing.assert_allclose(f1, vectors[f"dirft2d1_iflag{iflag}"].view(np.complex128),
                                   rtol=0, atol=1e-12)
        c2 = O.direct_type2(x, y, None, fk, (ms, mt), iflag, np.arange(M))
        np.testing.assert_allclose(c2, vectors[f"dirft2d2_iflag{iflag}"].view(np.complex128),
                                   rtol=0, atol=1e-12)


def test_gauss_legendre_exactness():
    # an n-node rule integrates x^(2n-1) exactly
    for n in (2, 7, 20, 52):
        x, w = O.gauss_legendre(n)
        assert np.all(np.diff(x) < 0)
        for p in range(0, 2 * n, 3):
            exact = 0.0 if p % 2 else 2.0 / (p + 1)
            assert np.sum(w * x ** p) == pytest.approx(exact, abs=1e-13)


@pytest.mark.parametrize("dim,modes,ntype,single", [
    (1, (50,), 1, False), (1, (37,), 2, False),
    (2, (24, 17), 1, True), (2, (16, 22), 2, False),
    (3, (10, 12, 8), 1, False), (3, (9, 10, 11), 2, True),
])
@pytest.mark.parametrize("tol", [1e-3, 1e-6, 1e-10])
def test_oracle_pipeline_meets_tol(dim, modes, ntype, single, tol):
    # the FP64 oracle pipeline (spread/interp -> FFT -> deconvolve) against the
    # FP64 direct sum; points include the folded ranges [-3pi,-pi), [pi,3pi).
    # The reference's width rule ns = ceil(-log10(tol/10)) (contrib/
    # spreadinterp.cpp:42) gives a rel-l2 error of about 1-3 x tol, not a
    # strict bound, so the algorithm's own error is bounded at 5 x tol.
    if single and tol < 1e-7:
        tol = 1e-6
    rng = np.random.default_rng(1000 * dim + ntype)
    M = 300
    pts = [rng.uniform(-3 * np.pi, 3 * np.pi, M) for _ in range(dim)]
    pts += [None] * (3 - dim)
    plan = O.OraclePlan(ntype, modes, +1 if ntype == 1 else -1, tol, single)
    N = int(np.prod(modes))
    if ntype == 1:
        c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        fk = plan.execute(*pts, data=c).ravel()
        ref = O.direct_type1(*pts, c, modes, +1, np.arange(N))
        err = O.rel_l2(fk, ref)
    else:
        fk = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        c = plan.execute(*pts, data=fk).ravel()
        ref = O.direct_type2(*pts, fk, modes, -1, np.arange(M))
        err = O.rel_l2(c, ref)
    assert err < 5 * tol, err


def _np_spread(dim, nf, pts, c, ns, beta, es_c):
    """Plain numpy restatement of the spreader (RESCALE fold,
    contrib/spreadinterp.h:36-38; taps ceil(xr - ns/2) .. + ns - 1 with
    phi = exp(beta sqrt(1 - c x^2)) inside the support,
    src/cuspreadinterp.h:6-40; periodic wrap) for small grids."""
    grid = np.zeros(tuple(nf[::-1]), dtype=np.complex128)
    for p in range(c.size):
        taps = []
        for d in range(dim):
            x = pts[d][p]
            sh = 1.5 if x < -np.pi else (-0.5 if x >= np.pi else 0.5)
            xr = (x / (2 * np.pi) + sh) * nf[d]
            j0 = int(np.ceil(xr - ns / 2.0))
            idx = [(j0 + j) % nf[d] for j in range(ns)]
            ker = []
            for j in range(ns):
                z = (j0 + j) - xr
                ker.append(0.0 if abs(z) >= ns / 2.0 else np.exp(beta * np.sqrt(1.0 - es_c * z * z)))
            taps.append((idx, ker))
        if dim == 1:
            for (i, k) in zip(*taps[0]):
                grid[i] += c[p] * k
        else:
            for (iy, ky) in zip(*taps[1]):
                for (ix, kx) in zip(*taps[0]):
                    grid[iy, ix] += c[p] * kx * ky
    return grid


@pytest.mark.parametrize("grid", [(40,), (24, 20)])
def test_oracle_spread_on_a_given_grid_matches_numpy(grid):
    """The oracle's spread with the grid given directly (spread/interp-only
    plans): against a numpy restatement, FP64 parameters at tol 1e-8."""
    rng = np.random.default_rng(17)
    dim, M = len(grid), 60
    pts = [rng.uniform(-np.pi, np.pi, M) for _ in range(dim)]
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    plan = O.OraclePlan(1, grid, 1, 1e-8, False, spreadinterponly=True)
    assert plan.nf == tuple(grid)
    args = pts + [None] * (3 - dim)
    got = plan.spread(*args, c=c, ntr=1)[0].reshape(tuple(grid[::-1]))
    ref = _np_spread(dim, grid, pts, c, plan.ns, plan.beta, plan.c)
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-9 * np.abs(ref).max())
    # interpolation is the adjoint: <spread(c), g> = <c, interp(g)>
    g = rng.standard_normal(tuple(grid[::-1])) + 1j * rng.standard_normal(tuple(grid[::-1]))
    back = plan.interp(*args, fw=g, ntr=1)[0]
    lhs = np.vdot(g.ravel(), got.ravel())
    rhs = np.vdot(back, c)
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs)


@pytest.mark.parametrize("modes,ns", [((60, 50), 8), ((60, 50), 13), ((40, 33), 11), ((16, 18, 14), 10),
                                      ((300,), 9)])
def test_oracle_spread_independent_of_threads(modes, ns):
    # The coloured bin schedule must be race-free: every cell receives its
    # additions in the same order whatever the thread count, so a serial and
    # a parallel spread agree bit for bit.  Grids whose last bin is narrower
    # than ns - 1 cells (nf 100 with 32-cell bins) once let the halo of the
    # bin before it wrap into bin 0 while bin 0 was being spread.
    rng = np.random.default_rng(ns)
    dim = len(modes)
    plan = O.OraclePlan(1, modes, 1, 1.01 * 10.0 ** (1 - ns), False)
    assert plan.ns == ns
    M = 6000
    pts = [rng.uniform(-np.pi, np.pi, M) for _ in range(dim)] + [None] * (3 - dim)
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    nthr = O.num_threads()
    try:
        O.set_num_threads(1)
        serial = plan.spread(*pts, c)
        O.set_num_threads(max(4, nthr))
        parallel = plan.spread(*pts, c)
    finally:
        O.set_num_threads(nthr)
    assert np.array_equal(serial, parallel)


@pytest.mark.parametrize("ntype,modes", [(1, (40,)), (2, (24, 20)), (1, (12, 10, 8))])
def test_fp32_arith_form_matches_fp64(ntype, modes):
    """The FP32-arithmetic form of the oracle (the CPU timing of FP32
    workloads) computes the same transform: within FP32 rounding of the
    rescaled coordinates (a few 1e-6 at these sizes) of the FP64 oracle."""
    rng = np.random.default_rng(40 + ntype)
    dim, M = len(modes), 3000
    pts = [rng.uniform(-3 * np.pi, 3 * np.pi, M) for _ in range(dim)] + [None] * (3 - dim)
    data = (rng.standard_normal(M) + 1j * rng.standard_normal(M) if ntype == 1 else
            rng.standard_normal(int(np.prod(modes))) + 1j * rng.standard_normal(int(np.prod(modes))))
    iflag = 1 if ntype == 1 else -1
    p64 = O.OraclePlan(ntype, modes, iflag, 1e-6, True)
    p32 = O.OraclePlan(ntype, modes, iflag, 1e-6, True, fp32_arith=True)
    a = p64.execute(*pts, data=data)
    b = p32.execute(*pts, data=data)
    assert b.dtype == np.complex64 and a.dtype == np.complex128
    assert np.linalg.norm(b - a) / np.linalg.norm(a) < 5e-5
