"""The tolerance-meeting kernel-width rule (cufinufft_set_width_rule, an
extension): the reference's rule ns = ceil(-log10(tol/10))
(contrib/spreadinterp.cpp:42) leaves relative l2 errors of one to four times
tol; rule 1 widens the kernel until the measured error bound meets tol.

CPU tests: the setter's semantics (pure host code).  GPU tests: plans made
under rule 1 meet tol against FP64 direct sums, and agree with the oracle run
at the same width (the rule changes only the width, not the algorithm)."""
import ctypes

import numpy as np
import pytest

from tests import nufft_cases as NC


def test_set_width_rule_semantics():
    from cufinufft_gb300 import _cufinufft as L
    prev = ctypes.c_int(7)
    assert L._set_width_rule(1, ctypes.byref(prev)) == 0
    first = prev.value
    assert L._set_width_rule(0, ctypes.byref(prev)) == 0
    assert prev.value == 1
    assert L._set_width_rule(-1, ctypes.byref(prev)) == 0
    assert prev.value == 0
    assert L._set_width_rule(first, None) == 0
    for bad in (2, -2, 99):
        assert L._set_width_rule(bad, None) == 13  # CUFINUFFT_ERR_ARG


def test_width_table_matches_generator():
    """The error table in csrc/planner.cpp is the one oracle/width_table.py
    prints (rows ns = 2..16, three dimensions, upsampfac 2 then 1.25)."""
    import os
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(root, "cufinufft_gb300", "csrc", "planner.cpp")).read()
    tables = re.findall(r"kWidthErr(?:2|125)\[15\]\[3\] = \{(.*?)\};", src, flags=re.S)
    assert len(tables) == 2
    for t in tables:
        rows = re.findall(r"\{([^{}]*)\}", t)
        assert len(rows) == 15
        vals = np.array([[float(v) for v in r.split(",")] for r in rows])
        assert vals.shape == (15, 3) and (vals > 0.3).all()


CASES = [
    # dim, type, single, tol, modes, M
    (1, 1, True, 1e-5, (400,), 6000),
    (2, 2, True, 1e-6, (64, 48), 20000),
    (2, 1, True, 1e-5, (50, 70), 20000),
    (3, 1, True, 1e-6, (20, 18, 16), 20000),
    (3, 2, False, 1e-9, (20, 18, 16), 20000),
    (2, 2, False, 1e-12, (64, 48), 20000),
    (1, 2, False, 1e-10, (400,), 6000),
    (2, 1, False, 3e-8, (50, 70), 20000),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dim,ntype,single,tol,modes,M", CASES)
def test_tol_rule_meets_tol(dim, ntype, single, tol, modes, M):
    from oracle import oracle as O
    rng = np.random.default_rng(31 + dim + 7 * ntype)
    dt = np.float32 if single else np.float64
    pts = NC.points(rng, dim, M, dtype=dt, edges=False)
    data = NC.strengths(rng, M) if ntype == 1 else NC.coeffs(rng, modes)
    if single:
        data = data.astype(np.complex64)
    out, info = NC.run_gpu(ntype, modes, pts, data, tol, single, width_rule="tol")
    ref_ns = O.setup_spreader(tol, single)[1]
    assert info["width_rule"] == 1
    assert ref_ns <= info["ns"] <= ref_ns + 2, info["ns"]
    p64 = [p.astype(np.float64) for p in pts]
    n_out = out.size
    idx = rng.choice(n_out, min(n_out, 500), replace=False)
    d = NC.direct(ntype, modes, p64, data.astype(np.complex128), 1 if ntype == 1 else -1, idx)
    err = np.linalg.norm(out.ravel()[idx] - d) / np.linalg.norm(d)
    assert err <= tol, (err, tol, info["ns"])
    # the same algorithm as the oracle at that width
    ref = NC.oracle_nufft(ntype, modes, p64, data.astype(np.complex128), tol, single,
                          ns=info["ns"])
    same = np.linalg.norm(out.ravel() - ref.ravel()) / np.linalg.norm(ref.ravel())
    assert same < (2e-5 if single else 1e-10), same


@pytest.mark.gpu
def test_default_rule_is_reference():
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    pts = NC.points(rng, 2, 2000, dtype=np.float32)
    c = NC.strengths(rng, 2000).astype(np.complex64)
    _, info = NC.run_gpu(1, (40, 30), pts, c, 1e-6, True)
    assert info["width_rule"] == 0
    assert info["ns"] == O.setup_spreader(1e-6, True)[1]
