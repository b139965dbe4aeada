"""Measures the error table behind the library's tolerance-meeting width rule
(test infrastructure: it runs the FP64 oracle; the library only holds the
numbers it prints, in csrc/planner.cpp).

For each upsampling factor (2 and 1.25), dimension and kernel width ns it
runs the oracle's type-1 and type-2 transforms on uniform random points in
[-pi, pi)^d with complex N(0,1) data against FP64 direct sums, over two mode
shapes and three seeds per dimension, and prints the worst relative l2 error
divided by the reference's own accuracy model for that width: 10^(1-ns) at
upsampfac 2 (one digit per unit of width), exp(-pi ns sqrt(1 - 1/upsampfac))
otherwise (contrib/spreadinterp.cpp:42-44):

    python oracle/width_table.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:] = [q for q in sys.path if os.path.abspath(q or ".") != _HERE]
sys.path.insert(0, os.path.dirname(_HERE))
from oracle import oracle as O  # noqa: E402

CASES = {1: [(2000,), (777,)], 2: [(100, 90), (64, 130)], 3: [(24, 20, 22), (30, 16, 18)]}
M = 20000


def worst_error(dim: int, ns: int, upsampfac: float) -> float:
    worst = 0.0
    for seed in range(3):
        rng = np.random.default_rng(1000 * ns + 10 * dim + seed + int(100000 * (2 - upsampfac)))
        for modes in CASES[dim]:
            for ntype in (1, 2):
                plan = O.OraclePlan(ntype, modes, 1 if ntype == 1 else -1, 0.0, False,
                                    upsampfac=upsampfac, ns=ns)
                pts = [rng.uniform(-np.pi, np.pi, M) for _ in range(dim)]
                args = pts + [None] * (3 - dim)
                if ntype == 1:
                    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
                    out = plan.execute(*pts, data=c).ravel()
                    idx = rng.choice(out.size, min(out.size, 600), replace=False)
                    ref = O.direct_type1(*args, c, modes, 1, idx)
                else:
                    n = int(np.prod(modes))
                    fk = rng.standard_normal(n) + 1j * rng.standard_normal(n)
                    out = plan.execute(*pts, data=fk).ravel()
                    idx = rng.choice(M, min(M, 600), replace=False)
                    ref = O.direct_type2(*args, fk, modes, -1, idx)
                worst = max(worst, O.rel_l2(out[idx], ref))
    return worst


def model(ns: int, upsampfac: float) -> float:
    if upsampfac == 2.0:
        return 10.0 ** (1 - ns)
    return float(np.exp(-np.pi * ns * np.sqrt(1.0 - 1.0 / upsampfac)))


def main() -> None:
    for usf in (2.0, 1.25):
        print(f"// upsampfac {usf}: worst rel-l2 / model, rows ns = 2..16, columns dim 1..3")
        for ns in range(2, 17):
            r = [worst_error(d, ns, usf) / model(ns, usf) for d in (1, 2, 3)]
            print("    {" + ", ".join(f"{x:.3g}" for x in r) + f"}},  // ns {ns}", flush=True)


if __name__ == "__main__":
    main()
