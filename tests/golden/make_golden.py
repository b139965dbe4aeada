"""Regenerate the golden fixtures in this folder from the reference's own code.

The reference (cuFINUFFT v1.3) ships no stored known-answer vectors; its
tests compare single modes against ad-hoc direct sums.  These fixtures are
produced by running the reference's own host-side helpers, compiled from its
sources by ``oracle/Makefile`` (target ``ref``) into
``oracle/_ref/libref_contrib.so``:

* spreader parameters (ns, beta, c, warning flag) from ``setup_spreader``
  (contrib/spreadinterp.cpp:6-67), FP32 and FP64 builds;
* fine-grid sizes from ``SET_NF_TYPE12`` (contrib/common.cpp:24-37);
* kernel Fourier-series samples from ``onedim_fseries_kernel``
  (contrib/common.cpp:39-124), FP64 build (and FP32 build for reference);
* ES kernel values from ``evaluate_kernel`` (contrib/spreadinterp.cpp:69-81);
* 2D direct sums from ``dirft2d1``/``dirft2d2`` (contrib/dirft2d.cpp:7-64).

Run from the repository root, where the reference tree is present:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libref_contrib.so")

TOLS = [1e-1, 1e-2, 1e-3, 1e-4, 3e-5, 1e-5, 1e-6, 5e-7, 1e-7, 2e-8, 1e-8, 1e-9, 1e-10,
        1e-11, 1e-12, 1e-13, 1e-14, 1e-15, 1e-16, 1e-17]
NF_MODES = [1, 2, 3, 7, 10, 16, 17, 64, 100, 128, 255, 256, 500, 512, 1000, 1024, 1536, 2047, 4096]

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)


def _lib():
    L = ctypes.CDLL(REFLIB)
    for s in ("d", "f"):
        getattr(L, f"ref_setup_spreader_{s}").argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                          _i, _d, _d]
        getattr(L, f"ref_set_nf_{s}").argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        getattr(L, f"ref_fseries_{s}").argtypes = [ctypes.c_int, ctypes.c_double, _d]
        getattr(L, f"ref_evaluate_kernel_{s}").argtypes = [ctypes.c_double, ctypes.c_double]
        getattr(L, f"ref_evaluate_kernel_{s}").restype = ctypes.c_double
        getattr(L, f"ref_dirft2d1_{s}").argtypes = [ctypes.c_int, _d, _d, _d, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_int, _d]
        getattr(L, f"ref_dirft2d2_{s}").argtypes = [ctypes.c_int, _d, _d, _d, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_int, _d]
    return L


def _p(a):
    return a.ctypes.data_as(_d)


def main() -> None:
    L = _lib()
    params = []
    for prec in ("f", "d"):
        for tol in TOLS:
            ns, beta, c = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
            ier = getattr(L, f"ref_setup_spreader_{prec}")(tol, 2.0, 0, ctypes.byref(ns), ctypes.byref(beta),
                                                           ctypes.byref(c))
            params.append({"prec": prec, "tol": tol, "ier": ier, "ns": ns.value, "beta": beta.value,
                           "c": c.value})
    nfs = []
    for prec in ("f", "d"):
        for tol in (1e-3, 1e-6, 1e-9):
            for ms in NF_MODES:
                for method, bs in ((1, 1), (2, 1), (4, 8), (4, 16)):
                    nf = getattr(L, f"ref_set_nf_{prec}")(ms, tol, method, bs)
                    nfs.append({"prec": prec, "tol": tol, "ms": ms, "method": method, "bs": bs, "nf": nf})
    with open(os.path.join(HERE, "spreader_params.json"), "w") as fh:
        json.dump({"setup_spreader": params, "set_nf_type12": nfs}, fh, indent=0)

    fs = {}
    for prec in ("d", "f"):
        for nf in (16, 64, 200, 512, 2048):
            for tol in ((1e-3, 1e-6, 1e-9, 1e-12) if prec == "d" else (1e-3, 1e-5, 1e-6)):
                out = np.zeros(nf // 2 + 1)
                getattr(L, f"ref_fseries_{prec}")(nf, tol, _p(out))
                fs[f"{prec}_nf{nf}_tol{tol:g}"] = out
    ker = []
    for prec in ("d", "f"):
        for tol in (1e-3, 1e-6, 1e-9):
            for x in np.linspace(-8.5, 8.5, 69):
                ker.append([0 if prec == "d" else 1, tol, x,
                            getattr(L, f"ref_evaluate_kernel_{prec}")(float(x), tol)])
    fs["evaluate_kernel"] = np.array(ker)

    rng = np.random.default_rng(20260301)
    M, ms, mt = 60, 12, 9
    x = rng.uniform(-np.pi, np.pi, M)
    y = rng.uniform(-np.pi, np.pi, M)
    c = rng.standard_normal(2 * M)
    fk = rng.standard_normal(2 * ms * mt)
    for iflag in (1, -1):
        f1 = np.zeros(2 * ms * mt)
        L.ref_dirft2d1_d(M, _p(x), _p(y), _p(c), iflag, ms, mt, _p(f1))
        c2 = np.zeros(2 * M)
        L.ref_dirft2d2_d(M, _p(x), _p(y), _p(c2), iflag, ms, mt, _p(fk))
        fs[f"dirft2d1_iflag{iflag}"] = f1
        fs[f"dirft2d2_iflag{iflag}"] = c2
    fs["dirft2d_x"] = x
    fs["dirft2d_y"] = y
    fs["dirft2d_c"] = c
    fs["dirft2d_fk"] = fk
    fs["dirft2d_shape"] = np.array([M, ms, mt])
    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **fs)
    print("wrote", len(params), "spreader cases,", len(nfs), "nf cases,", len(fs), "arrays")


if __name__ == "__main__":
    main()
