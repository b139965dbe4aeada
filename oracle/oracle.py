"""CPU oracle for the type-1/type-2 NUFFT path (test infrastructure only).

This module drives ``liboracle.so`` (the FP64 C restatement in
``nufft_oracle.c``) and numpy's FFT to compute, on the host, what the
reference cuFINUFFT v1.3 pipeline computes:

    type 1:  spread (src/2d/spreadinterp2d.cu:16-57) -> FFT
             (src/2d/cufinufft2d.cu:73) -> deconvolve
             (src/deconvolve_wrapper.cu:26-42)
    type 2:  amplify (src/deconvolve_wrapper.cu:82-98) -> FFT
             (src/2d/cufinufft2d.cu:141) -> interpolate
             (src/2d/spreadinterp2d.cu:516-553)

and FP64 direct sums on subsets of modes/targets (contrib/dirft2d.cpp:7-64).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU baseline
leg and its ``--impl reference`` arm) may import this module.  The product
path never calls it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()

_d_p = ctypes.POINTER(ctypes.c_double)
_f_p = ctypes.POINTER(ctypes.c_float)
_ll_p = ctypes.POINTER(ctypes.c_longlong)
_i_p = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile ``oracle/liboracle.so`` with gcc (plain C99 + OpenMP)."""
    path = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "nufft_oracle.c")
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return path


def lib() -> ctypes.CDLL:
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = build()
            L = ctypes.CDLL(path)
            L.orc_setup_spreader.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_int, _i_p, _d_p, _d_p]
            L.orc_setup_spreader.restype = ctypes.c_int
            L.orc_es_kernel.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double]
            L.orc_es_kernel.restype = ctypes.c_double
            L.orc_next235beven.argtypes = [ctypes.c_int, ctypes.c_int]
            L.orc_next235beven.restype = ctypes.c_int
            L.orc_set_nf_type12.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int]
            L.orc_set_nf_type12.restype = ctypes.c_int
            L.orc_gauss_legendre.argtypes = [ctypes.c_int, _d_p, _d_p]
            L.orc_fseries.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _d_p]
            L.orc_spread.argtypes = [ctypes.c_int] * 5 + [_d_p] * 3 + [ctypes.c_int, _d_p, _d_p,
                                                                      ctypes.c_int, ctypes.c_double,
                                                                      ctypes.c_double]
            L.orc_interp.argtypes = L.orc_spread.argtypes
            L.orc_deconvolve.argtypes = [ctypes.c_int] * 9 + [_d_p, _d_p, _d_p, _d_p, _d_p]
            L.orc_dirft_type1.argtypes = [ctypes.c_int] * 5 + [_d_p] * 4 + [ctypes.c_int, ctypes.c_int,
                                                                             _ll_p, _d_p]
            L.orc_dirft_type2.argtypes = [ctypes.c_int] * 4 + [_d_p] * 4 + [ctypes.c_int, ctypes.c_int,
                                                                             _ll_p, _d_p]
            L.orc_dirft_type3.argtypes = [ctypes.c_int, ctypes.c_int] + [_d_p] * 7 + [
                ctypes.c_int, ctypes.c_int, _ll_p, _d_p]
            # FP32-arithmetic stages (the CPU timing of FP32 workloads)
            L.orc_spread_f32.argtypes = [ctypes.c_int] * 5 + [_f_p] * 3 + [ctypes.c_int, _f_p, _f_p,
                                                                          ctypes.c_int, ctypes.c_double,
                                                                          ctypes.c_double]
            L.orc_interp_f32.argtypes = L.orc_spread_f32.argtypes
            L.orc_deconvolve_f32.argtypes = [ctypes.c_int] * 9 + [_f_p, _f_p, _d_p, _d_p, _d_p]
            L.orc_num_threads.restype = ctypes.c_int
            L.orc_set_num_threads.argtypes = [ctypes.c_int]
            _LIB = L
    return _LIB


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_d_p)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def setup_spreader(tol: float, single: bool, upsampfac: float = 2.0, kerevalmeth: int = 0):
    """(ier, ns, beta, c) as contrib/spreadinterp.cpp:6-67 sets them."""
    ns = ctypes.c_int()
    beta = ctypes.c_double()
    c = ctypes.c_double()
    ier = lib().orc_setup_spreader(float(tol), float(upsampfac), int(kerevalmeth), int(bool(single)),
                                   ctypes.byref(ns), ctypes.byref(beta), ctypes.byref(c))
    return ier, ns.value, beta.value, c.value


def es_kernel(x: float, ns: int, beta: float, c: float) -> float:
    return lib().orc_es_kernel(float(x), int(ns), float(beta), float(c))


def next235beven(n: int, b: int = 1) -> int:
    return lib().orc_next235beven(int(n), int(b))


def set_nf_type12(ms: int, ns: int, gpu_method: int = 1, bs: int = 1, upsampfac: float = 2.0) -> int:
    return lib().orc_set_nf_type12(int(ms), float(upsampfac), int(ns), int(gpu_method), int(bs))


def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauss_legendre(int(n), _dp(x), _dp(w))
    return x, w


def fseries(nf: int, ns: int, beta: float, c: float) -> np.ndarray:
    out = np.zeros(nf // 2 + 1)
    lib().orc_fseries(int(nf), int(ns), float(beta), float(c), _dp(out))
    return out


def tol_for_width(ns: int, upsampfac: float = 2.0) -> float:
    """A tolerance for which setup_spreader (contrib/spreadinterp.cpp:29-45)
    chooses kernel width ns: ns = ceil(-log10(tol/10)) at upsampfac 2,
    ceil(-ln(tol) / (pi sqrt(1 - 1/upsampfac))) otherwise."""
    if upsampfac == 2.0:
        return 1.01 * 10.0 ** (1 - ns)
    import math
    return math.exp(-(ns - 0.5) * math.pi * math.sqrt(1.0 - 1.0 / upsampfac))


class OraclePlan:
    """FP64 restatement of a cuFINUFFT type-1/2 plan (test infrastructure).

    ``modes`` is (N1,), (N1, N2) or (N1, N2, N3) with N1 the fastest index,
    as in cufinufft_makeplan's nmodes (src/cufinufft.cu:78).  ``single``
    selects the spreader parameters of the FP32 build (ns, beta, c as the
    reference's SINGLE build computes them); the arithmetic is FP64 always.
    """

    def __init__(self, nufft_type: int, modes, iflag: int, tol: float, single: bool,
                 gpu_method: int = 0, obin: tuple = (8, 8, 8), spreadinterponly: bool = False,
                 upsampfac: float = 2.0, ns: int | None = None, fp32_arith: bool = False):
        # fp32_arith: spread, interpolation, FFT and deconvolution in FP32
        # (the CPU form of the reference's FP32 build, for timing FP32
        # workloads); the default is FP64 arithmetic, the accuracy oracle
        self.fp32 = bool(fp32_arith)
        self.type = int(nufft_type)
        self.modes = tuple(int(m) for m in modes)
        self.dim = len(self.modes)
        self.iflag = 1 if iflag >= 0 else -1
        self.upsampfac = float(upsampfac)
        if ns is not None:
            # a given kernel width (a plan made under another width rule):
            # the same shape formulas at that width
            tol = tol_for_width(int(ns), self.upsampfac)
        ier, self.ns, self.beta, self.c = setup_spreader(tol, single, self.upsampfac)
        if ier > 1:
            raise ValueError(f"setup_spreader error {ier}")
        if ns is not None and self.ns != int(ns):
            raise ValueError(f"width {ns} not reachable ({self.ns})")
        if spreadinterponly:
            # the grid is the modes array itself (the reference's spread /
            # interp tests set gpu_spreadinterponly and pass nf directly,
            # test/spread2d_test.cu:80,133)
            self.nf = self.modes
        else:
            self.nf = tuple(set_nf_type12(m, self.ns, gpu_method, obin[d], self.upsampfac)
                            for d, m in enumerate(self.modes))
        self.ker = [fseries(nf, self.ns, self.beta, self.c) for nf in self.nf]

    def _pts(self, x, y, z):
        rd = np.float32 if self.fp32 else np.float64
        cv = (lambda a: np.ascontiguousarray(np.asarray(a, dtype=rd)))
        pts = [cv(x)]
        M = pts[0].size
        dummy = np.zeros(max(M, 1), dtype=rd)
        pts.append(cv(y) if self.dim > 1 else dummy)
        pts.append(cv(z) if self.dim > 2 else dummy)
        return M, pts

    def _cplx(self, a) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(a, dtype=np.complex64 if self.fp32 else np.complex128))

    def _nf3(self):
        nf = list(self.nf) + [1] * (3 - self.dim)
        return nf

    def _modes3(self):
        return list(self.modes) + [1] * (3 - self.dim)

    fft_workers = 0  # > 0: scipy.fft with that many threads (CPU baseline timing)

    def _fft(self, fw: np.ndarray) -> np.ndarray:
        axes = tuple(range(-self.dim, 0))
        # cuFFT's CUFFT_INVERSE (iflag>=0) is the unnormalised +i transform.
        if self.fft_workers > 0:
            import scipy.fft as sf
            if self.iflag > 0:
                return sf.ifftn(fw, axes=axes, norm="forward", workers=self.fft_workers,
                                overwrite_x=True)
            return sf.fftn(fw, axes=axes, workers=self.fft_workers, overwrite_x=True)
        if self.iflag > 0:
            return np.fft.ifftn(fw, axes=axes, norm="forward")
        return np.fft.fftn(fw, axes=axes)

    def _stage(self, name):
        # (C function, real view, pointer cast) of the plan's arithmetic
        if self.fp32:
            return getattr(lib(), name + "_f32"), np.float32, _fp
        return getattr(lib(), name), np.float64, _dp

    def spread(self, x, y, z, c, ntr: int = 1) -> np.ndarray:
        M, (px, py, pz) = self._pts(x, y, z)
        nf = self._nf3()
        cc = self._cplx(c).reshape(ntr, M)
        fw = np.zeros((ntr, nf[2], nf[1], nf[0]), dtype=cc.dtype)
        fn, rv, pp = self._stage("orc_spread")
        fn(self.dim, nf[0], nf[1], nf[2], M, pp(px), pp(py), pp(pz), ntr, pp(cc.view(rv)),
           pp(fw.view(rv)), self.ns, self.beta, self.c)
        return fw

    def interp(self, x, y, z, fw: np.ndarray, ntr: int = 1) -> np.ndarray:
        M, (px, py, pz) = self._pts(x, y, z)
        nf = self._nf3()
        g = self._cplx(fw).reshape(ntr, nf[2], nf[1], nf[0])
        c = np.zeros((ntr, M), dtype=g.dtype)
        fn, rv, pp = self._stage("orc_interp")
        fn(self.dim, nf[0], nf[1], nf[2], M, pp(px), pp(py), pp(pz), ntr, pp(c.view(rv)),
           pp(g.view(rv)), self.ns, self.beta, self.c)
        return c

    def _deconv(self, direction: int, fw: np.ndarray, fk: np.ndarray, ntr: int):
        nf = self._nf3()
        N = self._modes3()
        kers = [self.ker[d] if d < self.dim else np.ones(1) for d in range(3)]
        fn, rv, pp = self._stage("orc_deconvolve")
        fn(direction, self.dim, N[0], N[1], N[2], nf[0], nf[1], nf[2], ntr, pp(fw.view(rv)),
           pp(fk.view(rv)), _dp(kers[0]), _dp(kers[1]), _dp(kers[2]))

    def execute(self, x, y=None, z=None, data=None, ntr: int = 1) -> np.ndarray:
        """Type 1: data = c (ntr*M) -> fk (ntr, N3, N2, N1).  Type 2: data = fk
        (ntr*N) -> c (ntr, M)."""
        N = self._modes3()
        cdt = np.complex64 if self.fp32 else np.complex128
        if self.type == 1:
            fw = self.spread(x, y, z, data, ntr)
            fw = np.ascontiguousarray(self._fft(fw), dtype=cdt)
            fk = np.zeros((ntr, N[2], N[1], N[0]), dtype=cdt)
            self._deconv(1, fw, fk, ntr)
            return fk
        nf = self._nf3()
        fk = self._cplx(data).reshape(ntr, N[2], N[1], N[0]).copy()
        fw = np.zeros((ntr, nf[2], nf[1], nf[0]), dtype=cdt)
        self._deconv(2, fw, fk, ntr)
        fw = np.ascontiguousarray(self._fft(fw), dtype=cdt)
        return self.interp(x, y, z, fw, ntr)


def direct_type1(x, y, z, c, modes, iflag: int, mode_idx) -> np.ndarray:
    """FP64 direct sum f[m] = sum_j c_j exp(i sgn k(m).x_j) at flat CMCL mode
    indices ``mode_idx`` (k1 fastest)."""
    modes = tuple(int(m) for m in modes)
    dim = len(modes)
    N = list(modes) + [1] * (3 - dim)
    px = _f64(x)
    M = px.size
    dummy = np.zeros(max(M, 1))
    py = _f64(y) if dim > 1 else dummy
    pz = _f64(z) if dim > 2 else dummy
    cc = _c128(c).reshape(M)
    idx = np.ascontiguousarray(np.asarray(mode_idx, dtype=np.int64))
    out = np.zeros(idx.size, dtype=np.complex128)
    lib().orc_dirft_type1(dim, N[0], N[1], N[2], M, _dp(px), _dp(py), _dp(pz),
                          _dp(cc.view(np.float64)), int(iflag), idx.size,
                          idx.ctypes.data_as(_ll_p), _dp(out.view(np.float64)))
    return out


def direct_type2(x, y, z, fk, modes, iflag: int, target_idx) -> np.ndarray:
    """FP64 direct sum c[j] = sum_k fk[k] exp(i sgn k.x_j) at targets
    ``target_idx``; fk flat in CMCL order (k1 fastest)."""
    modes = tuple(int(m) for m in modes)
    dim = len(modes)
    N = list(modes) + [1] * (3 - dim)
    px = _f64(x)
    M = px.size
    dummy = np.zeros(max(M, 1))
    py = _f64(y) if dim > 1 else dummy
    pz = _f64(z) if dim > 2 else dummy
    f = _c128(fk).reshape(-1)
    idx = np.ascontiguousarray(np.asarray(target_idx, dtype=np.int64))
    out = np.zeros(idx.size, dtype=np.complex128)
    lib().orc_dirft_type2(dim, N[0], N[1], N[2], _dp(px), _dp(py), _dp(pz),
                          _dp(f.view(np.float64)), int(iflag), idx.size,
                          idx.ctypes.data_as(_ll_p), _dp(out.view(np.float64)))
    return out


def rel_l2(est, ref) -> float:
    est = np.asarray(est).ravel()
    ref = np.asarray(ref).ravel()
    return float(np.linalg.norm(est - ref) / np.linalg.norm(ref))


def direct_type3(x, y, z, c, s, t, u, iflag: int, target_idx) -> np.ndarray:
    """FP64 direct sum of the type-3 transform f_k = sum_j c_j exp(i sgn s_k.x_j)
    at targets ``target_idx`` (sources x, y, z; target frequencies s, t, u;
    unused axes None)."""
    px = _f64(x)
    M = px.size
    dim = 1 + (y is not None) + (z is not None)
    ps = _f64(s)
    dummy = np.zeros(max(M, 1))
    dummy_t = np.zeros(max(ps.size, 1))
    py = _f64(y) if y is not None else dummy
    pz = _f64(z) if z is not None else dummy
    pt = _f64(t) if t is not None else dummy_t
    pu = _f64(u) if u is not None else dummy_t
    cc = _c128(c).reshape(M)
    idx = np.ascontiguousarray(np.asarray(target_idx, dtype=np.int64))
    out = np.zeros(idx.size, dtype=np.complex128)
    lib().orc_dirft_type3(dim, M, _dp(px), _dp(py), _dp(pz), _dp(cc.view(np.float64)), _dp(ps),
                          _dp(pt), _dp(pu), int(iflag), idx.size, idx.ctypes.data_as(_ll_p),
                          _dp(out.view(np.float64)))
    return out
