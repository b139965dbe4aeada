"""High-level Python interface, mirroring the reference's ``cufinufft`` class
(python/cufinufft/cufinufft.py:34-267 of cuFINUFFT v1.3): same constructor
arguments, ``set_pts``/``execute`` methods, error types and messages.

Arrays are device arrays that expose either ``.ptr`` and ``.dtype`` (the
pycuda ``GPUArray`` protocol the reference uses) or a CUDA ``torch.Tensor``
(contiguous).  Shapes follow the reference: ``modes`` is given C-ordered
(..., nY, nX) and reversed for the library; 2D points are passed as
(kx, ky) for axes (0, 1) of the C-ordered mode array.
"""
from __future__ import annotations

import atexit
import ctypes
import sys
from ctypes import byref, c_int, c_void_p

import numpy as np

from cufinufft_gb300._cufinufft import (NufftOpts, PlanInfo, _default_opts, _destroy_plan,
                                        _destroy_planf, _exec_plan, _exec_planf, _get_info,
                                        _get_infof, _make_plan, _make_planf, _set_pts, _set_ptsf,
                                        _set_stream, _set_streamf, _set_timing, _set_timingf,
                                        _set_width_rule, _stage_times, _stage_timesf)

# If Python is shutting down, __del__ does nothing (as in the reference).
exiting = False
atexit.register(setattr, sys.modules[__name__], 'exiting', True)

_TORCH_TO_NP = {}


def _np_dtype(a):
    dt = getattr(a, "dtype", None)
    if dt is None:
        raise TypeError("array has no dtype")
    if isinstance(dt, np.dtype):
        return dt
    try:
        return np.dtype(dt)
    except TypeError:
        pass
    if not _TORCH_TO_NP:
        import torch
        _TORCH_TO_NP.update({torch.float32: np.dtype(np.float32), torch.float64: np.dtype(np.float64),
                             torch.complex64: np.dtype(np.complex64),
                             torch.complex128: np.dtype(np.complex128)})
    if dt in _TORCH_TO_NP:
        return _TORCH_TO_NP[dt]
    raise TypeError(f"unsupported dtype {dt}")


def _ptr(a) -> int:
    if hasattr(a, "ptr"):
        return int(a.ptr)
    if hasattr(a, "data_ptr"):
        if not getattr(a, "is_cuda", False):
            raise TypeError("cufinufft expects device (CUDA) arrays")
        if not a.is_contiguous():
            raise TypeError("cufinufft expects contiguous arrays")
        return int(a.data_ptr())
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        return int(cai["data"][0])
    raise TypeError("cufinufft expects device arrays exposing .ptr or a CUDA tensor")


def _size(a) -> int:
    if hasattr(a, "numel"):
        return int(a.numel())
    s = a.size
    return int(s() if callable(s) else s)


class cufinufft:
    """A type-1 or type-2 NUFFT plan on one GPU.

    :param nufft_type: 1, 2 or 3 (type 3: nonuniform points to nonuniform
        frequencies, which the reference reserves without implementing).
    :param modes: C-ordered shape of the mode array, 1 to 3 dimensions (for
        type 3 only its length, the dimension, is used).
    :param n_trans: number of transforms per execute.
    :param eps: requested relative tolerance.
    :param isign: sign of the exponent; default +1 for type 1, -1 for type 2.
    :param dtype: np.float32 or np.float64 (selects the FP32/FP64 library).
    :param kwargs: fields of the options struct (e.g. gpu_method=2), and the
        extension ``width_rule``: "reference" (the default: the reference's
        kernel width for eps) or "tol" (the narrowest width whose measured
        error meets eps; see cufinufft_set_width_rule).
    """

    def __init__(self, nufft_type, modes, n_trans=1, eps=1e-6, isign=None, dtype=np.float32,
                 **kwargs):
        if isign is None:
            isign = -1 if nufft_type == 2 else +1
        self.plan = None
        self.dtype = np.dtype(dtype)
        if self.dtype == np.float64:
            self._make_plan = _make_plan
            self._set_pts = _set_pts
            self._exec_plan = _exec_plan
            self._destroy_plan = _destroy_plan
            self._set_stream = _set_stream
            self._get_info = _get_info
            self._set_timing = _set_timing
            self._stage_times = _stage_times
            self.complex_dtype = np.dtype(np.complex128)
        elif self.dtype == np.float32:
            self._make_plan = _make_planf
            self._set_pts = _set_ptsf
            self._exec_plan = _exec_planf
            self._destroy_plan = _destroy_planf
            self._set_stream = _set_streamf
            self._get_info = _get_infof
            self._set_timing = _set_timingf
            self._stage_times = _stage_timesf
            self.complex_dtype = np.dtype(np.complex64)
        else:
            raise TypeError("Expected np.float32 or np.float64.")

        self.dim = len(modes)
        self._finufft_type = nufft_type
        self.isign = isign
        self.eps = float(eps)
        self.n_trans = n_trans
        self._maxbatch = kwargs.pop("maxbatchsize", 1)
        rule = kwargs.pop("width_rule", None)
        if rule not in (None, "reference", "tol", 0, 1):
            raise TypeError(f"Invalid width_rule '{rule}'")
        self._width_rule = None if rule is None else (1 if rule in ("tol", 1) else 0)

        modes = tuple(modes)[::-1] + (1,) * (3 - self.dim)
        self.modes = (c_int * 3)(*modes)
        self.opts = self._default_opts(nufft_type, self.dim)
        field_names = [name for name, _ in self.opts._fields_]
        for k, v in kwargs.items():
            if k in field_names:
                setattr(self.opts, k, v)
            else:
                raise TypeError(f"Invalid option '{k}'")
        self._plan()
        self.references = []

    @staticmethod
    def _default_opts(nufft_type, dim):
        nufft_opts = NufftOpts()
        ier = _default_opts(nufft_type, dim, nufft_opts)
        if ier != 0:
            raise RuntimeError('Configuration not yet implemented.')
        return nufft_opts

    def _plan(self):
        self.plan = c_void_p(None)
        prev = c_int(-1)
        if self._width_rule is not None:
            _set_width_rule(self._width_rule, byref(prev))
        try:
            ier = self._make_plan(self._finufft_type, self.dim, self.modes, self.isign,
                                  self.n_trans, self.eps, self._maxbatch, byref(self.plan),
                                  self.opts)
        finally:
            if self._width_rule is not None:
                _set_width_rule(prev.value, None)
        if ier != 0:
            raise RuntimeError('Error creating plan.')

    def set_pts(self, kx, ky=None, kz=None, s=None, t=None, u=None):
        """Set the nonuniform points (device arrays of the plan's real dtype);
        type 3 also takes its target frequencies s (t, u in 2D/3D), in the
        same C-ordered axis convention as the points."""
        if _np_dtype(kx) != self.dtype:
            raise TypeError("cufinufft plan.dtype and kx dtypes do not match.")
        if ky is not None and _np_dtype(ky) != self.dtype:
            raise TypeError("cufinufft plan.dtype and ky dtypes do not match.")
        if kz is not None and _np_dtype(kz) != self.dtype:
            raise TypeError("cufinufft plan.dtype and kz dtypes do not match.")
        M = _size(kx)
        if ky is not None and _size(ky) != M:
            raise TypeError("Number of elements in kx and ky must be equal")
        if kz is not None and _size(kz) != M:
            raise TypeError("Number of elements in kx and kz must be equal")
        # library axis order is (x fastest): (x,) ; (y, x) ; (z, y, x)
        fpts_axes = [_ptr(kx), None, None]
        self.references.append(kx)
        if ky is not None:
            fpts_axes.insert(0, _ptr(ky))
            self.references.append(ky)
        if kz is not None:
            fpts_axes.insert(0, _ptr(kz))
            self.references.append(kz)
        N, tgt = 0, [None, None, None]
        if self._finufft_type == 3:
            if s is None:
                raise TypeError("type 3 needs target frequencies s (t, u)")
            freqs = [f for f in (s, t, u) if f is not None]
            if len(freqs) != self.dim:
                raise TypeError("type 3 needs one frequency array per dimension")
            for f in freqs:
                if _np_dtype(f) != self.dtype:
                    raise TypeError("cufinufft plan.dtype and frequency dtypes do not match.")
            N = _size(freqs[0])
            if any(_size(f) != N for f in freqs):
                raise TypeError("Number of elements in s, t, u must be equal")
            # library axis order: the last C-ordered axis is x
            real_p = ctypes.POINTER(ctypes.c_double if self.dtype == np.float64 else ctypes.c_float)
            tgt = [ctypes.cast(c_void_p(_ptr(f)), real_p) for f in freqs[::-1]] + [None] * (3 - self.dim)
            self.references.extend(freqs)
        ier = self._set_pts(M, *fpts_axes[:3], N, *tgt, self.plan)
        if ier != 0:
            raise RuntimeError('Error setting non-uniform points.')

    def execute(self, c, fk):
        """Type 1: c -> fk.  Type 2: fk -> c.  Queued asynchronously on the
        plan's stream (ordered with the default stream)."""
        if not (_np_dtype(c) == _np_dtype(fk) == self.complex_dtype):
            raise TypeError("cufinufft execute expects {} dtype arguments "
                            "for this plan. Check plan and arguments.".format(self.complex_dtype))
        ier = self._exec_plan(_ptr(c), _ptr(fk), self.plan)
        if ier != 0:
            raise RuntimeError('Error executing plan.')

    # ---- extensions -----------------------------------------------------
    def set_stream(self, stream) -> None:
        """Queue later work on ``stream`` (a raw handle, a torch.cuda.Stream or
        None for the plan's own stream)."""
        handle = getattr(stream, "cuda_stream", stream)
        ier = self._set_stream(self.plan, c_void_p(handle or None))
        if ier != 0:
            raise RuntimeError('Error setting stream.')

    def set_timing(self, on: bool = True) -> None:
        """Record CUDA events around each stage of later executes."""
        if self._set_timing(self.plan, int(bool(on))) != 0:
            raise RuntimeError('Error setting timing.')

    def stage_times(self, reset: bool = False) -> dict:
        """Accumulated device milliseconds per stage since the last reset:
        'spreadinterp' (spread or interp kernel), 'fft', 'deconv' (deconvolve
        or amplify), and the number of batches timed."""
        ms = (ctypes.c_double * 3)()
        nb = ctypes.c_longlong()
        if self._stage_times(self.plan, ms, ctypes.byref(nb), int(bool(reset))) != 0:
            raise RuntimeError('Error reading stage times.')
        return {"spreadinterp": ms[0], "fft": ms[1], "deconv": ms[2], "batches": nb.value}

    def set_layout(self, method, binsize, maxsubprobsize=1024) -> None:
        """Re-sort the points for another method (1, 2, or 5: type-1
        cell-run spread), bin size (tuple in the library's x, y, z order) and
        subproblem cap; results unchanged."""
        from cufinufft_gb300._cufinufft import _set_layout, _set_layoutf
        fn = _set_layout if self.dtype == np.float64 else _set_layoutf
        b = tuple(binsize) + (1,) * (3 - len(binsize))
        ier = fn(self.plan, int(method), int(b[0]), int(b[1]), int(b[2]), int(maxsubprobsize))
        if ier != 0:
            raise RuntimeError(f'Error setting layout ({ier}).')

    def autotune(self) -> list:
        """Time candidate layouts on this plan's points and keep the fastest.
        Returns the chosen entry followed by every candidate tried."""
        from cufinufft_gb300._cufinufft import TuneEntry, _autotune, _autotunef
        fn = _autotune if self.dtype == np.float64 else _autotunef
        buf = (TuneEntry * 64)()
        n = ctypes.c_int(0)
        ier = fn(self.plan, buf, 64, ctypes.byref(n))
        if ier != 0:
            raise RuntimeError(f'Error autotuning ({ier}).')
        return [{f: getattr(buf[i], f) for f, _ in TuneEntry._fields_} for i in range(n.value)]

    def features(self) -> np.ndarray:
        """The layout-independent plan features the learned selector reads
        (14 floats, computed from the points' occupancy of the fine grid)."""
        from cufinufft_gb300._cufinufft import MLP_FEATURES, _features, _featuresf
        fn = _features if self.dtype == np.float64 else _featuresf
        f = np.zeros(MLP_FEATURES, dtype=np.float32)
        ier = fn(self.plan, f.ctypes.data)
        if ier != 0:
            raise RuntimeError(f'Error computing features ({ier}).')
        return f

    def set_layout_class(self, cls: int) -> None:
        """Re-sort the points into one of the twelve layout classes (the
        selector's and autotuner's candidates)."""
        from cufinufft_gb300._cufinufft import _set_layout_class, _set_layout_classf
        fn = _set_layout_class if self.dtype == np.float64 else _set_layout_classf
        ier = fn(self.plan, int(cls))
        if ier != 0:
            raise RuntimeError(f'Error setting layout class ({ier}).')

    def info(self) -> dict:
        """Plan facts: fine grid, kernel width, method run, bins."""
        inf = PlanInfo()
        if self._get_info(self.plan, ctypes.byref(inf)) != 0:
            raise RuntimeError('Error reading plan info.')
        return {name: getattr(inf, name) for name, _ in inf._fields_}

    def __del__(self):
        if exiting or self.plan is None or not self.plan.value:
            return
        ier = self._destroy_plan(self.plan)
        if ier != 0:
            raise RuntimeError('Error destroying plan.')
        self.plan = None
        self.references = []


class cufinufft_batch:
    """Many plans of one type, dimension, dtype and tolerance-derived kernel
    width executed together (an extension with no counterpart in the
    reference).  ``plans`` are ``cufinufft`` objects whose points are set;
    they must stay alive, with their points, as long as the batch.
    ``execute(c_list, fk_list)`` takes one (c, fk) pair per plan, as that
    plan's ``execute`` would, and runs all of them in one CUDA-graph replay."""

    def __init__(self, plans):
        from cufinufft_gb300._cufinufft import (_batch_destroy, _batch_destroyf, _batch_execute,
                                                _batch_executef, _batch_make, _batch_makef)
        self.batch = None
        self.plans = list(plans)
        if not self.plans:
            raise ValueError("a batch needs at least one plan")
        dt = self.plans[0].dtype
        if any(p.dtype != dt for p in self.plans):
            raise TypeError("all plans of a batch must share one dtype")
        self.dtype = dt
        self.complex_dtype = self.plans[0].complex_dtype
        make = _batch_make if dt == np.float64 else _batch_makef
        self._exec = _batch_execute if dt == np.float64 else _batch_executef
        self._destroy = _batch_destroy if dt == np.float64 else _batch_destroyf
        arr = (c_void_p * len(self.plans))(*[p.plan.value for p in self.plans])
        self.batch = c_void_p(None)
        ier = make(len(self.plans), arr, byref(self.batch))
        if ier != 0:
            self.batch = None
            raise RuntimeError(f'Error creating batch ({ier}).')

    def execute(self, c_list, fk_list):
        n = len(self.plans)
        if len(c_list) != n or len(fk_list) != n:
            raise TypeError("execute expects one c and one fk per plan")
        for c, fk in zip(c_list, fk_list):
            if not (_np_dtype(c) == _np_dtype(fk) == self.complex_dtype):
                raise TypeError("cufinufft batch execute expects {} arrays".format(self.complex_dtype))
        cs = (c_void_p * n)(*[_ptr(c) for c in c_list])
        fks = (c_void_p * n)(*[_ptr(f) for f in fk_list])
        ier = self._exec(self.batch, cs, fks)
        if ier != 0:
            raise RuntimeError(f'Error executing batch ({ier}).')

    def __del__(self):
        if exiting or self.batch is None or not self.batch.value:
            return
        self._destroy(self.batch)
        self.batch = None
