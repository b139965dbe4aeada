"""Low-level ctypes bindings to the in-tree ``libcufinufft.so``.

The names, argument types and the options structure mirror the reference's
bindings (python/cufinufft/_cufinufft.py:77-153 of cuFINUFFT v1.3), so code
written against them runs unchanged.  The library is the one built in-tree by
``cufinufft_gb300.build``; importing this module raises if it is missing --
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import c_double, c_float, c_int, c_void_p

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("CUFINUFFT_LIB", os.path.join(_PKG, "lib", "libcufinufft.so"))

c_int_p = ctypes.POINTER(c_int)
c_float_p = ctypes.POINTER(c_float)
c_double_p = ctypes.POINTER(c_double)

if not os.path.exists(LIB_PATH):
    raise RuntimeError(
        f"libcufinufft.so not found at {LIB_PATH}; build it with "
        "`python -m cufinufft_gb300.build` (nvcc, sm_103a)")
lib = ctypes.CDLL(LIB_PATH)


def _get_ctypes(dtype):
    """(real ctype, pointer ctype) for np.float32 / np.float64."""
    if dtype == np.float64:
        REAL_t = c_double
    elif dtype == np.float32:
        REAL_t = c_float
    else:
        raise TypeError("Expected np.float32 or np.float64.")
    return REAL_t, ctypes.POINTER(REAL_t)


def _get_NufftOpts():
    # field order is the ABI (include/cufinufft_opts.h)
    return [
        ('upsampfac', c_double),
        ('gpu_method', c_int),
        ('gpu_sort', c_int),
        ('gpu_binsizex', c_int),
        ('gpu_binsizey', c_int),
        ('gpu_binsizez', c_int),
        ('gpu_obinsizex', c_int),
        ('gpu_obinsizey', c_int),
        ('gpu_obinsizez', c_int),
        ('gpu_maxsubprobsize', c_int),
        ('gpu_nstreams', c_int),
        ('gpu_kerevalmeth', c_int),
        ('gpu_spreadinterponly', c_int),
        ('gpu_device_id', c_int)]


class NufftOpts(ctypes.Structure):
    pass


NufftOpts._fields_ = _get_NufftOpts()


class PlanInfo(ctypes.Structure):
    """Mirror of cufinufft_plan_info (an extension: plan facts)."""
    _fields_ = [(n, c_int) for n in (
        "type", "dim", "ms", "mt", "mu", "nf1", "nf2", "nf3", "ns", "M", "ntransf",
        "maxbatchsize", "method", "sort", "binsizex", "binsizey", "binsizez", "nbins",
        "nsubprob", "kerevalmeth")] + [("beta", c_double), ("es_c", c_double)]


CufinufftPlan = c_void_p
CufinufftPlanf = c_void_p
CufinufftPlan_p = ctypes.POINTER(CufinufftPlan)
CufinufftPlanf_p = ctypes.POINTER(CufinufftPlanf)
NufftOpts_p = ctypes.POINTER(NufftOpts)

_default_opts = lib.cufinufft_default_opts
_default_opts.argtypes = [c_int, c_int, NufftOpts_p]
_default_opts.restype = c_int

_default_optsf = lib.cufinufftf_default_opts
_default_optsf.argtypes = [c_int, c_int, NufftOpts_p]
_default_optsf.restype = c_int

_make_plan = lib.cufinufft_makeplan
_make_plan.argtypes = [c_int, c_int, c_int_p, c_int, c_int, c_double, c_int, CufinufftPlan_p,
                       NufftOpts_p]
_make_plan.restype = c_int

_make_planf = lib.cufinufftf_makeplan
_make_planf.argtypes = [c_int, c_int, c_int_p, c_int, c_int, c_float, c_int, CufinufftPlanf_p,
                        NufftOpts_p]
_make_planf.restype = c_int

_set_pts = lib.cufinufft_setpts
_set_pts.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_int, c_double_p, c_double_p,
                     c_double_p, c_void_p]
_set_pts.restype = c_int

_set_ptsf = lib.cufinufftf_setpts
_set_ptsf.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_int, c_float_p, c_float_p,
                      c_float_p, c_void_p]
_set_ptsf.restype = c_int

_exec_plan = lib.cufinufft_execute
_exec_plan.argtypes = [c_void_p, c_void_p, c_void_p]
_exec_plan.restype = c_int

_exec_planf = lib.cufinufftf_execute
_exec_planf.argtypes = [c_void_p, c_void_p, c_void_p]
_exec_planf.restype = c_int

_destroy_plan = lib.cufinufft_destroy
_destroy_plan.argtypes = [c_void_p]
_destroy_plan.restype = c_int

_destroy_planf = lib.cufinufftf_destroy
_destroy_planf.argtypes = [c_void_p]
_destroy_planf.restype = c_int

# extensions
_set_stream = lib.cufinufft_set_stream
_set_stream.argtypes = [c_void_p, c_void_p]
_set_stream.restype = c_int
_set_streamf = lib.cufinufftf_set_stream
_set_streamf.argtypes = [c_void_p, c_void_p]
_set_streamf.restype = c_int
_get_info = lib.cufinufft_get_info
_get_info.argtypes = [c_void_p, ctypes.POINTER(PlanInfo)]
_get_info.restype = c_int
_get_infof = lib.cufinufftf_get_info
_get_infof.argtypes = [c_void_p, ctypes.POINTER(PlanInfo)]
_get_infof.restype = c_int
_set_timing = lib.cufinufft_set_timing
_set_timing.argtypes = [c_void_p, c_int]
_set_timing.restype = c_int
_set_timingf = lib.cufinufftf_set_timing
_set_timingf.argtypes = [c_void_p, c_int]
_set_timingf.restype = c_int
_stage_times = lib.cufinufft_stage_times
_stage_times.argtypes = [c_void_p, c_double_p, ctypes.POINTER(ctypes.c_longlong), c_int]
_stage_times.restype = c_int
_stage_timesf = lib.cufinufftf_stage_times
_stage_timesf.argtypes = [c_void_p, c_double_p, ctypes.POINTER(ctypes.c_longlong), c_int]
_stage_timesf.restype = c_int
