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
        "nsubprob", "kerevalmeth")] + [("beta", c_double), ("es_c", c_double),
                                       ("line_fft", c_int), ("cell_order", c_int),
                                       ("width_rule", c_int), ("chain_fp32", c_int),
                                       ("half_fft", c_int), ("fp64_df", c_int),
                                       ("df_fft", c_int)]


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
_set_width_rule = lib.cufinufft_set_width_rule
_set_width_rule.argtypes = [c_int, c_int_p]
_set_width_rule.restype = c_int

_batch_make = lib.cufinufft_batch_make
_batch_make.argtypes = [c_int, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p)]
_batch_make.restype = c_int
_batch_makef = lib.cufinufftf_batch_make
_batch_makef.argtypes = [c_int, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p)]
_batch_makef.restype = c_int
_batch_execute = lib.cufinufft_batch_execute
_batch_execute.argtypes = [c_void_p, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p)]
_batch_execute.restype = c_int
_batch_executef = lib.cufinufftf_batch_execute
_batch_executef.argtypes = [c_void_p, ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p)]
_batch_executef.restype = c_int
_batch_destroy = lib.cufinufft_batch_destroy
_batch_destroy.argtypes = [c_void_p]
_batch_destroy.restype = c_int
_batch_destroyf = lib.cufinufftf_batch_destroy
_batch_destroyf.argtypes = [c_void_p]
_batch_destroyf.restype = c_int


class TuneEntry(ctypes.Structure):
    """Mirror of cufinufft_tune_entry (autotuning record)."""
    _fields_ = [("method", c_int), ("binsizex", c_int), ("binsizey", c_int), ("binsizez", c_int),
                ("maxsubprobsize", c_int), ("ms", c_float)]


for _name in ("cufinufft_set_layout", "cufinufftf_set_layout"):
    getattr(lib, _name).argtypes = [c_void_p, c_int, c_int, c_int, c_int, c_int]
    getattr(lib, _name).restype = c_int
for _name in ("cufinufft_autotune", "cufinufftf_autotune"):
    getattr(lib, _name).argtypes = [c_void_p, ctypes.POINTER(TuneEntry), c_int, c_int_p]
    getattr(lib, _name).restype = c_int
_set_layout = lib.cufinufft_set_layout
_set_layoutf = lib.cufinufftf_set_layout
_autotune = lib.cufinufft_autotune
_autotunef = lib.cufinufftf_autotune

# Learned layout selector: plan features, layout classes and the MLP kernels.
MLP_FEATURES, MLP_HIDDEN, MLP_CLASSES = 14, 32, 12
MLP_PARAMS = (MLP_HIDDEN * MLP_FEATURES + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN
              + MLP_CLASSES * MLP_HIDDEN + MLP_CLASSES)
for _name in ("cufinufft_features", "cufinufftf_features"):
    getattr(lib, _name).argtypes = [c_void_p, c_void_p]
    getattr(lib, _name).restype = c_int
for _name in ("cufinufft_set_layout_class", "cufinufftf_set_layout_class"):
    getattr(lib, _name).argtypes = [c_void_p, c_int]
    getattr(lib, _name).restype = c_int
_features = lib.cufinufft_features
_featuresf = lib.cufinufftf_features
_set_layout_class = lib.cufinufft_set_layout_class
_set_layout_classf = lib.cufinufftf_set_layout_class
mlp_forward = lib.cufinufft_mlp_forward
mlp_forward.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]
mlp_forward.restype = c_int
mlp_grad = lib.cufinufft_mlp_grad
mlp_grad.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_void_p, c_void_p,
                     c_void_p, c_void_p]
mlp_grad.restype = c_int
mlp_adam = lib.cufinufft_mlp_adam
mlp_adam.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float, c_void_p]
mlp_adam.restype = c_int

# Measured accumulation ceilings (shared FP32 / int32 atomicAdd, global 8-byte reduction).
atomic_rate = lib.cufinufft_atomic_rate
atomic_rate.argtypes = [c_int, c_double_p]
atomic_rate.restype = c_int
