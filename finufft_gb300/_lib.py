"""ctypes binding of the in-tree libcufinufft.so (the GB300 NUFFT engine).

The struct layouts mirror include/cufinufft_opts.h and include/gbnufft_ext.h.
Loading fails loudly when the shared library has not been built: there is no
fallback implementation.
"""
import ctypes
import os
from ctypes import (POINTER, Structure, c_double, c_float, c_int, c_int64, c_size_t,
                    c_void_p)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcufinufft.so")


class CufinufftOpts(Structure):
    """Same field order and types as cufinufft_opts (include/cufinufft_opts.h)."""

    _fields_ = [
        ("upsampfac", c_double),
        ("gpu_method", c_int),
        ("gpu_sort", c_int),
        ("gpu_binsizex", c_int),
        ("gpu_binsizey", c_int),
        ("gpu_binsizez", c_int),
        ("gpu_obinsizex", c_int),
        ("gpu_obinsizey", c_int),
        ("gpu_obinsizez", c_int),
        ("gpu_maxsubprobsize", c_int),
        ("gpu_kerevalmeth", c_int),
        ("gpu_spreadinterponly", c_int),
        ("gpu_maxbatchsize", c_int),
        ("gpu_device_id", c_int),
        ("gpu_stream", c_void_p),
        ("modeord", c_int),
        ("gpu_np", c_int),
        ("debug", c_int),
    ]


class PlanInfo(Structure):
    """gbnufft_plan_info (include/gbnufft_ext.h)."""

    _fields_ = [
        ("type", c_int), ("dim", c_int), ("ntransf", c_int), ("batchsize", c_int),
        ("ns", c_int), ("beta", c_double), ("upsampfac", c_double),
        ("nf", c_int * 3), ("bins", c_int * 3), ("method", c_int), ("nsub", c_int),
        ("M", c_int64), ("N", c_int64), ("spread_smem", c_size_t),
        ("horner_err", c_double), ("inner_nf", c_int * 3), ("spread_variant", c_int),
        ("maxsubprobsize", c_int), ("spread_fixed", c_int), ("kernel_form", c_int),
        ("planner_used", c_int), ("planned_slot", c_int), ("features", c_float * 12),
        ("tune_ms", c_double * 12),
    ]


class GbnufftOpts(Structure):
    """gbnufft_opts (include/gbnufft_ext.h)."""

    _fields_ = [("planner", c_int), ("spread_variant", c_int), ("fft_prune", c_int),
                ("spread_float_tile", c_int), ("kernel_form", c_int), ("kerformula", c_int),
                ("sort_keys", c_int), ("interp_mode", c_int), ("batch_cap", c_int),
                ("reserved", c_int * 7)]


class FinufftOpts(Structure):
    """Same layout as finufft_opts (include/finufft.h)."""

    _fields_ = [
        ("modeord", c_int), ("spreadinterponly", c_int), ("debug", c_int),
        ("spread_debug", c_int), ("showwarn", c_int), ("nthreads", c_int), ("fftw", c_int),
        ("spread_sort", c_int), ("spread_kerevalmeth", c_int), ("spread_kerpad", c_int),
        ("upsampfac", c_double), ("spread_thread", c_int), ("maxbatchsize", c_int),
        ("spread_nthr_atomic", c_int), ("spread_max_sp_size", c_int),
        ("spread_kerformula", c_int), ("allow_eps_too_small", c_int),
        ("fftw_lock_fun", c_void_p), ("fftw_unlock_fun", c_void_p),
        ("fftw_lock_data", c_void_p),
    ]


_lib = None


def load(path=LIB_PATH):
    """Load the engine library (raises OSError when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(
            "GB300 NUFFT library not built (%s missing): run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first" % path)
    lib = ctypes.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib):
    i64p = POINTER(c_int64)
    for pfx, real in (("cufinufft", c_double), ("cufinufftf", c_float)):
        f = getattr(lib, pfx + "_makeplan")
        f.argtypes = [c_int, c_int, i64p, c_int, c_int, real, POINTER(c_void_p),
                      POINTER(CufinufftOpts)]
        f.restype = c_int
        f = getattr(lib, pfx + "_makeplan_ext")
        f.argtypes = [c_int, c_int, i64p, c_int, c_int, real, POINTER(c_void_p),
                      POINTER(CufinufftOpts), POINTER(GbnufftOpts)]
        f.restype = c_int
        f = getattr(lib, pfx + "_setpts")
        f.argtypes = [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                      c_void_p, c_void_p]
        f.restype = c_int
        for name in ("_execute", "_execute_adjoint", "_graph_capture"):
            f = getattr(lib, pfx + name)
            f.argtypes = [c_void_p, c_void_p, c_void_p]
            f.restype = c_int
        for name in ("_destroy", "_graph_launch"):
            f = getattr(lib, pfx + name)
            f.argtypes = [c_void_p]
            f.restype = c_int
        f = getattr(lib, pfx + "_plan_info")
        f.argtypes = [c_void_p, POINTER(PlanInfo)]
        f.restype = c_int
        f = getattr(lib, pfx + "_stage_times")
        f.argtypes = [c_void_p, c_int, POINTER(c_float)]
        f.restype = c_int
        f = getattr(lib, pfx + "_get_sort")
        f.argtypes = [c_void_p, c_void_p, c_void_p]
        f.restype = c_int
    lib.cufinufft_default_opts.argtypes = [POINTER(CufinufftOpts)]
    lib.cufinufft_default_opts.restype = None
    lib.finufft_default_opts.argtypes = [POINTER(FinufftOpts)]
    lib.finufft_default_opts.restype = None
    lib.gbnufft_version.restype = ctypes.c_char_p
    for pfx, real in (("cufinufft", c_double), ("cufinufftf", c_float)):
        f = getattr(lib, pfx + "_batch_makeplan")
        f.argtypes = [c_int, c_int, c_int, i64p, c_int, real, POINTER(c_void_p),
                      POINTER(CufinufftOpts), POINTER(GbnufftOpts)]
        f.restype = c_int
        f = getattr(lib, pfx + "_batch_setpts")
        f.argtypes = [c_void_p, i64p, c_void_p, c_void_p, c_void_p]
        f.restype = c_int
        f = getattr(lib, pfx + "_batch_execute")
        f.argtypes = [c_void_p, c_void_p, c_void_p]
        f.restype = c_int
        f = getattr(lib, pfx + "_batch_destroy")
        f.argtypes = [c_void_p]
        f.restype = c_int
    lib.cufinufftf_spread_noalloc.argtypes = [c_int, POINTER(c_int64), c_int64, c_void_p,
                                              c_void_p, c_void_p, c_void_p, c_void_p, c_float,
                                              c_void_p]
    lib.cufinufftf_spread_noalloc.restype = c_int
    lib.gbnufft_default_opts.argtypes = [POINTER(GbnufftOpts)]
    lib.gbnufft_default_opts.restype = None
    lib.gbnufft_smem_atomic_rate.argtypes = [c_int, POINTER(c_double)]
    lib.gbnufft_smem_atomic_rate.restype = c_int
    lib.gbnufft_smem_atomic_rate_i32.argtypes = [c_int, POINTER(c_double)]
    lib.gbnufft_smem_atomic_rate_i32.restype = c_int
    lib.gbnufft_trim_scratch.argtypes = [c_int]
    lib.gbnufft_trim_scratch.restype = c_int
    lib.gbnufft_kernel_choice.argtypes = [c_double, c_double, c_int, c_int, c_int, c_int, c_int,
                                          POINTER(c_int), POINTER(c_double)]
    lib.gbnufft_kernel_choice.restype = c_int
    lib.gbnufft_kernel_eval.argtypes = [c_int, c_int, c_double, c_int64, c_void_p, c_void_p]
    lib.gbnufft_kernel_eval.restype = c_int
    lib.gbnufft_device_error.argtypes = [c_int, POINTER(c_int)]
    lib.gbnufft_device_error.restype = c_int
    ip = POINTER(c_int)
    fp = POINTER(c_float)
    lib.gbnufft_planner_dims.argtypes = [ip, ip, ip, ip]
    lib.gbnufft_planner_dims.restype = c_int
    lib.gbnufft_planner_candidate.argtypes = [c_int, c_int, c_int, POINTER(c_double), ip, ip,
                                              ip, ip]
    lib.gbnufft_planner_candidate.restype = c_int
    lib.gbnufft_planner_valid.argtypes = [c_int, c_int, c_int, c_double, c_int, ip]
    lib.gbnufft_planner_valid.restype = c_int
    lib.gbnufft_planner_model.argtypes = [ip, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_void_p, fp, fp]
    lib.gbnufft_planner_model.restype = c_int
    lib.gbnufft_planner_forward.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    lib.gbnufft_planner_forward.restype = c_int
    lib.gbnufft_planner_train.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_int, c_int,
                                          c_float, c_float, ctypes.c_uint, c_void_p, c_void_p]
    lib.gbnufft_planner_train.restype = c_int
    lib.gbnufft_point_features.argtypes = [c_int, c_int, c_int, c_int64, c_void_p, c_void_p,
                                           c_void_p, c_void_p, c_void_p, c_double, c_double,
                                           c_int, c_double, c_void_p, c_void_p]
    lib.gbnufft_point_features.restype = c_int
    for pfx, real in (("finufft", c_double), ("finufftf", c_float)):
        f = getattr(lib, pfx + "_makeplan")
        f.argtypes = [c_int, c_int, i64p, c_int, c_int, real, POINTER(c_void_p),
                      POINTER(FinufftOpts)]
        f.restype = c_int
        f = getattr(lib, pfx + "_setpts")
        f.argtypes = [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                      c_void_p, c_void_p]
        f.restype = c_int
        for name in ("_execute", "_execute_adjoint"):
            f = getattr(lib, pfx + name)
            f.argtypes = [c_void_p, c_void_p, c_void_p]
            f.restype = c_int
        f = getattr(lib, pfx + "_destroy")
        f.argtypes = [c_void_p]
        f.restype = c_int


def default_ext_opts():
    o = GbnufftOpts()
    load().gbnufft_default_opts(ctypes.byref(o))
    return o


def default_opts():
    o = CufinufftOpts()
    load().cufinufft_default_opts(ctypes.byref(o))
    return o
