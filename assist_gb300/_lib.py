"""Loader for libassist_gb300.so (mirrors assist/_libassist.py of ASSIST).

The library is built in place by ``python assist_gb300/build.py`` (a script:
importing the package needs the library) or ``__graft_entry__.build()``.  Set ASSIST_GB300_LIB to force a specific file.
There is no CPU fallback: a missing library is an ImportError.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_longlong, c_ulonglong, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.environ.get("ASSIST_GB300_LIB", os.path.join(HERE, "libassist_gb300.so"))
if not os.path.exists(LIBPATH):
    raise ImportError("libassist_gb300.so not found at %s: run `python assist_gb300/build.py` "
                      "(or __graft_entry__.build()) first" % LIBPATH)
clib = ctypes.CDLL(LIBPATH)
__libpath__ = LIBPATH


def _s(name: str) -> str:
    return c_char_p.in_dll(clib, name).value.decode("ascii")


__version__ = _s("assist_version_str")
__build__ = _s("assist_build_str")
__githash__ = _s("assist_githash_str")


def assist_error_messages(e: int) -> str:
    n = c_int.in_dll(clib, "assist_error_messages_N").value
    if e >= n:
        raise RuntimeError("An error occured while trying to process an ASSIST error message.")
    return (c_char_p * n).in_dll(clib, "assist_error_messages")[e].decode("ascii")


D = POINTER(c_double)
I = POINTER(c_int)


class Options(ctypes.Structure):
    """struct assist_gb300_options (include/assist.h)."""
    _fields_ = [("forces", c_int), ("gr_eih_sources", c_int), ("geocentric", c_int),
                ("alpha", c_double), ("nk", c_double), ("nm", c_double), ("nn", c_double), ("r0", c_double),
                ("epsilon", c_double), ("min_dt", c_double), ("dt0", c_double), ("max_steps", c_int),
                ("warm_start", c_int), ("threads_per_block", c_int), ("group_steps", c_int),
                ("dt_floor", c_double), ("group_order", c_int), ("blocks_per_sm", c_int),
                ("ephem_staging", c_int)]


class BatchStats(ctypes.Structure):
    """struct assist_gb300_batch_stats (include/assist.h)."""
    _fields_ = [("steps_accepted", c_longlong), ("steps_rejected", c_longlong), ("force_evals", c_longlong),
                ("pc_iterations", c_longlong), ("warm_start_used", c_longlong), ("warm_start_fallback", c_longlong),
                ("kernel_ms", c_double), ("tables_built", c_longlong)]


class TuneResult(ctypes.Structure):
    """struct assist_gb300_tune_result (include/assist.h)."""
    _fields_ = [("chosen", c_int), ("n_candidates", c_int), ("candidate", c_int * 4), ("kernel_ms", c_double * 4),
                ("signature", ctypes.c_char * 512)]


clib.assist_gb300_autotune_device.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p, c_void_p,
                                              c_void_p, c_int, c_void_p, c_void_p, POINTER(TuneResult)]
clib.assist_gb300_autotune_device.restype = c_int
clib.assist_gb300_plan_create.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_int, c_void_p, c_void_p, c_void_p, POINTER(c_void_p)]
clib.assist_gb300_plan_create.restype = c_int
clib.assist_gb300_plan_launch.argtypes = [c_void_p, c_void_p]
clib.assist_gb300_plan_launch.restype = c_int
clib.assist_gb300_plan_stats.argtypes = [c_void_p, POINTER(BatchStats)]
clib.assist_gb300_plan_stats.restype = c_int
clib.assist_gb300_plan_free.argtypes = [c_void_p]
clib.assist_gb300_plan_free.restype = None
clib.assist_gb300_default_options.argtypes = [POINTER(Options)]
clib.assist_gb300_default_options.restype = None
clib.assist_gb300_integrate_batch.argtypes = [c_void_p, POINTER(Options), c_int, D, D, D, D, c_int, D, I,
                                              POINTER(BatchStats)]
clib.assist_gb300_integrate_batch.restype = c_int
clib.assist_gb300_integrate_batch_device.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p, c_void_p,
                                                     c_void_p, c_int, c_void_p, c_void_p, c_void_p, POINTER(BatchStats)]
clib.assist_gb300_integrate_batch_device.restype = c_int
clib.assist_gb300_integrate_batch_dense_device.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p,
                                                           c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                           c_void_p, c_void_p, POINTER(BatchStats)]
clib.assist_gb300_integrate_batch_dense_device.restype = c_int
clib.assist_gb300_integrate_batch_device_static.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p,
                                                            c_void_p, c_void_p, c_void_p, c_void_p, POINTER(BatchStats)]
clib.assist_gb300_integrate_batch_device_static.restype = c_int
STATIC_MAX_PARTICLES = 1048576       # ASSIST_GB300_STATIC_MAX_PARTICLES
clib.assist_gb300_warm_n_params.restype = c_int
clib.assist_gb300_warm_init.argtypes = [c_ulonglong]
clib.assist_gb300_warm_init.restype = c_int
clib.assist_gb300_warm_set_params.argtypes = [c_void_p, c_int]
clib.assist_gb300_warm_set_params.restype = c_int
clib.assist_gb300_warm_get_params.argtypes = [c_void_p, c_int]
clib.assist_gb300_warm_get_params.restype = c_int
clib.assist_gb300_warm_grad.argtypes = [c_void_p, c_void_p, c_int, c_void_p, POINTER(c_double)]
clib.assist_gb300_warm_grad.restype = c_int
clib.assist_gb300_warm_adam_step.argtypes = [c_void_p, c_float]
clib.assist_gb300_warm_adam_step.restype = c_int
clib.assist_gb300_warm_train.argtypes = [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_ulonglong,
                                         POINTER(c_double)]
clib.assist_gb300_warm_train.restype = c_int
clib.assist_gb300_warm_infer.argtypes = [c_void_p, c_int, c_void_p]
clib.assist_gb300_warm_infer.restype = c_int
clib.assist_gb300_warm_set_log.argtypes = [c_void_p, c_void_p, c_int, c_int]
clib.assist_gb300_warm_set_log.restype = c_int
clib.assist_gb300_warm_log_count.restype = c_int
clib.assist_gb300_forces_device.argtypes = [c_void_p, POINTER(Options), c_int, c_void_p, c_void_p, c_void_p, c_int,
                                            c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
clib.assist_gb300_forces_device.restype = c_int
clib.assist_gb300_forces_shared_time_device.argtypes = [c_void_p, POINTER(Options), c_int, c_double, c_void_p, c_void_p,
                                                        c_void_p, c_void_p, c_void_p]
clib.assist_gb300_forces_shared_time_device.restype = c_int
clib.assist_gb300_ephem_device.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
clib.assist_gb300_ephem_device.restype = c_int
clib.assist_gb300_encounter_ratio_device.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
clib.assist_gb300_encounter_ratio_device.restype = c_int
clib.assist_gb300_group_plan.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double,
                                         c_void_p, c_void_p, c_void_p, POINTER(c_int)]
clib.assist_gb300_group_plan.restype = c_int
clib.assist_gb300_n_bodies.argtypes = [c_void_p]
clib.assist_gb300_n_bodies.restype = c_int
clib.assist_gb300_last_error.restype = c_char_p
clib.assist_gb300_fp64_peak_gflops.restype = c_double
clib.assist_ephem_create.restype = c_void_p
clib.assist_ephem_create.argtypes = [c_char_p, c_char_p]
clib.assist_ephem_free.argtypes = [c_void_p]
clib.assist_ephem_init.restype = c_int
clib.assist_detect_ephemeris_file_format.argtypes = [c_int]
clib.assist_detect_ephemeris_file_format.restype = c_int
clib.assist_detect_ascii_bin_signature.argtypes = [c_int]
clib.assist_detect_ascii_bin_signature.restype = c_int
clib.assist_discover_planets_path.argtypes = [c_char_p, ctypes.c_size_t, c_char_p]
clib.assist_discover_planets_path.restype = c_int


def last_error() -> str:
    v = clib.assist_gb300_last_error()
    return v.decode() if v else ""
