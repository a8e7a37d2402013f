"""ctypes binding of the C ABI in include/genpk_gb300.h.

The shared library is built in-tree (genpk_gb300/build.py).  Loading fails
loudly when it is missing: there is no CPU fallback for the hot path.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None
_COMPAT = None

c_f32p = ctypes.POINTER(ctypes.c_float)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_i32p = ctypes.POINTER(ctypes.c_int)
c_i64p = ctypes.POINTER(ctypes.c_int64)
c_void_p = ctypes.c_void_p

# name -> (restype, argtypes); exactly the functions include/genpk_gb300.h declares.
ABI = {
    "genpk_ctx_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_uint,
                                        ctypes.POINTER(c_void_p)]),
    "genpk_ctx_destroy": (None, [c_void_p]),
    "genpk_last_error": (ctypes.c_char_p, [c_void_p]),
    "genpk_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "genpk_zero": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_deposit": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_double, c_void_p, c_void_p,
                                     ctypes.c_double, ctypes.c_int64]),
    "genpk_power": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, c_f64p, c_i32p, c_f64p]),
    "genpk_power_multi": (ctypes.c_int, [c_void_p, ctypes.c_int, c_i32p, c_f64p, c_f64p, c_i32p,
                                         c_f64p]),
    "genpk_invwindow": (ctypes.c_double, [ctypes.c_int64] * 4),
    "genpk_geometry": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_i32p, c_f64p]),
    "genpk_load_spectrum": (ctypes.c_int, [c_void_p, ctypes.c_int, c_f64p]),
    "genpk_bin_of": (ctypes.c_int, [c_void_p, ctypes.c_int64]),
    "genpk_sync": (ctypes.c_int, [c_void_p]),
    "genpk_read_field": (ctypes.c_int, [c_void_p, ctypes.c_int, c_f64p]),
    "genpk_adjoint": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_double, c_void_p, c_void_p,
                                     ctypes.c_double, ctypes.c_int64, ctypes.c_double, c_f64p,
                                     c_void_p, c_void_p, c_f64p, ctypes.c_int]),
    "genpk_stage_times": (ctypes.c_int, [c_void_p, ctypes.POINTER(ctypes.c_char_p), c_f32p,
                                         ctypes.c_int]),
    "genpk_deposit_config": (ctypes.c_int, [c_void_p, c_i32p, c_i32p, c_i32p, c_i32p]),
    "genpk_kernel_launches": (ctypes.c_int64, [c_void_p]),
    "genpk_set_deposit_tile": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "genpk_timing_reset": (ctypes.c_int, [c_void_p]),
    "genpk_set_deposit_engine": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_last_deposit_engine": (ctypes.c_int, [c_void_p]),
    "genpk_set_fft_mode": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_inject_copy_timeout": (ctypes.c_int, [c_void_p, ctypes.c_int64, ctypes.c_int64]),
    "genpk_deposit_trials": (ctypes.c_int, [c_void_p, c_i32p, c_i32p, c_i32p, c_i32p, c_f32p,
                                            ctypes.c_int]),
    "genpk_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.c_int, ctypes.c_uint,
                                          ctypes.POINTER(c_void_p)]),
    "genpk_batch_destroy": (None, [c_void_p]),
    "genpk_batch_last_error": (ctypes.c_char_p, [c_void_p]),
    "genpk_batch_power": (ctypes.c_int, [c_void_p, c_f64p, ctypes.POINTER(c_void_p),
                                         ctypes.POINTER(c_void_p), c_f64p,
                                         ctypes.POINTER(ctypes.c_int64), c_f64p, c_f64p, c_i32p,
                                         c_f64p]),
    "genpk_batch_box": (c_void_p, [c_void_p, ctypes.c_int]),
    "genpk_batch_launches": (ctypes.c_int64, [c_void_p]),
    "genpk_batch_use_graph": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_power_step": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_double, c_void_p,
                                        c_void_p, c_f64p, c_i64p, ctypes.c_int, c_i32p, c_f64p,
                                        c_f64p, c_i32p, c_f64p]),
    "genpk_power_step_use_graph": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_power_step_replays": (ctypes.c_int64, [c_void_p]),
    "genpk_batch_graph_replays": (ctypes.c_int64, [c_void_p]),
    "genpk_batch_set_mode": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "genpk_batch_last_mode": (ctypes.c_int, [c_void_p]),
    "genpk_batch_auto_times": (ctypes.c_int, [c_void_p, c_f64p, c_f64p]),
    "genpk_batch_groups": (ctypes.c_int, [c_void_p]),
    "genpk_batch_group": (c_void_p, [c_void_p, ctypes.c_int, c_i32p, c_i32p]),
    "genpk_power_noalloc": (ctypes.c_int, [c_void_p, c_void_p, ctypes.c_int64, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_double, c_void_p, c_i32p,
                                           c_f64p, c_void_p]),
}

COMPAT_ABI = {
    "invwindow": (ctypes.c_double, [ctypes.c_int64] * 4),
    "powerspectrum": (ctypes.c_int, [ctypes.c_int64, c_f64p, c_f64p, ctypes.c_int, c_f64p,
                                     c_i32p, c_f64p, ctypes.c_double, ctypes.c_double]),
    "genpk_compat_bind": (ctypes.c_int, [c_void_p, ctypes.c_int, c_void_p]),
    "genpk_compat_unbind": (ctypes.c_int, [c_void_p]),
    "genpk_compat_release": (None, []),
}
# fieldize keeps the reference's C++ linkage (gen-pk.h:93).
COMPAT_FIELDIZE = "_Z8fieldizediPdlPfS0_di"


def lib_path() -> str:
    return _build.LIB


def load():
    """Load libgenpk_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"genpk_gb300 native library missing at {path}; "
                           "run genpk_gb300.build.build() (or __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in ABI.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def load_compat():
    """Load libgenpk_compat.so: the reference-signature drop-in."""
    global _COMPAT
    if _COMPAT is not None:
        return _COMPAT
    load()
    path = _build.COMPAT_LIB
    if not os.path.exists(path):
        raise RuntimeError(f"genpk_gb300 compat library missing at {path}")
    lib = ctypes.CDLL(path)
    for name, (res, args) in COMPAT_ABI.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    f = getattr(lib, COMPAT_FIELDIZE)
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_double, ctypes.c_int, c_f64p, ctypes.c_int64, c_f32p, c_f32p,
                  ctypes.c_double, ctypes.c_int]
    lib.fieldize = f
    _COMPAT = lib
    return lib
