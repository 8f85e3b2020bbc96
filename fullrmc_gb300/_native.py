"""ctypes binding of ``libfrmc_gpu.so`` (the C ABI in ``include/frmc_gpu.h``).

The library is built in-tree by ``fullrmc_gb300.build``.  There is no CPU
fallback: if the shared library is missing or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libfrmc_gpu.so")

F32P = ctypes.POINTER(ctypes.c_float)
F64P = ctypes.POINTER(ctypes.c_double)
I32P = ctypes.POINTER(ctypes.c_int32)
I64P = ctypes.POINTER(ctypes.c_int64)
U32P = ctypes.POINTER(ctypes.c_uint32)
i64 = ctypes.c_int64
i32 = ctypes.c_int32
f32 = ctypes.c_float
f64 = ctypes.c_double
cint = ctypes.c_int
vp = ctypes.c_void_p

FRMC_OK = 0
FRMC_E_ARG = -1
FRMC_E_CUDA = -2
FRMC_E_NOMEM = -3
FRMC_E_NODEV = -4
FRMC_E_TIMEOUT = -5
FRMC_E_STATE = -6
FRMC_E_INDEX = -7

# name -> argtypes; every function returns int (status) unless listed in _RESTYPE.
SIGNATURES = {
    "frmc_version": [],
    "frmc_last_error": [],
    "frmc_set_device": [cint],
    "frmc_device_info": [ctypes.POINTER(cint)] * 4,
    "frmc_pairs_distances_to_indexcoords": [i32, F32P, i64, F32P, cint, cint, F32P],
    "frmc_pairs_distances_to_point": [F32P, F32P, i64, F32P, cint, F32P],
    "frmc_pairs_distances_to_multi_points": [F32P, i64, i64, F32P, i64, F32P, cint, F32P],
    "frmc_pairs_distances_to_multi_indexcoords": [I32P, i64, F32P, i64, F32P, cint, cint, F32P],
    "frmc_point_to_point_distance": [F32P, F32P, F32P, cint, F32P],
    "frmc_from_to_points_differences": [F32P, F32P, i64, F32P, cint, F32P],
    "frmc_pair_difference_to_point": [F32P, F32P, F32P, cint, F32P],
    "frmc_pairs_differences_to_point": [F32P, F32P, i64, F32P, cint, F32P],
    "frmc_pairs_differences_to_indexcoords": [i32, F32P, i64, F32P, cint, cint, F32P],
    "frmc_pairs_differences_to_multi_points": [F32P, i64, i64, F32P, i64, F32P, cint, F32P],
    "frmc_pairs_differences_to_multi_indexcoords": [I32P, i64, F32P, i64, F32P, cint, cint, F32P],
    "frmc_single_pairs_histograms": [i32, F32P, i64, I32P, I32P, i32, i32, F32P, F32P, f32, f32, f32, cint],
    "frmc_multiple_pairs_histograms_coords": [I32P, i64, F32P, i64, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32,
                                              cint, F32P, F32P],
    "frmc_full_pairs_histograms_coords": [F32P, i64, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32, F32P, F32P],
    "frmc_group_move_delta_histograms": [I32P, i64, F32P, i64, F32P, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32,
                                         I32P, I32P],
    "frmc_multiple_pairs_histograms_dists": [I32P, i64, F32P, i64, I32P, I32P, i32, f32, f32, f32, i32, cint, F32P,
                                             F32P],
    "frmc_gr_to_sq": [F32P, F32P, i64, F32P, i64, f64, F64P],
    "frmc_Gr_to_sq": [F32P, F32P, i64, F32P, i64, F64P],
    "frmc_sq_to_Gr": [F32P, i64, F32P, i64, F32P, F64P],
    "frmc_transform_coordinates": [F32P, F32P, i64, F32P],
    "frmc_dev_full_hist_counts": [vp, vp, i64, F32P, cint, i32, f32, f32, f32, i32, vp, vp],
    "frmc_set_full_tune": [cint, cint, cint, cint, cint, f64],
    "frmc_set_full_aggregate": [cint],
    "frmc_sq_limits": [f32, f32, F32P, F32P],
    "frmc_basis_mode": [F32P, cint],
    "frmc_full_items": [i64, ctypes.POINTER(i64)],
    "frmc_dev_full_hist_counts_range": [vp, vp, i64, F32P, cint, i32, f32, f32, f32, i32, i64, i64, vp, vp],
    "frmc_dev_multiple_hist_counts": [vp, i64, vp, i64, F32P, cint, vp, vp, i32, f32, f32, f32, i32, cint, vp, vp],
    "frmc_dev_pack_atoms": [vp, vp, i64, vp, vp],
    "frmc_dev_full_pairs_histograms_noalloc": [vp, vp, i64, F32P, cint, i32, f32, f32, f32, i32, vp, vp, vp],
    "frmc_dev_counts_to_f32": [vp, i64, vp, vp],
    "frmc_multiple_atomic_distances_coords": [I32P, i64, F32P, i64, F32P, cint, I32P, I32P, i32, F32P, F32P, cint,
                                              cint, I32P, F32P, I32P, F32P],
    "frmc_multiple_atomic_distances_dists": [I32P, i64, F32P, i64, I32P, I32P, i32, F32P, F32P, cint, cint, I32P,
                                             F32P, I32P, F32P],
    "frmc_single_atomic_distances_dists": [i32, F32P, i64, I32P, I32P, i32, F32P, F32P, I32P, I32P, F32P, F32P, cint,
                                           cint],
    "frmc_pair_elements_stats": [I32P, I32P, i64, i32, I32P, I32P],
    "frmc_shape_function": [F32P, i64, F32P, cint, I32P, I32P, i32, f32, f32, f32, i32, i32, I32P, I32P, F64P, F64P,
                            F64P, f64, F64P, i32, F64P, i32, F64P, F64P, F64P],
    "frmc_coordination_terms": [F32P, i64, F32P, cint, F32P, I64P, I32P, i32, I32P, I64P, i32, I32P, I32P, I32P, i64,
                                F32P, F32P, F32P, i32],
}
_RESTYPE = {"frmc_last_error": ctypes.c_char_p}

_lock = threading.Lock()
_lib = None


class NativeError(RuntimeError):
    """A CUDA or device-side failure reported by the library."""


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError("fullrmc_gb300: %s is missing; build it with "
                              "`python -m fullrmc_gb300.build`" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = lib
        return lib


_fast = None
_fast_tried = False


def fastcall():
    """The compiled fast path of the per-move drop-in calls
    (``csrc/fastcall.c``, built beside the library), or None when it was not
    built or ``FRMC_FASTCALL=0``.  It calls the same C entry points as the
    ctypes wrappers, for the common case of well-formed numpy arguments."""
    global _fast, _fast_tried
    if not _fast_tried:
        _fast_tried = True
        load()
        if os.environ.get("FRMC_FASTCALL", "1") != "0":
            import glob
            import importlib.machinery
            import importlib.util
            paths = sorted(glob.glob(os.path.join(_PKG, "_lib", "_fastcall*.so")))
            if paths:
                loader = importlib.machinery.ExtensionFileLoader("fullrmc_gb300._fastcall", paths[0])
                spec = importlib.util.spec_from_loader(loader.name, loader)
                mod = importlib.util.module_from_spec(spec)
                loader.exec_module(mod)
                _fast = mod
    return _fast


def register(name, argtypes, restype=ctypes.c_int):
    """Declare a further entry point (used by the engine modules)."""
    SIGNATURES[name] = argtypes
    if restype is not ctypes.c_int:
        _RESTYPE[name] = restype
    if _lib is not None:
        fn = getattr(_lib, name)
        fn.argtypes = argtypes
        fn.restype = restype


def last_error() -> str:
    msg = load().frmc_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    if rc == FRMC_OK:
        return
    msg = last_error()
    if rc == FRMC_E_ARG:
        raise ValueError(msg)
    if rc == FRMC_E_INDEX:
        raise IndexError(msg)
    if rc == FRMC_E_NOMEM:
        raise MemoryError(msg)
    raise NativeError("frmc error %d: %s" % (rc, msg))


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr(a: np.ndarray, t=F32P):
    return a.ctypes.data_as(t)


def device_info():
    lib = load()
    vals = [cint() for _ in range(4)]
    check(lib.frmc_device_info(*[ctypes.byref(v) for v in vals]))
    return {"sms": vals[0].value, "max_smem_optin": vals[1].value, "cc": (vals[2].value, vals[3].value)}
