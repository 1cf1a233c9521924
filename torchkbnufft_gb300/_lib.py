"""ctypes binding of the C ABI in ``include/tkbn_gb300.h``.

The library is built in-tree by :mod:`torchkbnufft_gb300._build`. Importing
this module does not load it; :func:`lib` loads it on first use and raises if
it is missing or cannot be built — there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import _build

TKBN_ABI_VERSION = 1
TKBN_OK = 0
TKBN_ERR_INVALID = -1
TKBN_ERR_UNSUPPORTED = -2
TKBN_ERR_CUDA = -3
TKBN_ERR_CUFFT = -4
TKBN_ERR_DEVICE = -5

TKBN_C64 = 0
TKBN_C128 = 1
TKBN_NORM_NONE = 0
TKBN_NORM_ORTHO = 1


class Geometry(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("im_size", ctypes.c_int64 * 3),
        ("grid_size", ctypes.c_int64 * 3),
        ("numpoints", ctypes.c_int32 * 3),
        ("table_oversamp", ctypes.c_int32 * 3),
        ("n_shift", ctypes.c_double * 3),
        ("flags", ctypes.c_int32),
    ]


TKBN_TABLES_CONJ_SYMMETRIC = 1
TKBN_ADJ_DETERMINISTIC = 2
TKBN_LAYOUT_FORWARD_ONLY = 4
TKBN_TABLES_LINEAR_PHASE = 8
TKBN_ADJ_REUSE_FACTORS = 16


class PointsDesc(ctypes.Structure):
    _fields_ = [
        ("npts", ctypes.c_int64),
        ("ntraj", ctypes.c_int64),
        ("tile", ctypes.c_int32 * 3),
        ("chunk", ctypes.c_int32),
    ]


class RaggedProblem(ctypes.Structure):
    _fields_ = [
        ("geom", Geometry),
        ("points", PointsDesc),
        ("workspace", ctypes.c_void_p),
        ("tables", ctypes.c_void_p * 3),
        ("ncoil", ctypes.c_int64),
        ("grid", ctypes.c_void_p),
        ("kdata", ctypes.c_void_p),
    ]


_P = ctypes.c_void_p
_GP = ctypes.POINTER(Geometry)
_DP = ctypes.POINTER(PointsDesc)
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_PP = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes (restype is int for all)
SIGNATURES = {
    "tkbn_abi_version": [],
    "tkbn_last_error": [],
    "tkbn_device_status": [_P, ctypes.POINTER(ctypes.c_int32)],
    "tkbn_points_workspace_size": [_GP, _DP, ctypes.POINTER(ctypes.c_size_t)],
    "tkbn_points_build": [_GP, _DP, _P, _P, ctypes.c_size_t, _P],
    "tkbn_interp_fwd": [_GP, _DP, _P, _PP, _P, _I64, _I64, _P, _P],
    "tkbn_interp_adj": [_GP, _DP, _P, _PP, _P, _I64, _I64, _P, _P],
    "tkbn_interp_grad_omega": [_GP, _DP, _P, _PP, _PP, _P, _P, _I64, _I64, _P, _P],
    "tkbn_fft_plan_create": [_GP, _I64, _I64, ctypes.POINTER(ctypes.c_void_p)],
    "tkbn_fft_plan_destroy": [_P],
    "tkbn_fft_and_scale": [_GP, _P, _P, _P, _I64, _P, _I64, _I64, _INT, _P, _P],
    "tkbn_ifft_and_scale": [_GP, _P, _P, _P, _I64, _P, _I64, _I64, _INT, _P, _P],
    "tkbn_nufft_fwd": [_GP, _DP, _P, _P, _PP, _P, _P, _P, _I64, _I64, _I64, _INT, _P, _P, _P],
    "tkbn_nufft_adj": [_GP, _DP, _P, _P, _PP, _P, _P, _P, _I64, _I64, _I64, _INT, _P, _P, _P],
    "tkbn_fft_filter": [_GP, _P, _P, _P, _I64, _I64, _I64, _INT, _P, _P, _P],
    "tkbn_toep_apply": [_GP, _P, _P, _P, _I64, _P, _I64, _I64, _I64, _INT, _P, _P, _P],
    "tkbn_toep_kernel_assemble": [_INT, _INT, _P, _P, ctypes.c_double, _P, _P],
    "tkbn_interp_fwd_noalloc": [_GP, _PP, _P, _I64, _P, _I64, _I64, _P, _P],
    "tkbn_spmat_interp": [_INT, _I64, _I64, _P, _P, _P, _P, _I64, _P, _P],
    "tkbn_spmat_interp_adjoint": [_INT, _I64, _I64, _I64, _P, _P, _P, _P, _I64, _P, _P],
    "tkbn_ragged_plan_create": [ctypes.POINTER(RaggedProblem), _I64, ctypes.POINTER(ctypes.c_void_p)],
    "tkbn_ragged_plan_destroy": [_P],
    "tkbn_ragged_interp_fwd": [_P, _P],
    "tkbn_ragged_interp_adj": [_P, _P],
}

_lock = threading.Lock()
_lib = None


def load(path: str | None = None, build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) and type the shared library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if path is None:
            path = _build.lib_path()
            if not os.path.isfile(path) or not _build.up_to_date():
                if not build_if_missing:
                    raise RuntimeError(f"CUDA library not built: {path}")
                _build.build()
        cdll = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(cdll, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_char_p if name == "tkbn_last_error" else ctypes.c_int
        if cdll.tkbn_abi_version() != TKBN_ABI_VERSION:
            raise RuntimeError("tkbn ABI version mismatch")
        _lib = cdll
        return _lib


def lib() -> ctypes.CDLL:
    return _lib if _lib is not None else load()


def check(rc: int) -> None:
    """Map a C status to the Python exception the reference raises."""
    if rc == TKBN_OK:
        return
    msg = (lib().tkbn_last_error() or b"").decode(errors="replace")
    if rc == TKBN_ERR_INVALID:
        raise ValueError(msg)
    if rc == TKBN_ERR_UNSUPPORTED:
        raise TypeError(msg)
    raise RuntimeError(f"tkbn error {rc}: {msg}")


def ptr_array(ptrs) -> ctypes.Array:
    arr = (ctypes.c_void_p * 3)()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr
