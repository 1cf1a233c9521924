"""CPU port of the reference table path used as the timed CPU baseline — TEST / CPU-BASELINE INFRASTRUCTURE.

Forward: ``image * smaps * scaling`` -> zero-pad -> FFT -> table interpolation;
adjoint: table interpolation adjoint -> unnormalised IFFT -> crop ->
``* conj(scaling)`` -> ``sum_c conj(smaps)`` — the steps of
``torchkbnufft/modules/kbnufft.py:125-410`` and ``torchkbnufft/_nufft/fft.py:35-118``.
Interpolation runs in the C restatement (``interp_oracle.c``, OpenMP over
points / planes like the reference's forks); FFTs use scipy.fft with all host
threads. Only ``bench.py`` (CPU-baseline leg / reference arm) and tests use it.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import kbnufft_oracle as O

_lib = None
_ops = {}


def _load():
    global _lib
    if _lib is None:
        from . import build_oracle

        path = build_oracle.build()
        lib = ctypes.CDLL(path)
        for suf, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            for name in ("fwd", "adj"):
                fn = getattr(lib, f"tkbn_oracle_interp_{name}_{suf}")
                fn.restype = None
                fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ct), ctypes.POINTER(ctypes.c_void_p),
                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                               ctypes.c_void_p, ctypes.c_int]
        lib.tkbn_oracle_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def threads() -> int:
    return int(os.environ.get("TKBN_CPU_THREADS", os.cpu_count() or 1))


def describe() -> str:
    return f"C port (OpenMP, {threads()} threads) + scipy.fft ({threads()} workers), complex64"


def _args(op: O.Operator, rdt):
    nd = len(op.grid_size)
    K = (ctypes.c_int64 * 3)(*op.grid_size, *([1] * (3 - nd)))
    J = (ctypes.c_int * 3)(*op.numpoints, *([1] * (3 - nd)))
    Lo = (ctypes.c_int * 3)(*op.table_oversamp, *([1] * (3 - nd)))
    ct = ctypes.c_float if rdt == np.float32 else ctypes.c_double
    ns = (ct * 3)(*op.n_shift, *([0.0] * (3 - nd)))
    tabs = [np.ascontiguousarray(t) for t in op.tables]
    tp = (ctypes.c_void_p * 3)(*[t.ctypes.data for t in tabs], *([None] * (3 - nd)))
    return nd, K, J, Lo, ns, tp, tabs


def interp_forward(op: O.Operator, grid: np.ndarray, omega: np.ndarray) -> np.ndarray:
    lib = _load()
    rdt = np.float32 if grid.dtype == np.complex64 else np.float64
    suf = "f32" if rdt == np.float32 else "f64"
    grid = np.ascontiguousarray(grid)
    om = np.ascontiguousarray(omega, dtype=rdt)
    B, C = grid.shape[:2]
    M = om.shape[-1]
    out = np.empty((B, C, M), dtype=grid.dtype)
    nd, K, J, Lo, ns, tp, keep = _args(op, rdt)
    getattr(lib, f"tkbn_oracle_interp_fwd_{suf}")(nd, K, J, Lo, ns, tp, grid.ctypes.data, B, C, om.ctypes.data, M,
                                                  out.ctypes.data, threads())
    return out


def interp_adjoint(op: O.Operator, kdata: np.ndarray, omega: np.ndarray) -> np.ndarray:
    lib = _load()
    rdt = np.float32 if kdata.dtype == np.complex64 else np.float64
    suf = "f32" if rdt == np.float32 else "f64"
    kdata = np.ascontiguousarray(kdata)
    om = np.ascontiguousarray(omega, dtype=rdt)
    B, C, M = kdata.shape
    out = np.empty((B, C) + tuple(op.grid_size), dtype=kdata.dtype)
    nd, K, J, Lo, ns, tp, keep = _args(op, rdt)
    getattr(lib, f"tkbn_oracle_interp_adj_{suf}")(nd, K, J, Lo, ns, tp, kdata.ctypes.data, B, C, om.ctypes.data, M,
                                                  out.ctypes.data, threads())
    return out


class PortOperator(O.Operator):
    """The oracle's ``Operator`` with its interpolation run by the C port
    (one shared ``(d, M)`` trajectory), for benchmark-size trajectories in
    ``kbnufft_oracle.toeplitz_kernel`` / ``density_compensation``."""

    def interp(self, grid, omega):
        om = np.asarray(omega)
        if om.ndim == 3:
            return np.concatenate([interp_forward(self, grid[b:b + 1], om[b]) for b in range(om.shape[0])])
        return interp_forward(self, grid, om)

    def interp_adj(self, kdata, omega, grid_size=None):
        if grid_size is not None and tuple(grid_size) != tuple(self.grid_size):
            raise ValueError("the C port adjoint writes the operator's own grid size")
        om = np.asarray(omega)
        if om.ndim == 3:
            return np.concatenate([interp_adjoint(self, kdata[b:b + 1], om[b]) for b in range(om.shape[0])])
        return interp_adjoint(self, kdata, om)


def _op(im_size, cdtype):
    key = (tuple(im_size), np.dtype(cdtype))
    if key not in _ops:
        _ops[key] = O.Operator(im_size, cdtype=cdtype)
    return _ops[key]


def nufft_forward(image: np.ndarray, omega: np.ndarray, smaps=None, im_size=None) -> np.ndarray:
    """``KbNufft.forward`` (modules/kbnufft.py:125-228): ``image * smaps * scaling``
    -> zero-pad -> FFT -> table interpolation at ``omega`` (d, M). complex64 or
    complex128, following the image's dtype. ``smaps`` None: image (B, C, *N)."""
    import scipy.fft as sfft

    im_size = tuple(image.shape[2:]) if im_size is None else tuple(im_size)
    op = _op(im_size, image.dtype)
    nd = len(im_size)
    ax = tuple(range(-nd, 0))
    x = image * smaps if smaps is not None else image
    x = x * op.scaling
    pad = [(0, 0), (0, 0)] + [(0, g - n) for g, n in zip(op.grid_size, im_size)]
    grid = sfft.fftn(np.pad(x, pad), axes=ax, workers=threads()).astype(image.dtype, copy=False)
    del x
    return interp_forward(op, grid, omega)


def nufft_adjoint(kdata: np.ndarray, omega: np.ndarray, im_size, smaps=None) -> np.ndarray:
    """``KbNufftAdjoint.forward`` (modules/kbnufft.py:307-410): table
    interpolation adjoint -> unnormalised IFFT -> crop -> ``* conj(scaling)``
    -> ``sum_c conj(smaps)`` when maps are given."""
    import scipy.fft as sfft

    im_size = tuple(im_size)
    op = _op(im_size, kdata.dtype)
    nd = len(im_size)
    ax = tuple(range(-nd, 0))
    g2 = interp_adjoint(op, kdata, omega)
    img = sfft.ifftn(g2, axes=ax, norm="forward", workers=threads()).astype(kdata.dtype, copy=False)
    del g2
    img = img[(Ellipsis,) + tuple(slice(0, n) for n in im_size)] * np.conj(op.scaling)
    if smaps is None:
        return img
    return np.sum(img * np.conj(smaps), axis=1, keepdims=True)


def forward_adjoint(image: np.ndarray, smaps: np.ndarray, omega: np.ndarray):
    """One SENSE forward NUFFT and one adjoint NUFFT of its output; returns
    (k-space data, adjoint image)."""
    kdata = nufft_forward(image, omega, smaps)
    return kdata, nufft_adjoint(kdata, omega, image.shape[2:], smaps)
