"""Sparse-matrix interpolation (``interp_mats=``).

``calc_tensor_spmatrix`` builds torchkbnufft's interpolation matrices
(torchkbnufft/_nufft/spmat.py:10-105 and build_numpy_spmatrix,
torchkbnufft/_nufft/utils.py:16-119): exact Kaiser-Bessel weights (no table),
the kernel's linear phase, the fftshift phase and a conjugation, as a
``(real, imag)`` pair of sparse COO tensors of shape ``(M, prod(grid_size))``.
Like the tables, it is host setup (numpy/scipy, once per trajectory).

The interpolation itself (``spmat_interp`` / ``spmat_interp_adjoint``,
torchkbnufft/_nufft/interp.py:13-85, there two real ``torch.mm`` calls per
direction) runs in CUDA (``tkbn_spmat_interp(_adjoint)``) on a CSR copy of
the matrix kept per matrix pair. Any matrix pair of that layout works,
including the reference's own.
"""

from __future__ import annotations

import threading
import weakref
from typing import Optional, Sequence, Tuple, Union

import numpy as np
import torch
from torch import Tensor

from . import _lib as L
from . import _runtime as R
from . import _setup as S
from ._setup import validate_args


def calc_tensor_spmatrix(omega: Tensor, im_size: Sequence[int], grid_size: Optional[Sequence[int]] = None,
                         numpoints: Union[int, Sequence[int]] = 6, n_shift: Optional[Sequence[int]] = None,
                         table_oversamp: Union[int, Sequence[int]] = 2**10, kbwidth: float = 2.34,
                         order: Union[float, Sequence[float]] = 0.0) -> Tuple[Tensor, Tensor]:
    """Sparse interpolation matrices ``(real, imag)`` for ``interp_mats=`` (signature as torchkbnufft's)."""
    if not omega.ndim == 2:
        raise ValueError("Sparse matrix calculation not implemented for batched omega.")
    im_size, grid_size, numpoints, n_shift, table_oversamp, order, alpha, dtype, device = validate_args(
        im_size, grid_size, numpoints, n_shift, table_oversamp, kbwidth, order, omega.dtype, omega.device)
    coo = S.build_numpy_spmatrix(omega.detach().cpu().numpy(), numpoints, im_size, grid_size, n_shift, order, alpha)
    idx = torch.tensor(np.stack((coo.row, coo.col)).astype(np.int64), dtype=torch.long, device=device)
    shape = torch.Size(coo.shape)
    # the indices are in range by construction (column wrap mod K, rows 0..M-1)
    with torch.sparse.check_sparse_tensor_invariants(enable=False):
        real = torch.sparse_coo_tensor(idx, torch.tensor(np.real(coo.data), dtype=dtype, device=device), shape)
        imag = torch.sparse_coo_tensor(idx, torch.tensor(np.imag(coo.data), dtype=dtype, device=device), shape)
    return real, imag


class _CSR:
    """Complex CSR copy of a (real, imag) sparse matrix pair on the device."""

    def __init__(self, real: Tensor, imag: Tensor, cdtype: torch.dtype, device: torch.device):
        rdt = R.real_of(cdtype)
        # the indices are those of two valid sparse tensors of this shape
        with torch.sparse.check_sparse_tensor_invariants(enable=False):
            both = torch.sparse_coo_tensor(
                torch.cat((real._indices(), imag._indices()), dim=1),
                torch.cat((real._values().to(rdt).to(cdtype), 1j * imag._values().to(rdt).to(cdtype))),
                real.shape).coalesce()
        idx = both.indices().to(device)
        self.nrows, self.ncols = int(real.shape[0]), int(real.shape[1])
        self.nnz = int(idx.shape[1])
        self.row = idx[0].to(torch.int32).contiguous()
        self.col = idx[1].to(torch.int32).contiguous()
        self.val = both.values().to(device=device, dtype=cdtype).contiguous()
        counts = torch.bincount(idx[0], minlength=self.nrows)
        self.crow = torch.zeros(self.nrows + 1, dtype=torch.int64, device=device)
        self.crow[1:] = torch.cumsum(counts, 0)


_lock = threading.Lock()
_csr_cache: dict = {}


def _csr_of(interp_mats, cdtype: torch.dtype, device: torch.device) -> _CSR:
    if not isinstance(interp_mats, tuple) or len(interp_mats) != 2:
        raise TypeError("interp_mats must be 2-tuple of (real_mat, imag_mat.")
    real, imag = interp_mats
    key = (id(real), id(imag), real._version, imag._version, cdtype, device)
    with _lock:
        hit = _csr_cache.get(key)
        if hit is not None and hit[0]() is real and hit[1]() is imag:
            return hit[2]
    csr = _CSR(real, imag, cdtype, device)
    with _lock:
        _csr_cache[key] = (weakref.ref(real), weakref.ref(imag), csr)
        while len(_csr_cache) > 16:
            _csr_cache.pop(next(iter(_csr_cache)))
    return csr


def spmat_interp(image: Tensor, interp_mats) -> Tensor:
    """kdata (B, C, M) = A @ grid for every (batch, coil) plane."""
    dev = R.require_cuda(image)
    image = image.contiguous()
    csr = _csr_of(interp_mats, image.dtype, dev)
    B, C = image.shape[:2]
    if image[0, 0].numel() != csr.ncols:
        raise ValueError("interp_mats columns do not match the grid size")
    out = torch.empty((B, C, csr.nrows), dtype=image.dtype, device=dev)
    L.check(L.lib().tkbn_spmat_interp(R.dtype_code(image.dtype), csr.nrows, csr.ncols, csr.crow.data_ptr(),
                                      csr.col.data_ptr(), csr.val.data_ptr(), image.data_ptr(), B * C,
                                      out.data_ptr(), R.stream_handle(dev)))
    return out


def spmat_interp_adjoint(data: Tensor, interp_mats, grid_size) -> Tensor:
    """grid (B, C, *grid_size) = A^H @ kdata for every (batch, coil) plane."""
    dev = R.require_cuda(data)
    data = data.contiguous()
    csr = _csr_of(interp_mats, data.dtype, dev)
    B, C = data.shape[:2]
    gs = tuple(R.host_values(grid_size, int))
    out = torch.empty((B, C) + gs, dtype=data.dtype, device=dev)
    L.check(L.lib().tkbn_spmat_interp_adjoint(R.dtype_code(data.dtype), csr.nrows, csr.ncols, csr.nnz,
                                              csr.row.data_ptr(), csr.col.data_ptr(), csr.val.data_ptr(),
                                              data.data_ptr(), B * C, out.data_ptr(), R.stream_handle(dev)))
    return out


class SpmatInterp(torch.autograd.Function):
    """Forward sparse interpolation; backward is the adjoint (and vice versa)."""

    @staticmethod
    def forward(ctx, image, interp_mats, grid_shape):
        ctx.interp_mats = interp_mats
        ctx.grid_shape = grid_shape
        return spmat_interp(image, interp_mats)

    @staticmethod
    def backward(ctx, grad):
        return spmat_interp_adjoint(grad, ctx.interp_mats, ctx.grid_shape), None, None


class SpmatInterpAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, interp_mats, grid_shape):
        ctx.interp_mats = interp_mats
        return spmat_interp_adjoint(data, interp_mats, grid_shape)

    @staticmethod
    def backward(ctx, grad):
        return spmat_interp(grad, ctx.interp_mats), None, None


class SpmatNufft(torch.autograd.Function):
    """image -> FFT stage -> sparse interpolation; backward is the adjoint NUFFT."""

    @staticmethod
    def forward(ctx, image, interp_mats, geom, scaling, norm):
        ctx.interp_mats, ctx.geom, ctx.norm = interp_mats, geom, norm
        ctx.save_for_backward(scaling)
        return spmat_interp(R.fft_and_scale(geom, image, None, scaling, norm), interp_mats)

    @staticmethod
    def backward(ctx, grad):
        (scaling,) = ctx.saved_tensors
        g = spmat_interp_adjoint(grad.contiguous(), ctx.interp_mats, ctx.geom.grid_size)
        return R.ifft_and_scale(ctx.geom, g, None, scaling, ctx.norm, overwrite=True), None, None, None, None


class SpmatNufftAdjoint(torch.autograd.Function):
    """sparse adjoint interpolation -> inverse FFT stage; backward is the forward NUFFT."""

    @staticmethod
    def forward(ctx, data, interp_mats, geom, scaling, norm):
        ctx.interp_mats, ctx.geom, ctx.norm = interp_mats, geom, norm
        ctx.save_for_backward(scaling)
        g = spmat_interp_adjoint(data, interp_mats, geom.grid_size)
        return R.ifft_and_scale(geom, g, None, scaling, norm, overwrite=True)

    @staticmethod
    def backward(ctx, grad):
        (scaling,) = ctx.saved_tensors
        grid = R.fft_and_scale(ctx.geom, grad.contiguous(), None, scaling, ctx.norm)
        return spmat_interp(grid, ctx.interp_mats), None, None, None, None
