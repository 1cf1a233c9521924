"""Toeplitz kernel construction (``torchkbnufft/_nufft/toep.py:11-307``).

The kernel D satisfies ``F^H D F ~= A^H W A`` on the 2x-embedded grid. Its
2^(d-1) sign-flipped adjoint NUFFTs of the weights (n_shift = 0) run as ONE
batched adjoint call on the GPU (the flips become a batched trajectory),
instead of the reference's recursion of separate calls. The reference's
flip-and-concatenate, conjugate-reflection and Hermitian-averaging steps
(``toep.py:185-307``) are one CUDA kernel (``tkbn_toep_kernel_assemble``,
each output cell read from at most two of the adjoint images, the scale
folded in), and the final FFT runs through the library's FFT stage.
"""

from __future__ import annotations

import ctypes
import itertools
import math
from typing import Optional, Sequence, Union

import torch
from torch import Tensor

from . import _lib as L
from . import _runtime as R
from .modules import KbNufftAdjoint


def calc_toeplitz_kernel(
    omega: Tensor,
    im_size: Sequence[int],
    weights: Optional[Tensor] = None,
    norm: Optional[str] = None,
    grid_size: Optional[Sequence[int]] = None,
    numpoints: Union[int, Sequence[int]] = 6,
    table_oversamp: Union[int, Sequence[int]] = 2**10,
    kbwidth: float = 2.34,
    order: Union[float, Sequence[float]] = 0.0,
) -> Tensor:
    """FFT kernel for :class:`~torchkbnufft_gb300.ToepNufft` (same signature as the reference).

    omega: ``(d, M)`` or ``(N, d, M)``; weights: ``(1, M)`` / ``(N, 1, M)``
    (or ``(N, M)`` with batched omega). Returns ``(2*im_size)`` or
    ``(N, *2*im_size)`` complex.
    """
    if omega.ndim not in (2, 3):
        raise ValueError("Unrecognized k-space shape.")
    if weights is not None:
        if weights.ndim not in (2, 3):
            raise ValueError("Unrecognized weights dimension.")
        if omega.ndim == 3 and weights.ndim == 2:
            if weights.shape[0] == 1:
                weights = weights.repeat(omega.shape[0], 1)
            if not weights.shape[0] == omega.shape[0]:
                raise ValueError("weights and omega do not have same batch size")
    args = dict(im_size=im_size, norm=norm, grid_size=grid_size, numpoints=numpoints, table_oversamp=table_oversamp,
                kbwidth=kbwidth, order=order)
    if omega.ndim == 2:
        return _one_kernel(omega, weights, **args)
    return torch.stack([_one_kernel(omega[i], None if weights is None else weights[i], **args)
                        for i in range(omega.shape[0])])


def _flip_patterns(nd: int):
    """Sign patterns (+1 for dim 0) in the order the reference recursion visits them."""
    return [(1,) + tuple(-1 if f else 1 for f in bits) for bits in itertools.product((0, 1), repeat=nd - 1)]


def _one_kernel(omega, weights, im_size, norm, grid_size, numpoints, table_oversamp, kbwidth, order):
    nd = omega.shape[0]
    adj = KbNufftAdjoint(im_size=im_size, grid_size=grid_size, numpoints=numpoints, n_shift=[0] * nd,
                         table_oversamp=table_oversamp, kbwidth=kbwidth, order=order, dtype=omega.dtype,
                         device=omega.device)
    cdt = adj.table_0.dtype
    M = omega.shape[-1]
    if weights is None:
        w = torch.ones((1, 1, M), dtype=cdt, device=omega.device)
    else:
        w = weights.to(cdt).reshape(1, 1, M)

    pats = _flip_patterns(nd)
    signs = torch.tensor(pats, dtype=omega.dtype, device=omega.device).unsqueeze(-1)  # (P, d, 1)
    om_b = signs * omega.unsqueeze(0)  # (P, d, M)
    parts = adj(w.expand(len(pats), 1, M).contiguous(), om_b, norm=norm).contiguous()  # (P, 1, *N)

    geom = adj._geom(cdt)
    im = geom.im_size
    big = tuple(2 * n for n in im)
    if norm == "ortho":
        scale = math.sqrt(math.prod(big) / math.prod(geom.grid_size))
    else:
        scale = 1.0 / math.prod(big)
    kern = torch.empty((1, 1) + big, dtype=cdt, device=omega.device)
    sizes = (ctypes.c_int64 * 3)(*im, *([1] * (3 - nd)))
    L.check(L.lib().tkbn_toep_kernel_assemble(R.dtype_code(cdt), nd, ctypes.addressof(sizes), parts.data_ptr(),
                                              scale, kern.data_ptr(), R.stream_handle(omega.device)))
    fgeom = R.GeomKey(nd, R.dtype_code(cdt), big, big, (1,) * nd, (1,) * nd, (0.0,) * nd)
    return R.fft_and_scale(fgeom, kern, None, None, norm)[0, 0]
