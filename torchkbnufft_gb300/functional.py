"""Functional API with the reference's signatures (``torchkbnufft/functional``).

Each function accepts complex tensors, or real tensors with a trailing
dimension of size 2 (converted with ``view_as_complex`` and back), exactly as
the reference does (``functional/nufft.py:164-191``, ``functional/interp.py:82-172``).
All work runs in the CUDA library; CPU tensors raise.
"""

from __future__ import annotations

from typing import List, Optional, Tuple

import torch
from torch import Tensor

from . import _runtime as R
from ._autograd import KbTableInterpAdjoint, KbTableInterpForward, NufftAdjoint, NufftForward, ToepApply

__all__ = [
    "kb_table_interp",
    "kb_table_interp_adjoint",
    "kb_table_nufft",
    "kb_table_nufft_adjoint",
    "kb_spmat_interp",
    "kb_spmat_interp_adjoint",
    "kb_spmat_nufft",
    "kb_spmat_nufft_adjoint",
    "fft_filter",
]


def _to_complex(x: Tensor) -> Tuple[Tensor, bool]:
    if x.is_complex():
        return x, True
    if x.shape[-1] != 2:
        raise ValueError("For real inputs, last dimension must be size 2.")
    return torch.view_as_complex(x.contiguous()), False


def _back(x: Tensor, was_complex: bool) -> Tensor:
    return x if was_complex else torch.view_as_real(x)


def kb_table_interp(image: Tensor, omega: Tensor, tables: List[Tensor], n_shift: Tensor, numpoints: Tensor,
                    table_oversamp: Tensor, offsets: Tensor) -> Tensor:
    """Table interpolation from the grid to k-space (``functional/interp.py:82-124``)."""
    image, is_complex = _to_complex(image)
    _check_omega(omega, image.shape[0])
    data = KbTableInterpForward.apply(image, omega, tables, n_shift, numpoints, table_oversamp, offsets)
    return _back(data, is_complex)


def kb_table_interp_adjoint(data: Tensor, omega: Tensor, tables: List[Tensor], n_shift: Tensor, numpoints: Tensor,
                            table_oversamp: Tensor, offsets: Tensor, grid_size: Tensor) -> Tensor:
    """Adjoint table interpolation from k-space to the grid (``functional/interp.py:127-172``)."""
    data, is_complex = _to_complex(data)
    _check_omega(omega, data.shape[0], "data")
    image = KbTableInterpAdjoint.apply(data, omega, tables, n_shift, numpoints, table_oversamp, offsets, grid_size)
    return _back(image, is_complex)


def kb_table_nufft(image: Tensor, scaling_coef: Tensor, im_size: Tensor, grid_size: Tensor, omega: Tensor,
                   tables: List[Tensor], n_shift: Tensor, numpoints: Tensor, table_oversamp: Tensor, offsets: Tensor,
                   norm: Optional[str] = None) -> Tensor:
    """Forward NUFFT with table interpolation (``functional/nufft.py:126-191``)."""
    image, is_complex = _to_complex(image)
    R.norm_code(norm)
    _check_omega(omega, image.shape[0])
    geom = R.make_geom(image.dtype, im_size, grid_size, numpoints, table_oversamp, n_shift)
    data = NufftForward.apply(image, None, omega, geom, tables, scaling_coef, norm)
    return _back(data, is_complex)


def kb_table_nufft_adjoint(data: Tensor, scaling_coef: Tensor, im_size: Tensor, grid_size: Tensor, omega: Tensor,
                           tables: List[Tensor], n_shift: Tensor, numpoints: Tensor, table_oversamp: Tensor,
                           offsets: Tensor, norm: Optional[str] = None) -> Tensor:
    """Adjoint NUFFT with table interpolation (``functional/nufft.py:194-260``)."""
    data, is_complex = _to_complex(data)
    R.norm_code(norm)
    _check_omega(omega, data.shape[0], "data")
    geom = R.make_geom(data.dtype, im_size, grid_size, numpoints, table_oversamp, n_shift)
    image = NufftAdjoint.apply(data, None, omega, geom, tables, scaling_coef, norm)
    return _back(image, is_complex)


def fft_filter(image: Tensor, kernel: Tensor, norm: Optional[str] = "ortho") -> Tensor:
    """pad -> FFT -> multiply by kernel -> IFFT -> crop (``_nufft/fft.py:121-173``).

    The kernel multiplies the ``(B, C, *grid)`` spectrum with torch broadcasting,
    as in the reference: a ``(*grid)`` kernel is shared; a ``(K, *grid)`` kernel
    needs ``K == C`` (kernel k filters channel k) or ``C == 1`` (the output then
    has ``K`` channels, one per kernel).
    """
    R.norm_code(norm)
    nd = image.ndim - 2
    if kernel.ndim == nd:
        return ToepApply.apply(image, kernel, None, norm, "shared")
    if kernel.ndim != nd + 1:
        raise NotImplementedError("fft_filter supports kernels of shape (*grid) or (K, *grid)")
    K, C = kernel.shape[0], image.shape[1]
    if K == 1:
        return ToepApply.apply(image, kernel[0], None, norm, "shared")
    if C == 1:
        image = image.expand((image.shape[0], K) + tuple(image.shape[2:]))
    elif C != K:
        raise RuntimeError(
            f"The size of tensor a ({C}) must match the size of tensor b ({K}) at non-singleton dimension 1")
    return ToepApply.apply(image, kernel, None, norm, "channel")


def _check_omega(omega: Tensor, batch: int, what: str = "image") -> None:
    if omega.ndim not in (2, 3):
        raise ValueError("omega must have 2 or 3 dimensions.")
    if omega.ndim == 3 and omega.shape[0] not in (1, batch):
        raise ValueError(f"If omega has batch dim, omega batch dimension must match {what}.")


def kb_spmat_interp(image: Tensor, interp_mats: Tuple[Tensor, Tensor]) -> Tensor:
    """Sparse-matrix interpolation grid -> k-space (``functional/interp.py:11-44``)."""
    from .spmat import SpmatInterp

    image, is_complex = _to_complex(image)
    return _back(SpmatInterp.apply(image, interp_mats, tuple(image.shape[2:])), is_complex)


def kb_spmat_interp_adjoint(data: Tensor, interp_mats: Tuple[Tensor, Tensor], grid_size: Tensor) -> Tensor:
    """Sparse-matrix adjoint interpolation k-space -> grid (``functional/interp.py:47-79``)."""
    from .spmat import SpmatInterpAdjoint

    data, is_complex = _to_complex(data)
    gs = tuple(R.host_values(grid_size, int))
    return _back(SpmatInterpAdjoint.apply(data, interp_mats, gs), is_complex)


def _fft_geom(dtype, im_size, grid_size) -> R.GeomKey:
    nd = len(R.host_values(grid_size, int))
    return R.make_geom(dtype, im_size, grid_size, (1,) * nd, (1,) * nd, (0.0,) * nd)


def kb_spmat_nufft(image: Tensor, scaling_coef: Tensor, im_size: Tensor, grid_size: Tensor,
                   interp_mats: Tuple[Tensor, Tensor], norm: Optional[str] = None) -> Tensor:
    """Forward NUFFT with sparse-matrix interpolation (``functional/nufft.py:16-66``)."""
    from .spmat import SpmatNufft

    image, is_complex = _to_complex(image)
    R.norm_code(norm)
    data = SpmatNufft.apply(image, interp_mats, _fft_geom(image.dtype, im_size, grid_size), scaling_coef, norm)
    return _back(data, is_complex)


def kb_spmat_nufft_adjoint(data: Tensor, scaling_coef: Tensor, im_size: Tensor, grid_size: Tensor,
                           interp_mats: Tuple[Tensor, Tensor], norm: Optional[str] = None) -> Tensor:
    """Adjoint NUFFT with sparse-matrix interpolation (``functional/nufft.py:69-123``)."""
    from .spmat import SpmatNufftAdjoint

    data, is_complex = _to_complex(data)
    R.norm_code(norm)
    image = SpmatNufftAdjoint.apply(data, interp_mats, _fft_geom(data.dtype, im_size, grid_size), scaling_coef, norm)
    return _back(image, is_complex)
