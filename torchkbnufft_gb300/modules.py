"""Modules with the reference's constructor and forward signatures.

Buffers carry the same names as the reference's (``table_0..``, ``im_size``,
``grid_size``, ``n_shift``, ``numpoints``, ``offsets``, ``table_oversamp``,
``order``, ``alpha``, ``scaling_coef``; ``torchkbnufft/modules/_kbmodule.py:53-62``,
``modules/kbnufft.py:41-52``), so state dicts load either way.
"""

from __future__ import annotations

from typing import Optional, Sequence, Tuple, Union

import torch
import torch.nn as nn
from torch import Tensor

from . import _runtime as R
from . import functional as F
from ._autograd import NufftAdjoint, NufftForward, ToepApply
from ._setup import DTYPE_MAP, compute_scaling_coefs, init_fn

__all__ = ["KbModule", "KbInterp", "KbInterpAdjoint", "KbNufft", "KbNufftAdjoint", "ToepNufft"]


class KbModule(nn.Module):
    """Holds the precomputed NUFFT buffers (``modules/_kbmodule.py:9-116``)."""

    def __init__(
        self,
        im_size: Sequence[int],
        grid_size: Optional[Sequence[int]] = None,
        numpoints: Union[int, Sequence[int]] = 6,
        n_shift: Optional[Sequence[int]] = None,
        table_oversamp: Union[int, Sequence[int]] = 2**10,
        kbwidth: float = 2.34,
        order: Union[float, Sequence[float]] = 0.0,
        dtype: Optional[torch.dtype] = None,
        device: Optional[torch.device] = None,
    ):
        super().__init__()
        (tables, im_size_t, grid_size_t, n_shift_t, numpoints_t, offsets_t, table_oversamp_t, order_t,
         alpha_t) = init_fn(im_size=im_size, grid_size=grid_size, numpoints=numpoints, n_shift=n_shift,
                            table_oversamp=table_oversamp, kbwidth=kbwidth, order=order, dtype=dtype, device=device)
        for i, table in enumerate(tables):
            self.register_buffer(f"table_{i}", table)
        self.register_buffer("im_size", im_size_t)
        self.register_buffer("grid_size", grid_size_t)
        self.register_buffer("n_shift", n_shift_t)
        self.register_buffer("numpoints", numpoints_t)
        self.register_buffer("offsets", offsets_t)
        self.register_buffer("table_oversamp", table_oversamp_t)
        self.register_buffer("order", order_t)
        self.register_buffer("alpha", alpha_t)

    def to(self, *args, **kwargs):
        """``nn.Module.to`` that maps a requested dtype onto both complex and real buffers.

        A complex dtype converts complex buffers to it and real floating
        buffers to the matching real dtype, and vice versa
        (``modules/_kbmodule.py:64-108``). Integer buffers keep their dtype.
        """
        device, dtype, non_blocking, convert_to_format = torch._C._nn._parse_to(*args, **kwargs)
        complex_dtype = real_dtype = None
        if dtype is not None:
            if not (dtype.is_floating_point or dtype.is_complex):
                raise TypeError(
                    "KbModule.to only accepts floating point or complex dtypes, but got desired dtype={}".format(dtype))
            for c, r in DTYPE_MAP:
                if dtype in (c, r):
                    complex_dtype, real_dtype = c, r
                    break
            else:
                raise TypeError("Unrecognized type.")

        def convert(t):
            if dtype is not None and t.is_floating_point():
                target = real_dtype
            elif dtype is not None and t.is_complex():
                target = complex_dtype
            else:
                target = None
            if convert_to_format is not None and t.dim() == 4:
                return t.to(device, target, non_blocking, memory_format=convert_to_format)
            return t.to(device, target, non_blocking)

        return self._apply(convert)

    def _tables(self):
        return [getattr(self, f"table_{i}") for i in range(len(self.im_size))]

    def __repr__(self):
        out = "\n{}\n".format(self.__class__.__name__)
        out += "----------------------------------------\n"
        out += "buffers\n"
        for name, val in self._buffers.items():
            out += f"\ttensor: {name}, shape: {tuple(val.shape)}\n"
        return out


class KbInterpModule(KbModule):
    """Parent of the interpolation modules (``modules/kbinterp.py:10-38``)."""


class KbInterp(KbInterpModule):
    """Kaiser-Bessel table interpolation grid -> k-space (``modules/kbinterp.py:41-159``)."""

    def forward(self, image: Tensor, omega: Tensor, interp_mats: Optional[Tuple[Tensor, Tensor]] = None) -> Tensor:
        if interp_mats is not None:
            return F.kb_spmat_interp(image, interp_mats)
        return F.kb_table_interp(image=image, omega=omega, tables=self._tables(), n_shift=self.n_shift,
                                 numpoints=self.numpoints, table_oversamp=self.table_oversamp,
                                 offsets=self.offsets.to(torch.long))


class KbInterpAdjoint(KbInterpModule):
    """Adjoint table interpolation k-space -> grid (``modules/kbinterp.py:162-294``)."""

    def forward(self, data: Tensor, omega: Tensor, interp_mats: Optional[Tuple[Tensor, Tensor]] = None,
                grid_size: Optional[Tensor] = None) -> Tensor:
        if grid_size is None:
            grid_size = self.grid_size
        if interp_mats is not None:
            return F.kb_spmat_interp_adjoint(data, interp_mats, grid_size)
        return F.kb_table_interp_adjoint(data=data, omega=omega, tables=self._tables(), n_shift=self.n_shift,
                                         numpoints=self.numpoints, table_oversamp=self.table_oversamp,
                                         offsets=self.offsets, grid_size=grid_size)


class KbNufftModule(KbModule):
    """Adds the ``scaling_coef`` buffer (``modules/kbnufft.py:11-52``)."""

    def __init__(self, im_size, grid_size=None, numpoints=6, n_shift=None, table_oversamp=2**10, kbwidth=2.34,
                 order=0.0, dtype=None, device=None):
        super().__init__(im_size=im_size, grid_size=grid_size, numpoints=numpoints, n_shift=n_shift,
                         table_oversamp=table_oversamp, kbwidth=kbwidth, order=order, dtype=dtype, device=device)
        scaling_coef = compute_scaling_coefs(im_size=self.im_size.tolist(), grid_size=self.grid_size.tolist(),
                                             numpoints=self.numpoints.tolist(), alpha=self.alpha.tolist(),
                                             order=self.order.tolist())
        self.register_buffer("scaling_coef", scaling_coef.to(dtype=self.table_0.dtype, device=device))

    def _geom(self, dtype):
        return R.make_geom(dtype, self.im_size, self.grid_size, self.numpoints, self.table_oversamp, self.n_shift)


def _complex_inputs(x: Tensor, smaps: Optional[Tensor], what: str):
    if smaps is not None and smaps.dtype != x.dtype:
        raise TypeError(f"{what} dtype does not match smaps dtype.")
    if x.is_complex():
        return x, smaps, True
    if x.shape[-1] != 2:
        raise ValueError("For real inputs, last dimension must be size 2.")
    if smaps is not None:
        if smaps.shape[-1] != 2:
            raise ValueError("For real inputs, last dimension must be size 2.")
        smaps = torch.view_as_complex(smaps.contiguous())
    return torch.view_as_complex(x.contiguous()), smaps, False


class KbNufft(KbNufftModule):
    """Forward NUFFT: image -> k-space (``modules/kbnufft.py:55-228``).

    ``forward(image, omega, interp_mats=None, smaps=None, norm=None)``; image
    is ``(B, C, *im_size)`` (``(B, 1, *im_size)`` with smaps ``(B or 1, C, *im_size)``),
    omega ``(d, M)`` or ``(B, d, M)``; returns ``(B, C, M)``.
    """

    def forward(self, image: Tensor, omega: Tensor, interp_mats: Optional[Tuple[Tensor, Tensor]] = None,
                smaps: Optional[Tensor] = None, norm: Optional[str] = None) -> Tensor:
        image, smaps, is_complex = _complex_inputs(image, smaps, "image")
        if interp_mats is not None:
            if smaps is not None:
                image = image * smaps
            out = F.kb_spmat_nufft(image, self.scaling_coef, self.im_size, self.grid_size, interp_mats, norm)
            return out if is_complex else torch.view_as_real(out)
        R.norm_code(norm)
        F._check_omega(omega, image.shape[0])
        if smaps is not None and image.shape[1] != 1:
            # reference semantics: image * smaps broadcast, then per-channel NUFFT
            image, smaps = image * smaps, None
        out = NufftForward.apply(image, smaps, omega, self._geom(image.dtype), self._tables(), self.scaling_coef, norm)
        return out if is_complex else torch.view_as_real(out)


class KbNufftAdjoint(KbNufftModule):
    """Adjoint NUFFT: k-space -> image (``modules/kbnufft.py:231-410``).

    ``forward(data, omega, interp_mats=None, smaps=None, norm=None)``; with
    smaps the coil images are combined with ``sum_c conj(smaps)``.
    """

    def forward(self, data: Tensor, omega: Tensor, interp_mats: Optional[Tuple[Tensor, Tensor]] = None,
                smaps: Optional[Tensor] = None, norm: Optional[str] = None) -> Tensor:
        data, smaps, is_complex = _complex_inputs(data, smaps, "data")
        if interp_mats is not None:
            out = F.kb_spmat_nufft_adjoint(data, self.scaling_coef, self.im_size, self.grid_size, interp_mats, norm)
            if smaps is not None:
                out = torch.sum(out * smaps.conj(), dim=1, keepdim=True)
            return out if is_complex else torch.view_as_real(out)
        R.norm_code(norm)
        F._check_omega(omega, data.shape[0], "data")
        out = NufftAdjoint.apply(data, smaps, omega, self._geom(data.dtype), self._tables(), self.scaling_coef, norm)
        return out if is_complex else torch.view_as_real(out)


class ToepNufft(nn.Module):
    """Toeplitz-embedded normal operator ``A^H W A`` (``modules/kbnufft.py:413-547``)."""

    def __init__(self):
        super().__init__()

    def forward(self, image: Tensor, kernel: Tensor, smaps: Optional[Tensor] = None,
                norm: Optional[str] = None) -> Tensor:
        if kernel.dtype != image.dtype:
            raise TypeError("kernel and image must have same dtype.")
        if smaps is not None and smaps.dtype != image.dtype:
            raise TypeError("image dtype does not match smaps dtype.")
        is_complex = True
        if not image.is_complex():
            if image.shape[-1] != 2 or kernel.shape[-1] != 2:
                raise ValueError("For real inputs, last dimension must be size 2.")
            if smaps is not None:
                if smaps.shape[-1] != 2:
                    raise ValueError("For real inputs, last dimension must be size 2.")
                smaps = torch.view_as_complex(smaps.contiguous())
            is_complex = False
            image = torch.view_as_complex(image.contiguous())
            kernel = torch.view_as_complex(kernel.contiguous())
        R.norm_code(norm)
        nd = image.ndim - 2
        if kernel.ndim > nd:
            if kernel.shape[0] == 1:
                kernel = kernel[0]
            elif kernel.shape[0] != image.shape[0]:
                raise ValueError("If using batch dimension, kernel must have same batch size as image")
        if smaps is None:
            # the reference applies fft_filter to the whole batch (modules/kbnufft.py:537-538)
            out = F.fft_filter(image, kernel, norm)
        else:
            # one kernel per batch item (toep_batch_loop, modules/kbnufft.py:441-484)
            out = ToepApply.apply(image, kernel, smaps, norm, "batch" if kernel.ndim > nd else "shared")
        return out if is_complex else torch.view_as_real(out)
