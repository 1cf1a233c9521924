"""Complex helpers with the behaviour of torchkbnufft's (``torchkbnufft/_math.py``).

Plain torch arithmetic on complex tensors, or on real tensors whose ``dim``
has size 2 (real, imaginary). Shapes, conventions and errors follow the
reference: ``absolute`` of a real pair keeps ``dim`` with size 1,
``complex_sign`` is ``exp(i atan2(im, re))`` (1 at zero) with a real pair
returned on the last axis, and ``inner_product`` is ``sum(conj(val1) val2)``.
"""

from __future__ import annotations

import torch
from torch import Tensor

_PAIR_ERROR = "Real input does not have dimension size 2 at dim."
_DTYPE_ERROR = "val1 has different dtype than val2."


def _pairs(dim: int, *vals: Tensor):
    """(real, imaginary) parts along ``dim`` of each real-layout tensor."""
    for v in vals:
        if v.shape[dim] != 2:
            raise ValueError(_PAIR_ERROR)
    return [(v.select(dim, 0), v.select(dim, 1)) for v in vals]


def _same_dtype(val1: Tensor, val2: Tensor) -> None:
    if val1.dtype != val2.dtype:
        raise ValueError(_DTYPE_ERROR)


def absolute(val: Tensor, dim: int = -1) -> Tensor:
    """``|val|``; a real-layout input keeps ``dim``, with size 1."""
    if val.is_complex():
        return val.abs()
    ((re, im),) = _pairs(dim, val)
    return torch.sqrt(re ** 2 + im ** 2).unsqueeze(dim)


def complex_mult(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """Complex product ``val1 * val2``."""
    _same_dtype(val1, val2)
    if val1.is_complex():
        return val1 * val2
    (a, b), (c, d) = _pairs(dim, val1, val2)
    return torch.stack((a * c - b * d, b * c + a * d), dim)


def conj_complex_mult(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """Complex product ``val1 * conj(val2)``."""
    _same_dtype(val1, val2)
    if val1.is_complex():
        return val1 * val2.conj()
    (a, b), (c, d) = _pairs(dim, val1, val2)
    return torch.stack((a * c + b * d, b * c - a * d), dim)


def imag_exp(val: Tensor, dim: int = -1, return_complex: bool = True) -> Tensor:
    """``exp(1j * val)``; as a real pair it sits on the last axis (``dim`` is not used)."""
    out = torch.stack((torch.cos(val), torch.sin(val)), -1)
    return torch.view_as_complex(out) if return_complex else out


def complex_sign(val: Tensor, dim: int = -1) -> Tensor:
    """``exp(i atan2(im, re))``: unit modulus, 1 where ``val`` is 0. A complex
    input gives a complex result; a real-layout input a real pair on the last axis."""
    if val.is_complex():
        parts = torch.view_as_real(val)
        return imag_exp(torch.atan2(parts[..., 1], parts[..., 0]), return_complex=True)
    ((re, im),) = _pairs(dim, val)
    return imag_exp(torch.atan2(im, re), return_complex=False)


def inner_product(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """``sum(conj(val1) * val2)``: a complex scalar, or for real-layout inputs
    the pair (real, imaginary) of shape (2,)."""
    _same_dtype(val1, val2)
    prod = conj_complex_mult(val2, val1, dim=dim)
    if val1.is_complex():
        return torch.sum(prod)
    return torch.stack((prod.select(dim, 0).sum(), prod.select(dim, 1).sum()))
