"""Complex helpers re-exported for API compatibility (``torchkbnufft/_math.py``).

Plain torch arithmetic on complex tensors or real tensors whose ``dim`` has
size 2 (real, imaginary).
"""

from __future__ import annotations

import torch
from torch import Tensor


def _split(x: Tensor, dim: int):
    return x.select(dim, 0), x.select(dim, 1)


def complex_mult(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """Complex product ``val1 * val2``."""
    if val1.is_complex():
        return val1 * val2
    a, b = _split(val1, dim)
    c, d = _split(val2, dim)
    return torch.stack((a * c - b * d, a * d + b * c), dim)


def conj_complex_mult(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """Complex product ``val1 * conj(val2)``."""
    if val1.is_complex():
        return val1 * val2.conj()
    a, b = _split(val1, dim)
    c, d = _split(val2, dim)
    return torch.stack((a * c + b * d, b * c - a * d), dim)


def absolute(val: Tensor, dim: int = -1) -> Tensor:
    """Complex magnitude (kept as the last dim of size 2 for real layouts)."""
    if val.is_complex():
        return val.abs()
    a, b = _split(val, dim)
    mag = torch.sqrt(a * a + b * b)
    return torch.stack((mag, torch.zeros_like(mag)), dim)


def complex_sign(val: Tensor, dim: int = -1) -> Tensor:
    """``val / |val|`` (0 where ``val`` is 0)."""
    if val.is_complex():
        mag = val.abs()
        return torch.where(mag > 0, val / torch.where(mag > 0, mag, torch.ones_like(mag)), torch.zeros_like(val))
    a, b = _split(val, dim)
    mag = torch.sqrt(a * a + b * b)
    safe = torch.where(mag > 0, mag, torch.ones_like(mag))
    return torch.stack((a / safe * (mag > 0), b / safe * (mag > 0)), dim)


def imag_exp(val: Tensor, dim: int = -1, return_complex: bool = True) -> Tensor:
    """``exp(1j * val)``."""
    out = torch.stack((torch.cos(val), torch.sin(val)), -1)
    return torch.view_as_complex(out) if return_complex else out


def inner_product(val1: Tensor, val2: Tensor, dim: int = -1) -> Tensor:
    """``sum(val1 * conj(val2))``."""
    if val1.dtype != val2.dtype:
        raise ValueError("val1 has different dtype than val2.")
    if not val1.is_complex():
        if not val1.shape[dim] == val2.shape[dim] == 2:
            raise ValueError("Real input does not have dimension size 2 at dim.")
        p = conj_complex_mult(val1, val2, dim)
        return torch.stack((p.select(dim, 0).sum(), p.select(dim, 1).sum()))
    return torch.sum(val1 * val2.conj())
