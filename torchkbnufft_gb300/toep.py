"""Toeplitz kernel construction (``torchkbnufft/_nufft/toep.py:11-307``).

The kernel D satisfies ``F^H D F ~= A^H W A`` on the 2x-embedded grid. Its
2^(d-1) sign-flipped adjoint NUFFTs of the weights (n_shift = 0) run as ONE
batched adjoint call on the GPU (the flips become a batched trajectory),
instead of the reference's recursion of separate calls; the Hermitian
completion, symmetrisation and final FFT follow the reference's steps.
"""

from __future__ import annotations

import itertools
from typing import Optional, Sequence, Union

import torch
from torch import Tensor

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
    parts = adj(w.expand(len(pats), 1, M).contiguous(), om_b, norm=norm)  # (P, 1, *N)
    lookup = {p: parts[i:i + 1] for i, p in enumerate(pats)}

    def assemble(dim: int, flips: tuple) -> Tensor:
        # mirrors adjoint_flip_and_concat (toep.py:185-237) without re-running adjoints
        axis = dim + 2
        if dim < nd - 1:
            k1 = assemble(dim + 1, flips)
            k2 = assemble(dim + 1, flips[:dim] + (-1,) + flips[dim + 1:])
        else:
            k1 = lookup[flips]
            k2 = lookup[flips[:dim] + (-1,) + flips[dim + 1:]]
        zshape = list(k1.shape)
        zshape[axis] = 1
        zero = torch.zeros(zshape, dtype=k1.dtype, device=k1.device)
        k2 = k2.narrow(axis, 1, k2.shape[axis] - 1)
        return torch.cat((k1, zero, k2.flip(axis)), axis)

    kern = assemble(1, (1,) * nd) if nd > 1 else parts[0:1]
    kern = _reflect_conj_concat(kern, 2)
    kern = _hermitify(kern, 2)
    im = adj.im_size.to(torch.float64)
    gs = adj.grid_size.to(torch.float64)
    if norm == "ortho":
        scale = torch.sqrt(torch.prod(2 * im) / torch.prod(gs)).item()
    else:
        scale = (1 / torch.prod(2 * im)).item()
    dims = tuple(range(-nd, 0))
    out = torch.fft.fftn(kern, dim=dims, norm="ortho" if norm == "ortho" else None)[0, 0] * scale
    return out


def _reverse_index(t: Tensor, d: int) -> Tensor:
    n = t.shape[d]
    idx = torch.remainder(-torch.arange(n, device=t.device), n)
    return t.index_select(d, idx)


def _reflect_conj_concat(kernel: Tensor, dim: int) -> Tensor:
    """Append the conjugate point reflection along ``dim`` (``toep.py:240-274``)."""
    tmp = kernel.conj()
    for d in range(dim, kernel.ndim):
        tmp = _reverse_index(tmp, d)
    zshape = list(kernel.shape)
    zshape[dim] = 1
    zero = torch.zeros(zshape, dtype=kernel.dtype, device=kernel.device)
    tmp = torch.cat((zero, tmp.narrow(dim, 1, tmp.shape[dim] - 1)), dim)
    return torch.cat((kernel, tmp), dim)


def _hermitify(kernel: Tensor, dim: int) -> Tensor:
    """Average with the conjugate point reflection (``toep.py:277-307``)."""
    rev = kernel
    for d in range(dim, kernel.ndim):
        rev = _reverse_index(rev, d)
    return (kernel + rev.conj()) / 2
