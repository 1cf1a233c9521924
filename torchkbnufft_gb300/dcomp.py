"""Pipe density compensation (``torchkbnufft/_nufft/dcomp.py:10-119``).

``w <- w / |A A^H w|`` for ``num_iterations`` rounds, with A the table
interpolation (no FFT), running on the CUDA interpolation kernels. The
trajectory layout is built once and reused by all 2*num_iterations calls.
"""

from __future__ import annotations

from typing import Optional, Sequence, Union

import torch
from torch import Tensor

from . import functional as F
from ._setup import init_fn


def calc_density_compensation_function(
    ktraj: Tensor,
    im_size: Sequence[int],
    num_iterations: int = 10,
    grid_size: Optional[Sequence[int]] = None,
    numpoints: Union[int, Sequence[int]] = 6,
    n_shift: Optional[Sequence[int]] = None,
    table_oversamp: Union[int, Sequence[int]] = 2**10,
    kbwidth: float = 2.34,
    order: Union[float, Sequence[float]] = 0.0,
) -> Tensor:
    """Density compensation weights for ``ktraj`` ``(d, M)`` or ``(N, d, M)``; returns complex ``(N, 1, M)``."""
    if ktraj.ndim not in (2, 3):
        raise ValueError("ktraj must have 2 or 3 dimensions")
    batch = 1
    if ktraj.ndim == 3:
        if ktraj.shape[0] == 1:
            ktraj = ktraj[0]
        else:
            batch = ktraj.shape[0]
    (tables, _, grid_size_t, n_shift_t, numpoints_t, offsets_t, table_oversamp_t, _, _) = init_fn(
        im_size=im_size, grid_size=grid_size, numpoints=numpoints, n_shift=n_shift, table_oversamp=table_oversamp,
        kbwidth=kbwidth, order=order, dtype=ktraj.dtype, device=ktraj.device)
    sig = torch.ones((batch, 1, ktraj.shape[-1]), dtype=tables[0].dtype, device=ktraj.device)
    for _ in range(num_iterations):
        grid = F.kb_table_interp_adjoint(sig, ktraj, tables, n_shift_t, numpoints_t, table_oversamp_t, offsets_t,
                                         grid_size_t)
        new = F.kb_table_interp(grid, ktraj, tables, n_shift_t, numpoints_t, table_oversamp_t, offsets_t)
        sig = sig / torch.abs(new)
    return sig
