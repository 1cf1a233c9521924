"""Layout autotuner: tile shape and work-item size of the trajectory layout.

The bin sort (``tkbn_points_build``) groups points by grid tile; the tile
shape sets the forward patch (tile + J - 1 cells per dim, staged in shared
memory), the adjoint's output tiles and how many tiles a footprint crosses,
and ``chunk`` bounds the points of one gather work item. The best choice
depends on the image size, the point density and the coil count, so this
module times the candidates on the caller's own trajectory (one forward and
one adjoint interpolation each, CUDA events, after a warm-up) and keeps the
fastest per problem class. The reference has no counterpart (its table path
has no tiling).
"""

from __future__ import annotations

import math
import threading
from typing import Dict, Optional, Sequence, Tuple

import torch

from . import _runtime as R

# candidate (tile, chunk) per dimension count; the first entry is the library default.
# 2D keeps the 16 x 14 tile of the register-accumulator adjoint (any other tile
# falls back to the shared-memory adjoint) and tunes the gather's work-item size.
CANDIDATES = {
    1: [((128,), 1024), ((64,), 1024), ((256,), 1024), ((128,), 2048)],
    2: [((16, 14), 1024), ((16, 14), 512), ((16, 14), 2048), ((16, 14), 256)],
    3: [((4, 4, 4), 1024), ((4, 4, 8), 1024), ((4, 8, 8), 1024), ((8, 8, 8), 1024), ((4, 4, 4), 2048)],
}

_lock = threading.Lock()
_best: Dict[tuple, Tuple[Tuple[int, ...], int]] = {}


def problem_key(geom: R.GeomKey, npts: int, ncoil: int, ntraj: int = 1) -> tuple:
    """Problems in one class share geometry, coil count and the power of two of the point count."""
    return (geom, int(math.log2(max(npts, 1))), int(ncoil), int(ntraj))


def _time_candidate(geom, omega, tables, ncoil, tile, chunk, reps) -> float:
    lay = R.PointsLayout(geom, omega, tile, chunk)
    cd = torch.complex64 if geom.dtype == 0 else torch.complex128
    B = 1 if omega.ndim == 2 else omega.shape[0]
    gen = torch.Generator(device=omega.device).manual_seed(0)
    grid = torch.randn((B, ncoil) + geom.grid_size, dtype=cd, device=omega.device, generator=gen)
    kdata = R.interp_fwd(geom, lay, tables, grid)
    R.interp_adj(geom, lay, tables, kdata)
    torch.cuda.synchronize(omega.device)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(reps):
        kdata = R.interp_fwd(geom, lay, tables, grid)
        R.interp_adj(geom, lay, tables, kdata)
    t1.record()
    torch.cuda.synchronize(omega.device)
    return t0.elapsed_time(t1) / reps


def tune_layout(geom: R.GeomKey, omega: torch.Tensor, tables: Sequence[torch.Tensor], ncoil: int,
                candidates: Optional[Sequence[Tuple[Tuple[int, ...], int]]] = None, reps: int = 3,
                cache: bool = True) -> Tuple[Tuple[int, ...], int]:
    """Fastest (tile, chunk) for forward + adjoint interpolation of this problem.

    Results are cached per problem class (``problem_key``); ``cache=False``
    re-times. Returns the library default when ``omega`` has no points.
    """
    R.require_cuda(omega)
    ntraj = 1 if omega.ndim == 2 else omega.shape[0]
    key = problem_key(geom, omega.shape[-1], ncoil, ntraj)
    if cache:
        with _lock:
            hit = _best.get(key)
        if hit is not None:
            return hit
    cands = list(candidates) if candidates is not None else CANDIDATES[geom.ndim]
    best = cands[0]
    if omega.shape[-1] > 0:
        times = []
        for tile, chunk in cands:
            tile = tuple(min(int(t), int(k)) for t, k in zip(tile, geom.grid_size))
            try:
                times.append((_time_candidate(geom, omega, tables, ncoil, tile, chunk, reps), (tile, chunk)))
            except (TypeError, ValueError):  # e.g. a patch that does not fit shared memory
                continue
        if times:
            best = min(times, key=lambda x: x[0])[1]
    with _lock:
        _best[key] = best
    return best


def clear() -> None:
    with _lock:
        _best.clear()
