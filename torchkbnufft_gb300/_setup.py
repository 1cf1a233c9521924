"""Host-side precompute for table-mode Kaiser-Bessel NUFFT.

Everything here runs once per operator (module construction), in float64 on the
host with numpy/scipy, and produces the small buffers the CUDA kernels read:

* one complex interpolation table per dimension (``J*L + 1`` entries),
* the separable image-domain scaling (de-apodisation) coefficients,
* the neighbour offset list and the normalised argument tuple.

The conventions follow the reference implementation so that module buffers and
state dicts are interchangeable:

* argument defaults and shapes: ``torchkbnufft/_nufft/utils.py:361-427``
  (``validate_args``: grid = 2*im, n_shift = im//2, alpha = kbwidth*J);
* table layout: ``torchkbnufft/_nufft/utils.py:122-179`` (``build_table``)
  together with the coefficient formula of ``build_numpy_spmatrix``
  (``utils.py:45-80``): entry ``k`` holds the kernel at distance
  ``u = k/L - J/2`` and the last entry is 0;
* scaling coefficients: ``torchkbnufft/_nufft/utils.py:182-254``;
* offsets: ``itertools.product`` over ``range(J_d)`` (``utils.py:329``).
"""

from __future__ import annotations

import itertools
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np
import torch
from scipy import special

# complex <-> real dtype pairs (reference: torchkbnufft/_nufft/utils.py:10-13)
DTYPE_MAP = [
    (torch.complex128, torch.float64),
    (torch.complex64, torch.float32),
]


def complex_and_real_dtype(dtype: torch.dtype) -> Tuple[torch.dtype, torch.dtype]:
    """Return ``(complex_dtype, real_dtype)`` for a float or complex dtype."""
    if dtype.is_complex:
        for c, r in DTYPE_MAP:
            if c == dtype:
                return c, r
    elif dtype.is_floating_point:
        for c, r in DTYPE_MAP:
            if r == dtype:
                return c, r
    raise TypeError("Unrecognized dtype.")


def validate_args(
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
    """Normalise NUFFT arguments to per-dimension tuples.

    Same defaults and return order as ``torchkbnufft/_nufft/utils.py:361-427``.
    """
    im_size = tuple(int(s) for s in im_size)
    ndim = len(im_size)
    grid_size = tuple(2 * s for s in im_size) if grid_size is None else tuple(int(s) for s in grid_size)
    if isinstance(numpoints, int):
        numpoints = (numpoints,) * len(grid_size)
    else:
        numpoints = tuple(int(j) for j in numpoints)
    n_shift = tuple(s // 2 for s in im_size) if n_shift is None else tuple(n_shift)
    if isinstance(table_oversamp, int):
        table_oversamp = (table_oversamp,) * len(grid_size)
    else:
        table_oversamp = tuple(int(t) for t in table_oversamp)
    alpha = tuple(kbwidth * j for j in numpoints)
    order = (order,) * len(grid_size) if isinstance(order, float) else tuple(order)
    dtype = torch.get_default_dtype() if dtype is None else dtype
    device = torch.device("cpu") if device is None else device

    for name, val in (
        ("grid_size", grid_size),
        ("n_shift", n_shift),
        ("numpoints", numpoints),
        ("alpha", alpha),
        ("order", order),
        ("table_oversamp", table_oversamp),
    ):
        assert len(val) == ndim, f"{name} must have one entry per image dimension"

    return im_size, grid_size, numpoints, n_shift, table_oversamp, order, alpha, dtype, device


def kb_kernel(u: np.ndarray, numpoints: int, alpha: float, order: float) -> np.ndarray:
    """Kaiser-Bessel kernel ``I_order(alpha*sqrt(1-(2u/J)^2)) / I_order(alpha)``.

    Zero for ``|u| >= J/2``. Formula of ``torchkbnufft/_nufft/utils.py:45-56``.
    """
    u = np.asarray(u, dtype=np.float64)
    half = numpoints / 2
    out = np.zeros(u.shape, dtype=np.float64)
    inside = np.abs(u) < half
    arg = np.sqrt(1.0 - (u[inside] / half) ** 2)
    out[inside] = np.real(special.iv(order, alpha * arg) / special.iv(order, alpha))
    return out


def kb_kernel_derivative(u: np.ndarray, numpoints: int, alpha: float, order: float) -> np.ndarray:
    """d/du of :func:`kb_kernel` (analytic; zero outside the support).

    Uses ``I_v'(x) = (I_{v-1}(x) + I_{v+1}(x)) / 2`` and the chain rule through
    ``s = sqrt(1 - (2u/J)^2)``: ``ds/du = -(2/J)^2 * u / s``.
    """
    u = np.asarray(u, dtype=np.float64)
    half = numpoints / 2
    out = np.zeros(u.shape, dtype=np.float64)
    inside = np.abs(u) < half
    s = np.sqrt(1.0 - (u[inside] / half) ** 2)
    x = alpha * s
    dI = 0.5 * (special.iv(order - 1, x) + special.iv(order + 1, x))
    # s -> 0 only at the support edge where u/s stays finite except exactly at
    # |u| = J/2, which is excluded by the strict inequality above.
    ds_du = -(u[inside] / (half * half)) / s
    out[inside] = np.real(dI * alpha * ds_du / special.iv(order, alpha))
    return out


def table_phase_rate(im_size: int, grid_size: int) -> float:
    """Linear phase rate of the tabulated kernel: ``gamma * (N - 1) / 2``.

    The table holds ``KB(u) * exp(-1j * rate * u)`` (the conjugate of the
    phase-modulated kernel of ``utils.py:76-80`` after ``utils.py:107``).
    """
    return (2 * np.pi / grid_size) * (im_size - 1) / 2


def build_table(
    im_size: Sequence[int],
    grid_size: Sequence[int],
    numpoints: Sequence[int],
    table_oversamp: Sequence[int],
    order: Sequence[float],
    alpha: Sequence[float],
) -> List[torch.Tensor]:
    """Complex128 interpolation tables, one per dimension, length ``J*L + 1``.

    Entry ``k`` is the interpolation weight at distance ``u = k/L - J/2``
    between a k-space sample and a grid cell (in cells); the final entry is the
    zero at ``u = J/2``. Equivalent to ``torchkbnufft/_nufft/utils.py:122-179``.
    """
    tables = []
    for n, k, j, L, m, a in zip(im_size, grid_size, numpoints, table_oversamp, order, alpha):
        u = np.arange(j * L, dtype=np.float64) / L - j / 2
        h = kb_kernel(u, j, a, m) * np.exp(-1j * table_phase_rate(n, k) * u)
        tables.append(torch.tensor(np.concatenate((h, np.zeros(1, dtype=np.complex128)))))
    return tables


def build_derivative_table(
    im_size: Sequence[int],
    grid_size: Sequence[int],
    numpoints: Sequence[int],
    table_oversamp: Sequence[int],
    order: Sequence[float],
    alpha: Sequence[float],
) -> List[torch.Tensor]:
    """d/du of each table entry (same abscissae as :func:`build_table`).

    Used by the trajectory gradient. Not part of the reference (which has no
    ktraj gradient, ``torchkbnufft/_autograd/interp.py:130``).
    """
    tables = []
    for n, k, j, L, m, a in zip(im_size, grid_size, numpoints, table_oversamp, order, alpha):
        u = np.arange(j * L, dtype=np.float64) / L - j / 2
        rate = table_phase_rate(n, k)
        ph = np.exp(-1j * rate * u)
        dh = (kb_kernel_derivative(u, j, a, m) - 1j * rate * kb_kernel(u, j, a, m)) * ph
        tables.append(torch.tensor(np.concatenate((dh, np.zeros(1, dtype=np.complex128)))))
    return tables


def kaiser_bessel_ft(omega: np.ndarray, numpoints: int, alpha: float, order: float, d: int) -> np.ndarray:
    """Fourier transform of the KB kernel (``torchkbnufft/_nufft/utils.py:182-209``)."""
    z = np.sqrt((2 * np.pi * (numpoints / 2) * omega) ** 2 - alpha**2 + 0j)
    nu = d / 2 + order
    val = (
        (2 * np.pi) ** (d / 2)
        * (numpoints / 2) ** d
        * alpha**order
        / special.iv(order, alpha)
        * special.jv(nu, z)
        / z**nu
    )
    return np.real(val)


def compute_scaling_coefs(
    im_size: Sequence[int],
    grid_size: Sequence[int],
    numpoints: Sequence[int],
    alpha: Sequence[float],
    order: Sequence[float],
) -> torch.Tensor:
    """Separable de-apodisation ``prod_d 1/KB_hat_d`` on the image grid.

    Same values as ``torchkbnufft/_nufft/utils.py:212-254``.
    """
    factors = []
    for n, k, j, a, m in zip(im_size, grid_size, numpoints, alpha, order):
        idx = np.arange(n) - (n - 1) / 2
        f = 1.0 / kaiser_bessel_ft(idx / k, j, a, m, 1)
        if j == 1:
            f = np.ones(f.shape)
        factors.append(f)
    coef = factors[0]
    for f in factors[1:]:
        coef = np.multiply.outer(coef, f)
    return torch.tensor(coef)


def init_fn(
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
    """Build every operator buffer; same return tuple as ``utils.py:257-358``.

    Returns ``(tables, im_size, grid_size, n_shift, numpoints, offsets,
    table_oversamp, order, alpha)`` as tensors on ``device``.
    """
    (im_size, grid_size, numpoints, n_shift, table_oversamp, order, alpha, dtype, device) = validate_args(
        im_size, grid_size, numpoints, n_shift, table_oversamp, kbwidth, order, dtype, device
    )
    tables = build_table(im_size, grid_size, numpoints, table_oversamp, order, alpha)
    offsets = list(itertools.product(*[range(j) for j in numpoints]))
    complex_dtype, real_dtype = complex_and_real_dtype(dtype)
    tables = [t.to(dtype=complex_dtype, device=device) for t in tables]
    return (
        tables,
        torch.tensor(im_size, dtype=torch.long, device=device),
        torch.tensor(grid_size, dtype=torch.long, device=device),
        torch.tensor(n_shift, dtype=real_dtype, device=device),
        torch.tensor(numpoints, dtype=torch.long, device=device),
        torch.tensor(offsets, dtype=torch.long, device=device),
        torch.tensor(table_oversamp, dtype=torch.long, device=device),
        torch.tensor(order, dtype=real_dtype, device=device),
        torch.tensor(alpha, dtype=real_dtype, device=device),
    )


def _exact_coefs(om: np.ndarray, npts: int, K: int, alpha: float, order: float):
    """Exact KB weights of each point's ``npts`` neighbours along one dim, and
    their kernel arguments (distance to each neighbour, in cells)."""
    gam = 2 * np.pi / K
    dist = om / gam - np.floor(om / gam - npts / 2)
    arg = dist[:, None] - np.arange(1, npts + 1)[None, :]
    coef = np.zeros(arg.shape, dtype=np.float64)
    inside = np.abs(arg) < npts / 2
    coef[inside] = special.iv(order, alpha * np.sqrt(1 - (arg[inside] / (npts / 2)) ** 2)) / special.iv(order, alpha)
    return coef, arg


def build_numpy_spmatrix(omega: np.ndarray, numpoints: Sequence[int], im_size: Sequence[int],
                         grid_size: Sequence[int], n_shift: Sequence[int], order: Sequence[float],
                         alpha: Sequence[float]):
    """Complex interpolation matrix ``(M, prod(grid_size))`` as a scipy COO matrix
    (``torchkbnufft/_nufft/utils.py:16-119``, same signature and entries).

    Entry (m, cell) is the conjugated product over dims of the exact KB weight
    times the kernel's linear phase ``exp(i gamma (N - 1)/2 u)``, times the
    fftshift phase ``exp(i omega_m . n_shift)``; neighbour columns wrap mod K.
    Entries are listed point by point (J^d per point), duplicates not summed.
    """
    from scipy.sparse import coo_matrix

    om = np.asarray(omega, dtype=np.float64)
    nd, M = om.shape
    coefs, cols = [], []
    for d in range(nd):
        K, N, J = int(grid_size[d]), int(im_size[d]), int(numpoints[d])
        c, arg = _exact_coefs(om[d], J, K, float(alpha[d]), float(order[d]))
        gam = 2 * np.pi / K
        coefs.append(c * np.exp(1j * gam * (N - 1) / 2 * arg))
        first = np.floor(om[d] / gam - J / 2)
        cols.append(np.mod(np.arange(1, J + 1)[None, :] + first[:, None], K) * int(np.prod(grid_size[d + 1:])))
    coef, col = coefs[0], cols[0]
    for d in range(1, nd):
        coef = (coef[:, :, None] * coefs[d][:, None, :]).reshape(M, -1)
        col = (col[:, :, None] + cols[d][:, None, :]).reshape(M, -1)
    coef = np.conj(coef) * np.exp(1j * (om.T @ np.asarray(n_shift, dtype=np.float64)))[:, None]
    rows = np.repeat(np.arange(M), coef.shape[1])
    return coo_matrix((coef.reshape(-1), (rows, col.reshape(-1).astype(np.int64))),
                      shape=(M, int(np.prod(grid_size))))
