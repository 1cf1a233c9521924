"""CPU oracle for the table-mode KB NUFFT — TEST INFRASTRUCTURE ONLY.

This module restates the reference algorithm (mmuckley/torchkbnufft, table
mode) in numpy so that the CUDA product path can be checked against it. It is
imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``; the product package never imports it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this oracle against
the reference's own golden vectors (``tests/data/interp_data.pkl`` and
``tests/data/nufft_data.pkl``, converted to ``tests/golden/*.npz``) and against
fixtures produced by running the reference itself (``tests/golden/make_golden.py``).

Arithmetic follows the reference operation by operation where the result is
sensitive to it (table-bin selection and the fftshift phase):

* ``tm = omega / (fl(1/K) * fl(2*pi))`` in the working real dtype — the
  reference writes ``omega / (2*np.pi / grid_size)`` inside TorchScript, which
  lowers ``scalar / tensor`` to ``reciprocal(tensor) * scalar``
  (``torchkbnufft/_nufft/interp.py:171, 663``);
* ``base = 1 + floor(tm - J/2)`` (``interp.py:177, 670``);
* ``bin = round_half_even((tm - (base + j)) * L) + floor(J*L/2)``
  (``interp.py:129-132, 174``);
* coefficient = product of per-dimension table entries, conjugated for the
  adjoint (``interp.py:138-144``);
* grid index = ``sum_d ((base_d + j_d) mod K_d) * prod(K[d+1:])``
  (``interp.py:146-148``);
* phase ``exp(1j * sum_d omega_d * n_shift_d)`` with the products rounded
  before the sum (``interp.py:200-203``; conjugated for the adjoint,
  ``interp.py:680-686``).
"""

from __future__ import annotations

import itertools
from typing import List, Sequence

import numpy as np

# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------


def _real_dtype(cdtype) -> np.dtype:
    return np.dtype(np.float32) if np.dtype(cdtype) == np.complex64 else np.dtype(np.float64)


def normalized_freq(omega: np.ndarray, grid_size: Sequence[int], rdt) -> np.ndarray:
    """``tm = omega / (fl(1/K) * fl(2 pi))`` in dtype ``rdt`` (interp.py:171)."""
    rdt = np.dtype(rdt)
    om = np.asarray(omega, dtype=rdt)
    K = np.asarray(grid_size, dtype=rdt).reshape(-1, 1)
    gam = (rdt.type(1) / K) * rdt.type(2 * np.pi)
    return om / gam


def point_indices(tm: np.ndarray, numpoints: Sequence[int], rdt):
    """``base_d = 1 + floor(tm_d - J_d/2)`` as int64 (interp.py:177)."""
    rdt = np.dtype(rdt)
    J = np.asarray(numpoints, dtype=rdt).reshape(-1, 1)
    return (1 + np.floor(tm - J / rdt.type(2))).astype(np.int64)


def fftshift_phase(omega: np.ndarray, n_shift: Sequence[float], rdt) -> np.ndarray:
    """``exp(1j * sum_d omega_d * n_shift_d)`` (interp.py:200-203)."""
    rdt = np.dtype(rdt)
    om = np.asarray(omega, dtype=rdt)
    ns = np.asarray(n_shift, dtype=rdt).reshape(-1, 1)
    prod = om * ns
    arg = prod[0].copy()
    for d in range(1, prod.shape[0]):
        arg = arg + prod[d]
    cdt = np.complex64 if rdt == np.float32 else np.complex128
    return (np.cos(arg) + 1j * np.sin(arg)).astype(cdt)


def coef_and_index(tm, base, offset, tables, numpoints, table_oversamp, grid_size, conj, rdt):
    """Coefficient and flat grid index for one neighbour offset (interp.py:88-150)."""
    rdt = np.dtype(rdt)
    M = tm.shape[-1]
    cdt = tables[0].dtype
    coef = np.ones(M, dtype=cdt)
    idx = np.zeros(M, dtype=np.int64)
    ndim = len(grid_size)
    for d in range(ndim):
        g = base[d] + offset[d]
        dist = np.rint((tm[d] - g.astype(rdt)) * rdt.type(table_oversamp[d])).astype(np.int64)
        center = (numpoints[d] * table_oversamp[d]) // 2
        t = tables[d][dist + center]
        coef = coef * (np.conj(t) if conj else t)
        stride = int(np.prod(grid_size[d + 1 :])) if d + 1 < ndim else 1
        idx = idx + np.mod(g, grid_size[d]) * stride
    return coef, idx


def _offsets(numpoints):
    return list(itertools.product(*[range(j) for j in numpoints]))


# ---------------------------------------------------------------------------
# interpolation (H3 / H4)
# ---------------------------------------------------------------------------


def interp_forward(
    grid: np.ndarray,
    omega: np.ndarray,
    tables: List[np.ndarray],
    n_shift: Sequence[float],
    numpoints: Sequence[int],
    table_oversamp: Sequence[int],
) -> np.ndarray:
    """Table interpolation grid -> k-space (``table_interp``, interp.py:153-203, 315-403).

    grid: (B, C, *K) complex; omega: (d, M) or (B, d, M) real.
    Returns (B, C, M) in grid's dtype.
    """
    grid = np.asarray(grid)
    cdt = grid.dtype
    rdt = _real_dtype(cdt)
    B, C = grid.shape[:2]
    K = grid.shape[2:]
    omega = np.asarray(omega)
    if omega.ndim == 3 and omega.shape[0] == 1:
        omega = omega[0]
    if omega.ndim == 3:
        if omega.shape[0] != B:
            raise ValueError("If omega has batch dim, omega batch dimension must match image.")
        return np.concatenate(
            [interp_forward(grid[b : b + 1], omega[b], tables, n_shift, numpoints, table_oversamp) for b in range(B)]
        )
    tabs = [np.asarray(t, dtype=cdt) for t in tables]
    tm = normalized_freq(omega, K, rdt)
    base = point_indices(tm, numpoints, rdt)
    flat = grid.reshape(B, C, -1)
    kdat = np.zeros((B, C, omega.shape[-1]), dtype=cdt)
    for off in _offsets(numpoints):
        coef, idx = coef_and_index(tm, base, off, tabs, numpoints, table_oversamp, K, False, rdt)
        kdat += coef * flat[:, :, idx]
    return kdat * fftshift_phase(omega, n_shift, rdt)


def interp_adjoint(
    kdata: np.ndarray,
    omega: np.ndarray,
    tables: List[np.ndarray],
    n_shift: Sequence[float],
    numpoints: Sequence[int],
    table_oversamp: Sequence[int],
    grid_size: Sequence[int],
) -> np.ndarray:
    """Adjoint table interpolation k-space -> grid (``table_interp_adjoint``, interp.py:587-726).

    kdata: (B, C, M) complex. Returns (B, C, *grid_size).
    """
    kdata = np.asarray(kdata)
    cdt = kdata.dtype
    rdt = _real_dtype(cdt)
    B, C, M = kdata.shape
    K = tuple(int(k) for k in grid_size)
    omega = np.asarray(omega)
    if omega.ndim == 3 and omega.shape[0] == 1:
        omega = omega[0]
    if omega.ndim == 3:
        if omega.shape[0] != B:
            raise ValueError("If omega has batch dim, omega batch dimension must match data.")
        return np.concatenate(
            [
                interp_adjoint(kdata[b : b + 1], omega[b], tables, n_shift, numpoints, table_oversamp, K)
                for b in range(B)
            ]
        )
    tabs = [np.asarray(t, dtype=cdt) for t in tables]
    tm = normalized_freq(omega, K, rdt)
    base = point_indices(tm, numpoints, rdt)
    nflat = int(np.prod(K))
    data = kdata * np.conj(fftshift_phase(omega, n_shift, rdt))
    acc_re = np.zeros((B, C, nflat), dtype=np.float64)
    acc_im = np.zeros((B, C, nflat), dtype=np.float64)
    for off in _offsets(numpoints):
        coef, idx = coef_and_index(tm, base, off, tabs, numpoints, table_oversamp, K, True, rdt)
        contrib = coef * data
        for b in range(B):
            for c in range(C):
                acc_re[b, c] += np.bincount(idx, weights=contrib[b, c].real, minlength=nflat)
                acc_im[b, c] += np.bincount(idx, weights=contrib[b, c].imag, minlength=nflat)
    return (acc_re + 1j * acc_im).astype(cdt).reshape((B, C) + K)


# ---------------------------------------------------------------------------
# FFT stages (H5 / H6 / H9)
# ---------------------------------------------------------------------------


def _check_norm(norm):
    if norm is not None and norm != "ortho":
        raise ValueError("Only option for norm is 'ortho'.")


def fft_and_scale(image, scaling_coef, im_size, grid_size, norm=None):
    """Scale, zero-pad at the end of each dim, unnormalised/ortho FFT (fft.py:35-76)."""
    _check_norm(norm)
    image = np.asarray(image)
    nd = len(im_size)
    pad = [(0, 0)] * (image.ndim - nd) + [(0, int(g) - int(n)) for g, n in zip(grid_size, im_size)]
    x = np.pad(image * np.asarray(scaling_coef, dtype=image.dtype), pad)
    out = np.fft.fftn(x, axes=tuple(range(-nd, 0)), norm="ortho" if norm == "ortho" else "backward")
    return out.astype(image.dtype)


def ifft_and_scale(grid, scaling_coef, im_size, grid_size, norm=None):
    """Unnormalised (or ortho) inverse FFT, crop to im_size, times conj(scaling) (fft.py:79-118)."""
    _check_norm(norm)
    grid = np.asarray(grid)
    nd = len(im_size)
    x = np.fft.ifftn(grid, axes=tuple(range(-nd, 0)), norm="ortho" if norm == "ortho" else "forward")
    sl = (Ellipsis,) + tuple(slice(0, int(n)) for n in im_size)
    return (x[sl] * np.conj(np.asarray(scaling_coef, dtype=grid.dtype))).astype(grid.dtype)


def fft_filter(image, kernel, norm="ortho"):
    """pad -> FFT -> * kernel -> IFFT -> crop (fft.py:121-173)."""
    _check_norm(norm)
    image = np.asarray(image)
    kernel = np.asarray(kernel)
    nd = image.ndim - 2
    im_size = image.shape[2:]
    grid_size = kernel.shape[-nd:]
    pad = [(0, 0), (0, 0)] + [(0, int(g) - int(n)) for g, n in zip(grid_size, im_size)]
    ax = tuple(range(-nd, 0))
    X = np.fft.fftn(np.pad(image, pad), axes=ax, norm="ortho" if norm == "ortho" else "backward")
    y = np.fft.ifftn(X * kernel, axes=ax, norm="ortho" if norm == "ortho" else "forward")
    sl = (Ellipsis,) + tuple(slice(0, int(n)) for n in im_size)
    return y[sl].astype(image.dtype)


# ---------------------------------------------------------------------------
# full operators (H7 / H11)
# ---------------------------------------------------------------------------


class Operator:
    """Geometry + precomputed buffers, built with the product's host setup.

    The host setup (tables, scaling) is itself checked against the reference
    in ``tests/test_host_setup.py``; the oracle reuses it so that both sides
    consume identical inputs.
    """

    def __init__(self, im_size, grid_size=None, numpoints=6, n_shift=None, table_oversamp=2**10,
                 kbwidth=2.34, order=0.0, cdtype=np.complex64):
        from torchkbnufft_gb300 import _setup as S

        (self.im_size, self.grid_size, self.numpoints, self.n_shift, self.table_oversamp, self.order,
         self.alpha, _, _) = S.validate_args(im_size, grid_size, numpoints, n_shift, table_oversamp, kbwidth, order)
        self.cdtype = np.dtype(cdtype)
        tabs = S.build_table(self.im_size, self.grid_size, self.numpoints, self.table_oversamp, self.order, self.alpha)
        self.tables = [t.numpy().astype(self.cdtype) for t in tabs]
        self.scaling = S.compute_scaling_coefs(self.im_size, self.grid_size, self.numpoints, self.alpha,
                                               self.order).numpy().astype(self.cdtype)
        self.n_shift = tuple(float(s) for s in self.n_shift)

    def interp(self, grid, omega):
        return interp_forward(grid, omega, self.tables, self.n_shift, self.numpoints, self.table_oversamp)

    def interp_adj(self, kdata, omega, grid_size=None):
        gs = self.grid_size if grid_size is None else grid_size
        return interp_adjoint(kdata, omega, self.tables, self.n_shift, self.numpoints, self.table_oversamp, gs)

    def forward(self, image, omega, smaps=None, norm=None):
        """``KbNufft.forward`` (modules/kbnufft.py:125-228)."""
        x = np.asarray(image)
        if smaps is not None:
            x = x * np.asarray(smaps)
        return self.interp(fft_and_scale(x, self.scaling, self.im_size, self.grid_size, norm), omega)

    def adjoint(self, kdata, omega, smaps=None, norm=None):
        """``KbNufftAdjoint.forward`` (modules/kbnufft.py:307-410)."""
        img = ifft_and_scale(self.interp_adj(kdata, omega), self.scaling, self.im_size, self.grid_size, norm)
        if smaps is not None:
            img = np.sum(img * np.conj(np.asarray(smaps)), axis=1, keepdims=True)
        return img


def toep_apply(image, kernel, smaps=None, norm=None):
    """``ToepNufft.forward`` (modules/kbnufft.py:441-547)."""
    image = np.asarray(image)
    kernel = np.asarray(kernel)
    nd = image.ndim - 2
    if kernel.ndim > nd and kernel.shape[0] == 1:
        kernel = kernel[0]
    if smaps is None:
        return fft_filter(image, kernel, norm)
    smaps = np.asarray(smaps)
    out = []
    for b in range(image.shape[0]):
        s = smaps[0 if smaps.shape[0] == 1 else b][None]
        k = kernel[b] if kernel.ndim > nd else kernel
        y = fft_filter(image[b][None] * s, k, norm)
        out.append(np.sum(y * np.conj(s), axis=1, keepdims=True)[0])
    return np.stack(out)


def toeplitz_kernel(omega, im_size, weights=None, norm=None, grid_size=None, numpoints=6,
                    table_oversamp=2**10, kbwidth=2.34, order=0.0, operator_cls=None):
    """``calc_toeplitz_kernel`` restated (``torchkbnufft/_nufft/toep.py:11-307``).

    ``operator_cls`` (default ``Operator``) supplies the interpolation; the
    CPU port's subclass runs it in C for benchmark-size trajectories."""
    operator_cls = Operator if operator_cls is None else operator_cls
    omega = np.asarray(omega)
    if omega.ndim == 3:
        ks = []
        for i in range(omega.shape[0]):
            w = None if weights is None else np.asarray(weights)[i]
            ks.append(toeplitz_kernel(omega[i], im_size, w, norm, grid_size, numpoints, table_oversamp,
                                      kbwidth, order, operator_cls))
        return np.stack(ks)
    rdt = omega.dtype
    cdt = np.complex64 if rdt == np.float32 else np.complex128
    nd = omega.shape[0]
    op = operator_cls(im_size, grid_size, numpoints, [0] * nd, table_oversamp, kbwidth, order, cdt)
    if weights is None:
        w = np.ones((1, 1, omega.shape[-1]), dtype=cdt)
    else:
        w = np.asarray(weights).astype(cdt)[None]

    def flip_concat(dim, om):
        axis = dim + 2
        flip = np.ones((nd, 1), dtype=rdt)
        flip[dim] = -1
        if dim < nd - 1:
            k1 = flip_concat(dim + 1, om)
            k2 = flip_concat(dim + 1, flip * om)
        else:
            k1 = op.adjoint(w, om, norm=norm)
            k2 = op.adjoint(w, (flip * om).astype(rdt), norm=norm)
        zshape = list(k1.shape)
        zshape[axis] = 1
        k2 = np.take(k2, np.arange(1, k2.shape[axis]), axis=axis)
        return np.concatenate((k1, np.zeros(zshape, dtype=k1.dtype), np.flip(k2, axis=axis)), axis=axis)

    kern = flip_concat(1, omega) if nd > 1 else op.adjoint(w, omega, norm=norm)
    # reflect-conjugate along dim 2 (toep.py:240-274)
    tmp = np.conj(kern)
    for d in range(2, kern.ndim):
        tmp = np.take(tmp, np.mod(-np.arange(tmp.shape[d]), tmp.shape[d]), axis=d)
    zshape = list(kern.shape)
    zshape[2] = 1
    tmp = np.concatenate((np.zeros(zshape, dtype=kern.dtype), np.take(tmp, np.arange(1, tmp.shape[2]), axis=2)), axis=2)
    kern = np.concatenate((kern, tmp), axis=2)
    # hermitify (toep.py:277-307)
    rev = kern
    for d in range(2, kern.ndim):
        rev = np.take(rev, np.mod(-np.arange(rev.shape[d]), rev.shape[d]), axis=d)
    kern = (kern + np.conj(rev)) / 2
    im = np.asarray(op.im_size)
    gs = np.asarray(op.grid_size)
    if norm == "ortho":
        scale = np.sqrt(np.prod(2 * im) / np.prod(gs))
    else:
        scale = 1 / np.prod(2 * im)
    ax = tuple(range(-nd, 0))
    out = np.fft.fftn(kern, axes=ax, norm="ortho" if norm == "ortho" else "backward")[0, 0] * scale
    return out.astype(cdt)


def density_compensation(ktraj, im_size, num_iterations=10, grid_size=None, numpoints=6, n_shift=None,
                         table_oversamp=2**10, kbwidth=2.34, order=0.0, operator_cls=None):
    """Pipe iteration ``w <- w / |A A^H w|`` (``torchkbnufft/_nufft/dcomp.py:10-119``).

    ``operator_cls`` as in ``toeplitz_kernel``."""
    operator_cls = Operator if operator_cls is None else operator_cls
    ktraj = np.asarray(ktraj)
    B = 1
    if ktraj.ndim == 3:
        if ktraj.shape[0] == 1:
            ktraj = ktraj[0]
        else:
            B = ktraj.shape[0]
    cdt = np.complex64 if ktraj.dtype == np.float32 else np.complex128
    op = operator_cls(im_size, grid_size, numpoints, n_shift, table_oversamp, kbwidth, order, cdt)
    sig = np.ones((B, 1, ktraj.shape[-1]), dtype=cdt)
    for _ in range(num_iterations):
        sig = sig / np.abs(op.interp(op.interp_adj(sig, ktraj), ktraj))
    return sig.astype(cdt)


# ---------------------------------------------------------------------------
# smooth operators for gradient checks and the FP64 NDFT oracle
# ---------------------------------------------------------------------------


def exact_kb_interp(grid, omega, im_size, numpoints=6, n_shift=None, kbwidth=2.34, order=0.0):
    """Interpolation with the KB kernel evaluated exactly (no table), complex128.

    This is the smooth operator the table approximates (the reference's
    sparse-matrix path builds the same coefficients, ``utils.py:16-119``); its
    derivative in ``omega`` is well defined, so central finite differences of
    it check a trajectory gradient.
    """
    from torchkbnufft_gb300 import _setup as S

    grid = np.asarray(grid, dtype=np.complex128)
    omega = np.asarray(omega, dtype=np.float64)
    K = grid.shape[2:]
    nd = len(K)
    J = (numpoints,) * nd if isinstance(numpoints, int) else tuple(numpoints)
    if n_shift is None:
        n_shift = tuple(n // 2 for n in im_size)
    alpha = [kbwidth * j for j in J]
    tm = omega / (2 * np.pi / np.asarray(K, dtype=np.float64).reshape(-1, 1))
    base = (1 + np.floor(tm - np.asarray(J).reshape(-1, 1) / 2)).astype(np.int64)
    flat = grid.reshape(grid.shape[0], grid.shape[1], -1)
    out = np.zeros(grid.shape[:2] + (omega.shape[-1],), dtype=np.complex128)
    for off in _offsets(J):
        coef = np.ones(omega.shape[-1], dtype=np.complex128)
        idx = np.zeros(omega.shape[-1], dtype=np.int64)
        for d in range(nd):
            g = base[d] + off[d]
            u = tm[d] - g
            rate = S.table_phase_rate(im_size[d], K[d])
            coef = coef * S.kb_kernel(u, J[d], alpha[d], order) * np.exp(-1j * rate * u)
            stride = int(np.prod(K[d + 1 :])) if d + 1 < nd else 1
            idx = idx + np.mod(g, K[d]) * stride
        out += coef * flat[:, :, idx]
    phase = np.exp(1j * np.sum(omega * np.asarray(n_shift, dtype=np.float64).reshape(-1, 1), axis=0))
    return out * phase


def ndft_forward(image: np.ndarray, omega: np.ndarray) -> np.ndarray:
    """Direct NDFT ``y_m = sum_n x[n] exp(-1j * omega_m . (n - N//2))`` in complex128.

    image: (B, C, *N); omega: (d, M). Cost O(M * prod(N)); callers subsample M.
    """
    image = np.asarray(image, dtype=np.complex128)
    omega = np.asarray(omega, dtype=np.float64)
    N = image.shape[2:]
    coords = [np.arange(n) - n // 2 for n in N]
    flat = image.reshape(image.shape[0], image.shape[1], -1)
    grids = np.meshgrid(*coords, indexing="ij")
    pos = np.stack([g.reshape(-1) for g in grids])  # (d, P)
    out = np.empty(image.shape[:2] + (omega.shape[-1],), dtype=np.complex128)
    chunk = max(1, int(2**22 // pos.shape[1]))
    for s in range(0, omega.shape[-1], chunk):
        ph = np.exp(-1j * (omega[:, s : s + chunk].T @ pos))  # (m, P)
        out[:, :, s : s + chunk] = flat @ ph.T
    return out


def ndft_forward_separable(image: np.ndarray, omega: np.ndarray, chunk: int = 512) -> np.ndarray:
    """The same NDFT as ``ndft_forward`` for one (N...) plane, contracted one
    dim at a time: the last dim by a matrix product with its phases
    ``exp(-1j * omega_d (n_d - N_d//2))``, then each earlier dim by a weighted
    sum. Cost O(M * prod(N)) multiply-adds in one BLAS call per chunk of
    points, so 3D images on thousands of points take seconds. Returns (M,)."""
    x = np.asarray(image, dtype=np.complex128)
    omega = np.asarray(omega, dtype=np.float64)
    N = x.shape
    nd = len(N)
    out = np.empty(omega.shape[-1], dtype=np.complex128)
    phases = lambda d, om: np.exp(-1j * om[:, None] * (np.arange(N[d]) - N[d] // 2)[None, :])  # (m, N_d)
    for s in range(0, omega.shape[-1], chunk):
        om = omega[:, s : s + chunk]
        t = x.reshape(-1, N[-1]) @ phases(nd - 1, om[nd - 1]).T  # (prod N[:-1], m)
        for d in range(nd - 2, -1, -1):
            t = np.einsum("...nm,mn->...m", t.reshape(N[:d] + (N[d], t.shape[-1])), phases(d, om[d]))
        out[s : s + chunk] = t.reshape(-1)
    return out


def _exact_coefs(omega, K, im_size, numpoints, kbwidth, order):
    """Per-offset exact-KB coefficients and flat indices (complex128)."""
    from torchkbnufft_gb300 import _setup as S

    nd = len(K)
    J = (numpoints,) * nd if isinstance(numpoints, int) else tuple(numpoints)
    alpha = [kbwidth * j for j in J]
    tm = omega / (2 * np.pi / np.asarray(K, dtype=np.float64).reshape(-1, 1))
    base = (1 + np.floor(tm - np.asarray(J).reshape(-1, 1) / 2)).astype(np.int64)
    for off in _offsets(J):
        coef = np.ones(omega.shape[-1], dtype=np.complex128)
        idx = np.zeros(omega.shape[-1], dtype=np.int64)
        for d in range(nd):
            g = base[d] + off[d]
            u = tm[d] - g
            rate = S.table_phase_rate(im_size[d], K[d])
            coef = coef * S.kb_kernel(u, J[d], alpha[d], order) * np.exp(-1j * rate * u)
            stride = int(np.prod(K[d + 1 :])) if d + 1 < nd else 1
            idx = idx + np.mod(g, K[d]) * stride
        yield coef, idx


def exact_kb_interp_adjoint(kdata, omega, grid_size, im_size, numpoints=6, n_shift=None, kbwidth=2.34, order=0.0):
    """Adjoint of :func:`exact_kb_interp` (complex128)."""
    kdata = np.asarray(kdata, dtype=np.complex128)
    omega = np.asarray(omega, dtype=np.float64)
    K = tuple(int(k) for k in grid_size)
    if n_shift is None:
        n_shift = tuple(n // 2 for n in im_size)
    phase = np.exp(-1j * np.sum(omega * np.asarray(n_shift, dtype=np.float64).reshape(-1, 1), axis=0))
    data = kdata * phase
    B, C, M = kdata.shape
    out = np.zeros((B, C, int(np.prod(K))), dtype=np.complex128)
    for coef, idx in _exact_coefs(omega, K, im_size, numpoints, kbwidth, order):
        contrib = np.conj(coef) * data
        for b in range(B):
            for c in range(C):
                out[b, c] += np.bincount(idx, weights=contrib[b, c].real, minlength=out.shape[-1]) + 1j * np.bincount(
                    idx, weights=contrib[b, c].imag, minlength=out.shape[-1])
    return out.reshape((B, C) + K)


def exact_nufft_forward(image, omega, im_size, grid_size=None, smaps=None, norm=None, numpoints=6, kbwidth=2.34,
                        order=0.0):
    """Forward NUFFT with the exact KB kernel (smooth in omega), complex128."""
    from torchkbnufft_gb300 import _setup as S

    nd = len(im_size)
    grid_size = tuple(2 * n for n in im_size) if grid_size is None else tuple(grid_size)
    J = (numpoints,) * nd
    alpha = tuple(kbwidth * j for j in J)
    scaling = S.compute_scaling_coefs(im_size, grid_size, J, alpha, (order,) * nd).numpy()
    x = np.asarray(image, dtype=np.complex128)
    if smaps is not None:
        x = x * np.asarray(smaps)
    grid = fft_and_scale(x, scaling, im_size, grid_size, norm)
    return exact_kb_interp(grid, omega, im_size, numpoints, None, kbwidth, order)


def exact_nufft_adjoint(kdata, omega, im_size, grid_size=None, smaps=None, norm=None, numpoints=6, kbwidth=2.34,
                        order=0.0):
    """Adjoint NUFFT with the exact KB kernel, complex128."""
    from torchkbnufft_gb300 import _setup as S

    nd = len(im_size)
    grid_size = tuple(2 * n for n in im_size) if grid_size is None else tuple(grid_size)
    J = (numpoints,) * nd
    alpha = tuple(kbwidth * j for j in J)
    scaling = S.compute_scaling_coefs(im_size, grid_size, J, alpha, (order,) * nd).numpy()
    grid = exact_kb_interp_adjoint(kdata, omega, grid_size, im_size, numpoints, None, kbwidth, order)
    img = ifft_and_scale(grid, scaling, im_size, grid_size, norm)
    if smaps is not None:
        img = np.sum(img * np.conj(np.asarray(smaps)), axis=1, keepdims=True)
    return img
