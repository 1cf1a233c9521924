"""Tensor-level wrappers of the C ABI: geometry, caches, launches.

Everything here takes and returns CUDA tensors and enqueues work on torch's
current stream. Inputs on the CPU raise: this package has no CPU path.

Caches (per process):

* geometry: parsed once per set of module buffers (reading CUDA buffers with
  ``tolist()`` would synchronise the device on every call);
* trajectory layouts (bin-sorted points): keyed by the omega tensor object,
  its version counter, shape and the geometry, so a trajectory that is
  modified in place or freed is never reused. A miss for a trajectory drops
  its entries of older versions (an optimiser stepping omega in place keeps
  one layout, not one per step), an entry goes when its trajectory is freed,
  and the cache holds at most ``TKBN_LAYOUT_CACHE_BYTES`` of workspaces
  (default 4 GiB; the newest layout is always kept) and 128 entries;
* cuFFT plans: keyed by geometry, batch*coils and device.
"""

from __future__ import annotations

import collections
import ctypes
import os
import threading
import weakref
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib as L

_lock = threading.RLock()


# ---------------------------------------------------------------- checks


def require_cuda(*tensors: Optional[torch.Tensor]) -> torch.device:
    dev = None
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise RuntimeError(
                "torchkbnufft_gb300 runs on CUDA devices only; got a tensor on "
                f"{t.device}. Move inputs and the module to a CUDA device."
            )
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise RuntimeError(f"tensors are on different devices: {dev} and {t.device}")
    return dev


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.complex64:
        return L.TKBN_C64
    if dtype == torch.complex128:
        return L.TKBN_C128
    raise TypeError(f"unsupported dtype {dtype}: use complex64 or complex128")


def real_of(dtype: torch.dtype) -> torch.dtype:
    return torch.float32 if dtype == torch.complex64 else torch.float64


def norm_code(norm: Optional[str]) -> int:
    if norm is None:
        return L.TKBN_NORM_NONE
    if norm == "ortho":
        return L.TKBN_NORM_ORTHO
    raise ValueError("Only option for norm is 'ortho'.")


# ---------------------------------------------------------------- geometry


@dataclass(frozen=True)
class GeomKey:
    ndim: int
    dtype: int
    im_size: Tuple[int, ...]
    grid_size: Tuple[int, ...]
    numpoints: Tuple[int, ...]
    table_oversamp: Tuple[int, ...]
    n_shift: Tuple[float, ...]

    def struct(self) -> L.Geometry:
        g = L.Geometry()
        g.ndim = self.ndim
        g.dtype = self.dtype
        for d in range(self.ndim):
            g.im_size[d] = self.im_size[d]
            g.grid_size[d] = self.grid_size[d]
            g.numpoints[d] = self.numpoints[d]
            g.table_oversamp[d] = self.table_oversamp[d]
            g.n_shift[d] = self.n_shift[d]
        return g


_geom_structs: dict = {}


def geom_struct(key: GeomKey, flags: int = 0) -> L.Geometry:
    s = _geom_structs.get((key, flags))
    if s is None:
        s = key.struct()
        s.flags = flags
        _geom_structs[(key, flags)] = s
    return s


def _as_tuple(x, cast) -> Tuple:
    if isinstance(x, torch.Tensor):
        return tuple(cast(v) for v in x.reshape(-1).tolist())
    if isinstance(x, (list, tuple)):
        return tuple(cast(v) for v in x)
    return (cast(x),)


_param_cache: "collections.OrderedDict" = collections.OrderedDict()


def host_values(t, cast) -> Tuple:
    """Host copy of a small parameter tensor, cached by object identity + version."""
    if not isinstance(t, torch.Tensor):
        return _as_tuple(t, cast)
    key = (id(t), t._version, t.data_ptr(), tuple(t.shape), cast)
    with _lock:
        hit = _param_cache.get(key)
        if hit is not None and hit[0]() is t:
            return hit[1]
        vals = _as_tuple(t, cast)
        _param_cache[key] = (weakref.ref(t), vals)
        while len(_param_cache) > 256:
            _param_cache.popitem(last=False)
        return vals


def make_geom(dtype, im_size, grid_size, numpoints, table_oversamp, n_shift) -> GeomKey:
    grid = host_values(grid_size, int)
    ndim = len(grid)
    im = host_values(im_size, int) if im_size is not None else grid
    J = host_values(numpoints, int)
    Lo = host_values(table_oversamp, int)
    ns = host_values(n_shift, float)
    if len(J) == 1 and ndim > 1:
        J = J * ndim
    if len(Lo) == 1 and ndim > 1:
        Lo = Lo * ndim
    if not (len(im) == len(J) == len(Lo) == len(ns) == ndim):
        raise ValueError("im_size, grid_size, numpoints, table_oversamp and n_shift must have one entry per dim")
    if ndim not in (1, 2, 3):
        raise ValueError("only 1D, 2D and 3D transforms are supported")
    return GeomKey(ndim, dtype_code(dtype), im, grid, J, Lo, ns)


# ---------------------------------------------------------------- trajectory layout


class PointsLayout:
    """Bin-sorted trajectory (K1) in a torch-owned workspace."""

    def __init__(self, geom: GeomKey, omega: torch.Tensor, tile=None, chunk: int = 0,
                 deterministic: Optional[bool] = None):
        require_cuda(omega)
        self.geom = geom
        if deterministic is None:
            deterministic = torch.are_deterministic_algorithms_enabled()
        # geometry flags every call with this layout must carry
        self.flags = L.TKBN_ADJ_DETERMINISTIC if deterministic else 0
        self.device = omega.device
        self.ntraj = 1 if omega.ndim == 2 else omega.shape[0]
        self.npts = omega.shape[-1]
        self.desc = L.PointsDesc()
        self.desc.npts = self.npts
        self.desc.ntraj = self.ntraj
        if tile is not None:
            for d, t in enumerate(tile):
                self.desc.tile[d] = int(t)
        self.desc.chunk = int(chunk)
        g = geom_struct(geom, self.flags)
        nbytes = ctypes.c_size_t(0)
        L.check(L.lib().tkbn_points_workspace_size(ctypes.byref(g), ctypes.byref(self.desc), ctypes.byref(nbytes)))
        self.nbytes = int(nbytes.value)
        self.workspace = torch.empty(self.nbytes, dtype=torch.uint8, device=self.device)
        om = omega.detach().to(real_of(torch.complex64 if geom.dtype == L.TKBN_C64 else torch.complex128)).contiguous()
        self._omega_keepalive = om
        # (tables, their versions, table flags) whose per-point table factors
        # the workspace holds, or None; the tables are kept alive, so identity
        # and version pin their contents
        self._factors = None
        L.check(
            L.lib().tkbn_points_build(ctypes.byref(g), ctypes.byref(self.desc), om.data_ptr(),
                                      self.workspace.data_ptr(), self.nbytes, stream_handle(self.device))
        )
        # cross-stream ordering: the build's stream, an event after the build,
        # the streams already ordered after it, and the stream of the last
        # interpolation call (forward and adjoint calls may write the per-point
        # factor scratch in the workspace)
        build_stream = torch.cuda.current_stream(self.device)
        self._built = None
        self._ready_streams = {build_stream.cuda_stream}
        self._factor_stream = build_stream
        if not stream_capturing(self.device):
            self._built = torch.cuda.Event()
            self._built.record(build_stream)

    def stream_for_call(self, writes_factors: bool) -> int:
        """Orders a call on torch's current stream after the work it depends on
        and returns that stream's handle.

        Every call waits (once per stream) for the layout build when it runs
        on another stream than the build, and the workspace is marked as used
        by that stream, so the caching allocator keeps it until the stream's
        work is done even after the layout is evicted. Forward and adjoint
        interpolation calls (``writes_factors``) also wait for the last such
        call on this layout when that ran on another stream: they write and
        read the per-point factor scratch. Trajectory-gradient calls only read
        what the build wrote. Under CUDA graph capture nothing is added (a
        captured sequence is ordered by its own stream)."""
        s = torch.cuda.current_stream(self.device)
        h = s.cuda_stream
        if stream_capturing(self.device):
            return h
        with _lock:
            if h not in self._ready_streams:
                if self._built is not None:
                    s.wait_event(self._built)
                self.workspace.record_stream(s)
                self._ready_streams.add(h)
            if writes_factors:
                prev = self._factor_stream
                if prev is not None and prev.cuda_stream != h:
                    ev = torch.cuda.Event()
                    ev.record(prev)
                    s.wait_event(ev)
                self._factor_stream = s
        return h

    def factor_call(self, tables: Sequence[torch.Tensor], table_flags: int, call) -> None:
        """Runs ``call(flags)``, a forward or adjoint entry point on this layout's
        workspace (either may fill the per-point factor scratch), with the
        layout's flags and TKBN_ADJ_REUSE_FACTORS when the workspace holds the
        factors of these same, unmodified table tensors. The record
        and the enqueue happen under one lock, so threads sharing a cached
        layout keep the record in the order their calls reach the stream.

        Under CUDA graph capture nothing runs when it is enqueued, so a captured
        call always recomputes the factors (the graph carries its own pre-pass)
        and leaves no record behind for the calls after it."""
        with _lock:
            capturing = stream_capturing(self.device)
            flags = table_flags | self.flags
            if not capturing and factors_reusable(self._factors, tables, table_flags):
                flags |= L.TKBN_ADJ_REUSE_FACTORS
            self._factors = None
            call(flags)
            if not capturing:
                self._factors = (tuple(tables), tuple(t._version for t in tables), table_flags)


def stream_capturing(device: torch.device) -> bool:
    """Whether torch's current stream on ``device`` is capturing a CUDA graph.
    A query that fails reads as not capturing (the eager behaviour)."""
    try:
        if device.index is None or device.index == torch.cuda.current_device():
            return bool(torch.cuda.is_current_stream_capturing())
        with torch.cuda.device(device):
            return bool(torch.cuda.is_current_stream_capturing())
    except (AttributeError, RuntimeError):
        return False


def factors_reusable(stored, tables: Sequence[torch.Tensor], table_flags: int) -> bool:
    """True when ``stored`` (tables, versions, flags) names tables with these
    contents, none modified since, with the same table flags. A table tensor
    other than the stored one counts when its contents are equal (a forward and
    an adjoint module hold separate copies of the same tables); that comparison
    is cached per pair of tensors and versions."""
    if stored is None:
        return False
    tabs, versions, flags = stored
    if flags != table_flags or len(tabs) != len(tables):
        return False
    for a, b, v in zip(tabs, tables, versions):
        if a._version != v:
            return False
        if a is b:
            continue
        same = _cached_prop(("eq", id(b), b._version, b.data_ptr(), a.data_ptr(), a._version), b,
                            lambda: (a.shape == b.shape and a.dtype == b.dtype and a.device == b.device
                                     and bool(torch.equal(a, b))))
        if not same:
            return False
    return True


_layout_cache: "collections.OrderedDict" = collections.OrderedDict()
_LAYOUT_CACHE_MAX = 128


def _layout_cache_bytes_max() -> int:
    try:
        return int(os.environ.get("TKBN_LAYOUT_CACHE_BYTES", 4 << 30))
    except ValueError:
        return 4 << 30


def _drop_layouts_of(base_id: int, keep_key=None) -> None:
    """Drops every cached layout of the trajectory object ``base_id`` except ``keep_key``."""
    for k in [k for k in _layout_cache if k[0] == base_id and k != keep_key]:
        del _layout_cache[k]


def _on_trajectory_freed(base_id: int):
    def cb(_ref):
        with _lock:
            _drop_layouts_of(base_id)
    return cb


def points_layout(geom: GeomKey, omega: torch.Tensor, tile=None, chunk: int = 0,
                  deterministic: Optional[bool] = None) -> PointsLayout:
    """Cached layout of omega. ``deterministic`` (default: torch's deterministic-algorithms
    setting) builds it without split adjoint tiles, so adjoints are bitwise repeatable."""
    if deterministic is None:
        deterministic = torch.are_deterministic_algorithms_enabled()
    base = omega._base if omega._base is not None else omega
    key = (id(base), omega.data_ptr(), omega._version, tuple(omega.shape), tuple(omega.stride()), omega.dtype,
           geom, tuple(tile) if tile else None, chunk, omega.device, bool(deterministic))
    with _lock:
        hit = _layout_cache.get(key)
        if hit is not None and hit[0]() is base:
            _layout_cache.move_to_end(key)
            return hit[1]
        # entries of this trajectory object at another version or storage can
        # never be hit again (versions only grow); entries of a dead object
        # whose id was reused are dropped as well
        stale = [k for k, v in _layout_cache.items() if k[0] == id(base) and
                 (v[0]() is not base or k[1] != key[1] or k[2] != key[2])]
        for k in stale:
            del _layout_cache[k]
        lay = PointsLayout(geom, omega, tile, chunk, deterministic)
        _layout_cache[key] = (weakref.ref(base, _on_trajectory_freed(id(base))), lay)
        cap = _layout_cache_bytes_max()
        total = sum(v[1].nbytes for v in _layout_cache.values())
        while len(_layout_cache) > 1 and (len(_layout_cache) > _LAYOUT_CACHE_MAX or total > cap):
            _, (_, old) = _layout_cache.popitem(last=False)
            total -= old.nbytes
        return lay


def layout_cache_info() -> Tuple[int, int]:
    """(entries, workspace bytes) held by the layout cache."""
    with _lock:
        return len(_layout_cache), sum(v[1].nbytes for v in _layout_cache.values())


def clear_caches() -> None:
    with _lock:
        _layout_cache.clear()
        _param_cache.clear()
        for p in list(_fft_cache.values()):
            p.destroy()
        _fft_cache.clear()


# ---------------------------------------------------------------- FFT plans


class FFTPlan:
    def __init__(self, geom: GeomKey, batch: int, coils: int, device: torch.device):
        self.handle = ctypes.c_void_p()
        self.geom = geom
        with torch.cuda.device(device):
            L.check(L.lib().tkbn_fft_plan_create(ctypes.byref(geom_struct(geom)), batch, coils, ctypes.byref(self.handle)))

    def destroy(self):
        if self.handle:
            L.lib().tkbn_fft_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()


_fft_cache: "collections.OrderedDict" = collections.OrderedDict()
_FFT_CACHE_MAX = 128


def fft_plan(geom: GeomKey, batch: int, coils: int, device: torch.device) -> FFTPlan:
    # plans depend on grid size, batch and dtype only
    key = (geom.ndim, geom.dtype, geom.grid_size, batch * coils, device)
    with _lock:
        p = _fft_cache.get(key)
        if p is None:
            g2 = GeomKey(geom.ndim, geom.dtype, geom.grid_size, geom.grid_size, geom.numpoints, geom.table_oversamp,
                         geom.n_shift)
            p = FFTPlan(g2, batch * coils, 1, device)
            _fft_cache[key] = p
            while len(_fft_cache) > _FFT_CACHE_MAX:
                _fft_cache.popitem(last=False)[1].destroy()
        else:
            _fft_cache.move_to_end(key)
        return p


def _plan_geom(geom: GeomKey, plan: FFTPlan, B: int, C: int) -> Tuple[L.Geometry, int, int]:
    """The C API checks the plan batch against B*C; plans are cached by B*C."""
    return geom_struct(geom), B * C, 1


# ---------------------------------------------------------------- tables


_table_props: "collections.OrderedDict" = collections.OrderedDict()


def _cached_prop(key, t, fn):
    with _lock:
        hit = _table_props.get(key)
        if hit is not None and hit[0]() is t:
            return hit[1]
    v = fn()
    with _lock:
        _table_props[key] = (weakref.ref(t), v)
        while len(_table_props) > 64:
            _table_props.popitem(last=False)
    return v


def _conj_symmetric(t: torch.Tensor) -> bool:
    """table[c + k] == conj(table[c - k]) bitwise (c = (len - 1) / 2)."""
    n = t.numel()
    if n % 2 == 0:
        return False
    c = (n - 1) // 2
    return _cached_prop(("sym", id(t), t._version, t.data_ptr()), t,
                        lambda: bool(torch.equal(t[c + 1:], t[:c].flip(0).conj())))


def _linear_phase(t: torch.Tensor) -> bool:
    """|t[k]| exp(i c (k - center) / L) == t[k] to within float rounding, c from the
    entry L/2 past the centre (the device fits c by least squares over the entries
    with u in (0, 1]); L = (len - 1) / J is not known here, so every even L dividing
    len - 1 into J = 2..8 is tried."""

    def check() -> bool:
        if not t.is_complex() or t.dtype != torch.complex64:
            return False
        h = t.detach().cpu().numpy().astype(np.complex128)
        n = h.size
        if n < 3 or n % 2 == 0:
            return False
        center = (n - 1) // 2
        scale = float(np.max(np.abs(h)))
        if scale == 0.0:
            return False
        for J in range(2, 9):
            if (n - 1) % J or ((n - 1) // J) % 2:
                continue
            L = (n - 1) // J
            c = 2.0 * np.angle(h[center + L // 2])
            u = (np.arange(n) - center) / L
            if np.max(np.abs(h - np.abs(h) * np.exp(1j * c * u))) <= 1e-6 * scale:
                return True
        return False

    return _cached_prop(("lin", id(t), t._version, t.data_ptr()), t, check)


def table_ptrs(tables: Sequence[torch.Tensor], dtype: torch.dtype):
    """Device pointers of the per-dim tables, the tensors kept alive, and geometry flags.

    Tables with identical contents share one pointer (one cache footprint);
    when every table is exactly conjugate-symmetric the kernels read half of it.
    """
    keep = []
    for t in tables:
        require_cuda(t)
        if t.dtype != dtype:
            t = t.to(dtype)
        keep.append(t.contiguous())
    ptrs = [t.data_ptr() for t in keep]
    for d in range(1, len(keep)):
        a, b = keep[0], keep[d]
        if a.shape == b.shape and ptrs[d] != ptrs[0]:
            same = _cached_prop(("eq", id(b), b._version, b.data_ptr(), a.data_ptr(), a._version), b,
                                lambda: bool(torch.equal(a, b)))
            if same:
                ptrs[d] = ptrs[0]
    flags = L.TKBN_TABLES_CONJ_SYMMETRIC if all(_conj_symmetric(t) for t in keep) else 0
    if all(_linear_phase(t) for t in keep):
        flags |= L.TKBN_TABLES_LINEAR_PHASE
    return L.ptr_array(ptrs), keep, flags


_dtable_cache: "collections.OrderedDict" = collections.OrderedDict()


def derivative_tables(tables: Sequence[torch.Tensor], table_oversamp: Sequence[int]) -> List[torch.Tensor]:
    """d/du of each table by central differences on the table grid (step 1/L).

    Error O(1/L^2) relative inside the support. Cached by table identity.
    """
    out = []
    for t, Lo in zip(tables, table_oversamp):
        key = (id(t), t._version, t.data_ptr(), int(Lo))
        with _lock:
            hit = _dtable_cache.get(key)
            if hit is not None and hit[0]() is t:
                out.append(hit[1])
                continue
        # entries 0 and J*L sit at u = -+J/2 where the truncated kernel is set to
        # zero; the two end bins use one-sided differences of interior entries.
        d = torch.empty_like(t)
        d[1:-1] = (t[2:] - t[:-2]) * (Lo / 2.0)
        d[0] = d[1] = (t[2] - t[1]) * Lo
        d[-1] = d[-2] = (t[-2] - t[-3]) * Lo
        with _lock:
            _dtable_cache[key] = (weakref.ref(t), d)
            while len(_dtable_cache) > 32:
                _dtable_cache.popitem(last=False)
        out.append(d)
    return out


# ---------------------------------------------------------------- launches


def _c(t: Optional[torch.Tensor]) -> int:
    return 0 if t is None else t.data_ptr()


def interp_fwd(geom: GeomKey, lay: PointsLayout, tables, grid: torch.Tensor) -> torch.Tensor:
    """kdata (B, C, M) = table interpolation of grid (B, C, *K)."""
    dev = require_cuda(grid)
    grid = grid.contiguous()
    B, C = grid.shape[:2]
    kdata = torch.empty((B, C, lay.npts), dtype=grid.dtype, device=dev)
    tp, keep, fl = table_ptrs(tables, grid.dtype)
    lay.factor_call(keep, fl, lambda flags: L.check(L.lib().tkbn_interp_fwd(
        ctypes.byref(geom_struct(geom, flags)), ctypes.byref(lay.desc), lay.workspace.data_ptr(), tp,
        grid.data_ptr(), B, C, kdata.data_ptr(), lay.stream_for_call(True))))
    return kdata


def interp_adj(geom: GeomKey, lay: PointsLayout, tables, kdata: torch.Tensor) -> torch.Tensor:
    """grid (B, C, *K) = adjoint table interpolation of kdata (B, C, M)."""
    dev = require_cuda(kdata)
    kdata = kdata.contiguous()
    B, C = kdata.shape[:2]
    grid = torch.empty((B, C) + geom.grid_size, dtype=kdata.dtype, device=dev)
    tp, keep, fl = table_ptrs(tables, kdata.dtype)
    lay.factor_call(keep, fl, lambda flags: L.check(L.lib().tkbn_interp_adj(
        ctypes.byref(geom_struct(geom, flags)), ctypes.byref(lay.desc), lay.workspace.data_ptr(), tp,
        kdata.data_ptr(), B, C, grid.data_ptr(), lay.stream_for_call(True))))
    return grid


def interp_grad_omega(geom: GeomKey, lay: PointsLayout, tables, grid: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """(T, d, M) real: Re sum_{b,c} conj(v) * d interp(grid) / d omega."""
    dev = require_cuda(grid, v)
    grid = grid.contiguous()
    v = v.contiguous()
    B, C = grid.shape[:2]
    rd = real_of(grid.dtype)
    grad = torch.empty((lay.ntraj, geom.ndim, lay.npts), dtype=rd, device=dev)
    tabs = [t.to(grid.dtype).contiguous() for t in tables]
    dtabs = derivative_tables(tabs, geom.table_oversamp)
    tp, keep, fl = table_ptrs(tabs, grid.dtype)
    dp, keep2, _ = table_ptrs(dtabs, grid.dtype)
    L.check(L.lib().tkbn_interp_grad_omega(ctypes.byref(geom_struct(geom, lay.flags)), ctypes.byref(lay.desc),
                                           lay.workspace.data_ptr(), tp, dp, grid.data_ptr(), v.data_ptr(), B, C,
                                           grad.data_ptr(), lay.stream_for_call(False)))
    return grad


def fft_and_scale(geom: GeomKey, image: torch.Tensor, smaps: Optional[torch.Tensor], scaling: Optional[torch.Tensor],
                  norm: Optional[str], coils: Optional[int] = None) -> torch.Tensor:
    """grid (B, C, *K) = FFT(pad(image [* smaps] * scaling))."""
    dev = require_cuda(image, smaps, scaling)
    image = image.contiguous()
    B = image.shape[0]
    C = smaps.shape[1] if smaps is not None else image.shape[1]
    sb = 0
    if smaps is not None:
        smaps = smaps.to(image.dtype).contiguous()
        sb = smaps.shape[0]
    if scaling is not None:
        scaling = scaling.to(image.dtype).contiguous()
    plan = fft_plan(geom, B, C, dev)
    grid = torch.empty((B, C) + geom.grid_size, dtype=image.dtype, device=dev)
    g, pb, pc = _plan_geom(geom, plan, B, C)
    # the plan's batch is B*C; pass the true (B, C) to the kernels
    L.check(L.lib().tkbn_fft_and_scale(ctypes.byref(g), plan.handle, image.data_ptr(), _c(smaps), sb, _c(scaling),
                                       B, C, norm_code(norm), grid.data_ptr(), stream_handle(dev)))
    return grid


def ifft_and_scale(geom: GeomKey, grid: torch.Tensor, smaps: Optional[torch.Tensor], scaling: Optional[torch.Tensor],
                   norm: Optional[str], overwrite: bool = False) -> torch.Tensor:
    """image = [sum_c conj(smaps) *] conj(scaling) * crop(IFFT(grid)); grid is clobbered if overwrite."""
    dev = require_cuda(grid, smaps, scaling)
    B, C = grid.shape[:2]
    work = grid.contiguous() if overwrite else grid.contiguous().clone()
    sb = 0
    if smaps is not None:
        smaps = smaps.to(grid.dtype).contiguous()
        sb = smaps.shape[0]
    if scaling is not None:
        scaling = scaling.to(grid.dtype).contiguous()
    plan = fft_plan(geom, B, C, dev)
    co = 1 if smaps is not None else C
    out = torch.empty((B, co) + geom.im_size, dtype=grid.dtype, device=dev)
    L.check(L.lib().tkbn_ifft_and_scale(ctypes.byref(geom_struct(geom)), plan.handle, work.data_ptr(), _c(smaps), sb,
                                        _c(scaling), B, C, norm_code(norm), out.data_ptr(), stream_handle(dev)))
    return out


def nufft_fwd(geom: GeomKey, lay: PointsLayout, tables, scaling, image, smaps, norm) -> torch.Tensor:
    """Fused forward NUFFT: kdata = interp(FFT(pad(image [* smaps] * scaling)))."""
    dev = require_cuda(image, smaps, scaling)
    image = image.contiguous()
    B = image.shape[0]
    C = smaps.shape[1] if smaps is not None else image.shape[1]
    sb = 0
    if smaps is not None:
        smaps = smaps.to(image.dtype).contiguous()
        sb = smaps.shape[0]
    if scaling is not None:
        scaling = scaling.to(image.dtype).contiguous()
    plan = fft_plan(geom, B, C, dev)
    grid = torch.empty((B, C) + geom.grid_size, dtype=image.dtype, device=dev)
    kdata = torch.empty((B, C, lay.npts), dtype=image.dtype, device=dev)
    tp, keep, fl = table_ptrs(tables, image.dtype)
    lay.factor_call(keep, fl, lambda flags: L.check(L.lib().tkbn_nufft_fwd(
        ctypes.byref(geom_struct(geom, flags)), ctypes.byref(lay.desc), lay.workspace.data_ptr(), plan.handle, tp,
        _c(scaling), image.data_ptr(), _c(smaps), sb, B, C, norm_code(norm), grid.data_ptr(), kdata.data_ptr(),
        lay.stream_for_call(True))))
    return kdata


def nufft_adj(geom: GeomKey, lay: PointsLayout, tables, scaling, kdata, smaps, norm) -> torch.Tensor:
    """Fused adjoint NUFFT: image = [sum_c conj(smaps)] conj(scaling) crop(IFFT(interp^H(kdata)))."""
    dev = require_cuda(kdata, smaps, scaling)
    kdata = kdata.contiguous()
    B, C = kdata.shape[:2]
    sb = 0
    if smaps is not None:
        smaps = smaps.to(kdata.dtype).contiguous()
        sb = smaps.shape[0]
    if scaling is not None:
        scaling = scaling.to(kdata.dtype).contiguous()
    plan = fft_plan(geom, B, C, dev)
    grid = torch.empty((B, C) + geom.grid_size, dtype=kdata.dtype, device=dev)
    co = 1 if smaps is not None else C
    image = torch.empty((B, co) + geom.im_size, dtype=kdata.dtype, device=dev)
    tp, keep, fl = table_ptrs(tables, kdata.dtype)
    lay.factor_call(keep, fl, lambda flags: L.check(L.lib().tkbn_nufft_adj(
        ctypes.byref(geom_struct(geom, flags)), ctypes.byref(lay.desc), lay.workspace.data_ptr(), plan.handle, tp,
        _c(scaling), kdata.data_ptr(), _c(smaps), sb, B, C, norm_code(norm), grid.data_ptr(), image.data_ptr(),
        lay.stream_for_call(True))))
    return image


def toep_apply(image: torch.Tensor, kernel: torch.Tensor, smaps: Optional[torch.Tensor], norm: Optional[str],
               kernel_mode: str) -> torch.Tensor:
    """Toeplitz normal operator / FFT filter on the oversampled grid of ``kernel``.

    kernel_mode: "shared" (kernel is ``*grid``), "batch" (``(B, *grid)``, one
    per batch item; with smaps) or "channel" (``(C, *grid)``, one per channel).
    """
    dev = require_cuda(image, kernel, smaps)
    image = image.contiguous()
    kernel = kernel.to(image.dtype).contiguous()
    nd = image.ndim - 2
    im_size = tuple(image.shape[2:])
    grid_size = tuple(kernel.shape[-nd:])
    geom = GeomKey(nd, dtype_code(image.dtype), im_size, grid_size, (1,) * nd, (1,) * nd, (0.0,) * nd)
    B = image.shape[0]
    kb = 1 if kernel_mode == "shared" else kernel.shape[0]
    if smaps is not None:
        smaps = smaps.to(image.dtype).contiguous()
        C = smaps.shape[1]
        sb = smaps.shape[0]
    else:
        C = image.shape[1]
        sb = 0
    plan = fft_plan(geom, B, C, dev)
    grid = torch.empty((B, C) + grid_size, dtype=image.dtype, device=dev)
    co = 1 if smaps is not None else C
    out = torch.empty((B, co) + im_size, dtype=image.dtype, device=dev)
    g = geom_struct(geom)
    if smaps is not None:
        L.check(L.lib().tkbn_toep_apply(ctypes.byref(g), plan.handle, image.data_ptr(), kernel.data_ptr(), kb,
                                        smaps.data_ptr(), sb, B, C, norm_code(norm), grid.data_ptr(), out.data_ptr(),
                                        stream_handle(dev)))
    else:
        L.check(L.lib().tkbn_fft_filter(ctypes.byref(g), plan.handle, image.data_ptr(), kernel.data_ptr(), kb, B, C,
                                        norm_code(norm), grid.data_ptr(), out.data_ptr(), stream_handle(dev)))
    return out


def device_status(device: torch.device) -> int:
    st = ctypes.c_int32(0)
    L.check(L.lib().tkbn_device_status(stream_handle(device), ctypes.byref(st)))
    return int(st.value)
