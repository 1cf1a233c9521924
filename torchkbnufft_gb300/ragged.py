"""Ragged batches of independent NUFFT problems in a few launches (K8).

torchkbnufft has no counterpart: there a caller loops over problems, one
``KbNufft`` / ``KbNufftAdjoint`` call each (torchkbnufft/modules/kbnufft.py:
125-228, 307-410). Here problems that differ in image size, trajectory and
coil count share the work of each stage:

* the interpolation of every problem is one launch
  (``tkbn_ragged_interp_fwd`` / ``tkbn_ragged_interp_adj``: a merged,
  longest-first job list over all problems' work items);
* the FFT stages run once per image size, over the coil planes of every
  problem of that size, which sit side by side in one buffer;
* the whole forward + adjoint sequence reads and writes fixed buffers, so
  ``capture()`` records it as one CUDA graph and ``replay()`` reruns it.

Each problem is ``(im_size, omega, ncoil)`` with omega ``(d, M)`` (one
trajectory per problem); images are ``(1, ncoil, *im_size)`` coil images (no
coil maps), k-space data ``(1, ncoil, M)``, the reference's layouts. The
optional autotuner picks the layout's tile shape per image size. The plan
computes each 2D problem's per-point adjoint factors once, into that problem's
layout workspace; the layouts are private to the plan.
"""

from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Tuple

import torch

from . import _lib as L
from . import _runtime as R
from . import autotune
from .modules import KbNufft


class _SizeClass:
    """Problems of one image size: shared tables, scaling, FFT plan and plane buffers."""

    def __init__(self, im_size, members, ncoils, nufft_kwargs, dtype, device):
        self.im_size = tuple(im_size)
        self.members = members
        self.module = KbNufft(im_size=self.im_size, dtype=dtype, device=device, **nufft_kwargs)
        self.geom = self.module._geom(dtype)
        self.tables = self.module._tables()
        self.tptrs, self.tkeep, self.flags = R.table_ptrs(self.tables, dtype)
        self.scaling = self.module.scaling_coef.to(dtype).contiguous()
        self.planes = sum(ncoils[p] for p in members)
        self.offset = {}
        o = 0
        for p in members:
            self.offset[p] = o
            o += ncoils[p]
        self.image = torch.zeros((1, self.planes) + self.im_size, dtype=dtype, device=device)
        self.grid = torch.zeros((1, self.planes) + self.geom.grid_size, dtype=dtype, device=device)
        self.out = torch.zeros_like(self.image)
        self.plan = R.fft_plan(self.geom, 1, self.planes, device)
        self.gstruct = R.geom_struct(self.geom)


class RaggedNufft:
    """Forward and adjoint NUFFT of many independent problems at once.

    Args:
        problems: sequence of ``(im_size, omega, ncoil)``; omega is a
            ``(d, M)`` tensor on the target CUDA device.
        numpoints, table_oversamp, kbwidth, order: as ``KbNufft`` (shared).
        dtype: complex64 or complex128.
        autotune: pick each image size's layout tile with the autotuner
            (timed on that size's largest problem); else the library default.
        norm: ``None`` or ``"ortho"``, applied to every FFT stage.
    """

    def __init__(self, problems: Sequence[Tuple[Sequence[int], torch.Tensor, int]], numpoints=6,
                 table_oversamp=2**10, kbwidth=2.34, order=0.0, dtype=torch.complex64, autotune_layout=False,
                 norm: Optional[str] = None):
        if len(problems) == 0:
            raise ValueError("need at least one problem")
        self.dtype = dtype
        self.norm = norm
        self.device = problems[0][1].device
        R.require_cuda(*[p[1] for p in problems])
        self.im_sizes = [tuple(int(v) for v in p[0]) for p in problems]
        self.omegas = [p[1] for p in problems]
        self.ncoils = [int(p[2]) for p in problems]
        if any(o.ndim != 2 for o in self.omegas):
            raise ValueError("each problem takes one trajectory of shape (d, M)")
        kw = dict(numpoints=numpoints, table_oversamp=table_oversamp, kbwidth=kbwidth, order=order)
        by_size = {}
        for p, im in enumerate(self.im_sizes):
            by_size.setdefault(im, []).append(p)
        self.classes = [_SizeClass(im, members, self.ncoils, kw, dtype, self.device) for im, members in by_size.items()]
        self.class_of = {}
        for k in self.classes:
            for p in k.members:
                self.class_of[p] = k
        self.tiles = {}
        for k in self.classes:
            tile, chunk = None, 0
            if autotune_layout:
                big = max(k.members, key=lambda p: self.omegas[p].shape[-1] * self.ncoils[p])
                tile, chunk = autotune.tune_layout(k.geom, self.omegas[big], k.tables, self.ncoils[big])
            self.tiles[k.im_size] = (tile, chunk)
        self.layouts = []
        self.kdata = []
        for p, om in enumerate(self.omegas):
            k = self.class_of[p]
            tile, chunk = self.tiles[k.im_size]
            self.layouts.append(R.PointsLayout(k.geom, om, tile, chunk))
            self.kdata.append(torch.zeros((1, self.ncoils[p], om.shape[-1]), dtype=dtype, device=self.device))
        self._plan = ctypes.c_void_p()
        self._build_plan()
        self.graph = None

    # -------------------------------------------------------------- plan
    def _build_plan(self):
        n = len(self.omegas)
        arr = (L.RaggedProblem * n)()
        esize = 8 if self.dtype == torch.complex64 else 16
        for p in range(n):
            k = self.class_of[p]
            g = L.Geometry.from_buffer_copy(k.gstruct)
            g.flags = k.flags | self.layouts[p].flags
            arr[p].geom = g
            arr[p].points = self.layouts[p].desc
            arr[p].workspace = self.layouts[p].workspace.data_ptr()
            for d in range(3):
                arr[p].tables[d] = k.tptrs[d]
            arr[p].ncoil = self.ncoils[p]
            gtot = 1
            for s in k.geom.grid_size:
                gtot *= s
            arr[p].grid = k.grid.data_ptr() + k.offset[p] * gtot * esize
            arr[p].kdata = self.kdata[p].data_ptr()
        with torch.cuda.device(self.device):
            L.check(L.lib().tkbn_ragged_plan_create(arr, n, ctypes.byref(self._plan)))

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                L.lib().tkbn_ragged_plan_destroy(plan)
            except Exception:
                pass

    # -------------------------------------------------------------- stages
    def _stream(self) -> int:
        return R.stream_handle(self.device)

    def _fft_forward(self):
        norm = R.norm_code(self.norm)
        for k in self.classes:
            L.check(L.lib().tkbn_fft_and_scale(ctypes.byref(k.gstruct), k.plan.handle, k.image.data_ptr(), None, 0,
                                               k.scaling.data_ptr(), 1, k.planes, norm, k.grid.data_ptr(),
                                               self._stream()))

    def _fft_adjoint(self):
        norm = R.norm_code(self.norm)
        for k in self.classes:
            L.check(L.lib().tkbn_ifft_and_scale(ctypes.byref(k.gstruct), k.plan.handle, k.grid.data_ptr(), None, 0,
                                                k.scaling.data_ptr(), 1, k.planes, norm, k.out.data_ptr(),
                                                self._stream()))

    def _interp_forward(self):
        L.check(L.lib().tkbn_ragged_interp_fwd(self._plan, self._stream()))

    def _interp_adjoint(self):
        L.check(L.lib().tkbn_ragged_interp_adj(self._plan, self._stream()))

    # -------------------------------------------------------------- public
    def image_view(self, p: int) -> torch.Tensor:
        """The input image buffer of problem p, ``(1, ncoil, *im_size)``."""
        k = self.class_of[p]
        return k.image[:, k.offset[p]:k.offset[p] + self.ncoils[p]]

    def output_view(self, p: int) -> torch.Tensor:
        """The adjoint output buffer of problem p, ``(1, ncoil, *im_size)``."""
        k = self.class_of[p]
        return k.out[:, k.offset[p]:k.offset[p] + self.ncoils[p]]

    def set_images(self, images: Sequence[torch.Tensor]) -> None:
        for p, x in enumerate(images):
            self.image_view(p).copy_(x.reshape(self.image_view(p).shape))

    def set_kdata(self, kdata: Sequence[torch.Tensor]) -> None:
        for p, y in enumerate(kdata):
            self.kdata[p].copy_(y.reshape(self.kdata[p].shape))

    def forward(self, images: Optional[Sequence[torch.Tensor]] = None) -> List[torch.Tensor]:
        """k-space data of every problem (views of the plan's buffers)."""
        if images is not None:
            self.set_images(images)
        self._fft_forward()
        self._interp_forward()
        return list(self.kdata)

    def adjoint(self, kdata: Optional[Sequence[torch.Tensor]] = None) -> List[torch.Tensor]:
        """Adjoint images of every problem (views of the plan's buffers)."""
        if kdata is not None:
            self.set_kdata(kdata)
        self._interp_adjoint()
        self._fft_adjoint()
        return [self.output_view(p) for p in range(len(self.omegas))]

    def forward_adjoint(self) -> None:
        """Forward of the image buffers, then adjoint of the result, in place."""
        self._fft_forward()
        self._interp_forward()
        self._interp_adjoint()
        self._fft_adjoint()

    def capture(self) -> None:
        """Record forward_adjoint as one CUDA graph (run once first to warm up)."""
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.forward_adjoint()
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.forward_adjoint()
        self.graph = g

    def replay(self) -> None:
        if self.graph is None:
            raise RuntimeError("call capture() first")
        self.graph.replay()
