"""Hand-written autograd for the table NUFFT, including d/d omega.

The reference differentiates only w.r.t. the image / k-space data: its
``KbTableInterpForward.backward`` returns ``None`` for omega
(``torchkbnufft/_autograd/interp.py:103-130``). Here every Function also returns
the trajectory gradient when omega requires grad:

    d loss / d omega_d[m] = Re sum_{b,c} conj(v[b,c,m]) * d interp(G)[b,c,m] / d omega_d

where (forward) G is the oversampled grid and v the upstream k-space
gradient, or (adjoint) G is the grid-domain upstream gradient and v the
k-space input. The derivative is that of the smooth KB interpolation the
table samples (value and d/du tables, linear interpolation inside a bin).

Memory: NUFFT-level Functions save the image (or k-space data), never the
oversampled grid; the grid is recomputed in backward when omega needs a
gradient (one FFT stage), which keeps 3D trajectories affordable.
"""

from __future__ import annotations

import torch
from torch.autograd import Function

from . import _runtime as R


def _reduce_to(t: torch.Tensor, shape) -> torch.Tensor:
    """Sum a broadcast gradient back to ``shape`` (leading batch of 1)."""
    if tuple(t.shape) == tuple(shape):
        return t
    return t.sum(dim=0, keepdim=True).reshape(shape)


def _omega_grad(geom, lay, tables, grid, v, omega):
    g = R.interp_grad_omega(geom, lay, tables, grid, v)
    return g.reshape(omega.shape).to(omega.dtype)


class KbTableInterpForward(Function):
    """Table interpolation grid -> k-space (reference: ``_autograd/interp.py:78-130``)."""

    @staticmethod
    def forward(ctx, image, omega, tables, n_shift, numpoints, table_oversamp, offsets):
        R.require_cuda(image, omega)
        geom = R.make_geom(image.dtype, None, tuple(image.shape[2:]), numpoints, table_oversamp, n_shift)
        lay = R.points_layout(geom, omega)
        out = R.interp_fwd(geom, lay, tables, image)
        ctx.geom, ctx.tables = geom, tables
        ctx.save_for_backward(omega, image if ctx.needs_input_grad[1] else None)
        return out

    @staticmethod
    def backward(ctx, grad):
        omega, image = ctx.saved_tensors
        lay = R.points_layout(ctx.geom, omega)
        gi = go = None
        if ctx.needs_input_grad[0]:
            gi = R.interp_adj(ctx.geom, lay, ctx.tables, grad)
        if ctx.needs_input_grad[1]:
            go = _omega_grad(ctx.geom, lay, ctx.tables, image, grad, omega)
        return gi, go, None, None, None, None, None


class KbTableInterpAdjoint(Function):
    """Adjoint table interpolation k-space -> grid (reference: ``_autograd/interp.py:133-178``)."""

    @staticmethod
    def forward(ctx, data, omega, tables, n_shift, numpoints, table_oversamp, offsets, grid_size):
        R.require_cuda(data, omega)
        geom = R.make_geom(data.dtype, None, grid_size, numpoints, table_oversamp, n_shift)
        lay = R.points_layout(geom, omega)
        out = R.interp_adj(geom, lay, tables, data)
        ctx.geom, ctx.tables = geom, tables
        ctx.save_for_backward(omega, data if ctx.needs_input_grad[1] else None)
        return out

    @staticmethod
    def backward(ctx, grad):
        omega, data = ctx.saved_tensors
        lay = R.points_layout(ctx.geom, omega)
        gd = go = None
        if ctx.needs_input_grad[0]:
            gd = R.interp_fwd(ctx.geom, lay, ctx.tables, grad)
        if ctx.needs_input_grad[1]:
            go = _omega_grad(ctx.geom, lay, ctx.tables, grad, data, omega)
        return gd, go, None, None, None, None, None, None


class NufftForward(Function):
    """kdata = interp(FFT(pad(image [* smaps] * scaling))) with fused kernels.

    image: (B, 1, *N) with smaps (Bs, C, *N), else (B, C, *N).
    """

    @staticmethod
    def forward(ctx, image, smaps, omega, geom, tables, scaling, norm):
        R.require_cuda(image, smaps, omega, scaling)
        lay = R.points_layout(geom, omega)
        out = R.nufft_fwd(geom, lay, tables, scaling, image, smaps, norm)
        ctx.geom, ctx.tables, ctx.scaling, ctx.norm = geom, tables, scaling, norm
        ctx.save_for_backward(image, smaps, omega)
        return out

    @staticmethod
    def backward(ctx, gy):
        image, smaps, omega = ctx.saved_tensors
        geom, tables, scaling, norm = ctx.geom, ctx.tables, ctx.scaling, ctx.norm
        lay = R.points_layout(geom, omega)
        need_img, need_s, need_om = ctx.needs_input_grad[:3]
        gi = gs = go = None
        if need_img or need_s:
            if smaps is None:
                gi = R.nufft_adj(geom, lay, tables, scaling, gy, None, norm)
            elif need_s:
                per_coil = R.nufft_adj(geom, lay, tables, scaling, gy, None, norm)
                gs = _reduce_to(image.conj() * per_coil, smaps.shape)
                if need_img:
                    gi = torch.sum(per_coil * smaps.conj(), dim=1, keepdim=True)
            else:
                gi = R.nufft_adj(geom, lay, tables, scaling, gy, smaps, norm)
        if need_om:
            grid = R.fft_and_scale(geom, image, smaps, scaling, norm)
            go = _omega_grad(geom, lay, tables, grid, gy, omega)
        return gi, gs, go, None, None, None, None


class NufftAdjoint(Function):
    """image = [sum_c conj(smaps)] conj(scaling) crop(IFFT(interp^H(kdata)))."""

    @staticmethod
    def forward(ctx, kdata, smaps, omega, geom, tables, scaling, norm):
        R.require_cuda(kdata, smaps, omega, scaling)
        lay = R.points_layout(geom, omega)
        out = R.nufft_adj(geom, lay, tables, scaling, kdata, smaps, norm)
        ctx.geom, ctx.tables, ctx.scaling, ctx.norm = geom, tables, scaling, norm
        ctx.save_for_backward(kdata, smaps, omega)
        return out

    @staticmethod
    def backward(ctx, gx):
        kdata, smaps, omega = ctx.saved_tensors
        geom, tables, scaling, norm = ctx.geom, ctx.tables, ctx.scaling, ctx.norm
        lay = R.points_layout(geom, omega)
        need_k, need_s, need_om = ctx.needs_input_grad[:3]
        gk = gs = go = None
        if need_k or need_om:
            # grid-domain upstream gradient: the adjoint of crop(IFFT(.)) * conj(scaling) [* conj(smaps)]
            gX = R.fft_and_scale(geom, gx, smaps, scaling, norm)
            if need_k:
                gk = R.interp_fwd(geom, lay, tables, gX)
            if need_om:
                go = _omega_grad(geom, lay, tables, gX, kdata, omega)
        if need_s:
            per_coil = R.nufft_adj(geom, lay, tables, scaling, kdata, None, norm)
            gs = _reduce_to(per_coil * gx.conj(), smaps.shape)
        return gk, gs, go, None, None, None, None


class ToepApply(Function):
    """Toeplitz normal operator; backward applies the conjugate kernel."""

    @staticmethod
    def forward(ctx, image, kernel, smaps, norm, kernel_mode):
        if kernel.requires_grad:
            raise NotImplementedError("gradients with respect to the Toeplitz kernel are not supported")
        R.require_cuda(image, kernel, smaps)
        ctx.norm, ctx.kernel_mode = norm, kernel_mode
        ctx.save_for_backward(kernel, smaps)
        return R.toep_apply(image, kernel, smaps, norm, kernel_mode)

    @staticmethod
    def backward(ctx, grad):
        kernel, smaps = ctx.saved_tensors
        gi = None
        if ctx.needs_input_grad[0]:
            gi = R.toep_apply(grad, kernel.conj(), smaps, ctx.norm, ctx.kernel_mode)
        if smaps is not None and ctx.needs_input_grad[2]:
            raise NotImplementedError("gradients with respect to smaps in ToepNufft are not supported")
        return gi, None, None, None, None
