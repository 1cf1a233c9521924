"""The allocation-free forward interpolation entry point (tkbn_interp_fwd_noalloc).

Callers that cannot allocate device memory after start-up (a fixed memory
budget, or a plain-C host that only holds raw device pointers) use this entry
point; it keeps the trajectory layout in a library-owned device array instead
of a caller-allocated workspace. This file is collected last so that a run
stopping at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL64 = 1e-5  # relative L2, the complex64 parity bar used throughout the GPU tests


def _case(seed, im, B, C, M):
    gen = torch.Generator().manual_seed(seed)
    grid = torch.view_as_complex(torch.randn((B, C) + im + (2,), generator=gen)).to(DEV)
    om = ((torch.rand((len(im), M), generator=gen) * 2 - 1) * np.pi).to(DEV)
    return grid, om


def _noalloc(lib, g, tp, om, grid):
    from torchkbnufft_gb300 import _runtime as R

    B, C = grid.shape[:2]
    out = torch.empty((B, C, om.shape[1]), dtype=grid.dtype, device=DEV)
    rc = lib.tkbn_interp_fwd_noalloc(ctypes.byref(g), tp, om.data_ptr(), om.shape[1], grid.data_ptr(), B, C,
                                     out.data_ptr(), R.stream_handle(DEV))
    return rc, out


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls():
    import torchkbnufft_gb300 as tkbn
    from torchkbnufft_gb300 import _lib as L
    from torchkbnufft_gb300 import _runtime as R

    lib = L.load()
    # two calls in a row with different sizes and data: the shared array must not leak state
    for seed, im, B, C, M in ((1, (64, 72), 2, 16, 20000), (2, (48, 40), 1, 5, 7000)):
        ob = tkbn.KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
        grid, om = _case(seed, im, B, C, M)
        geom = R.make_geom(torch.complex64, None, im, ob.numpoints, ob.table_oversamp, ob.n_shift)
        tp, keep, flags = R.table_ptrs(ob._tables(), torch.complex64)
        g = R.geom_struct(geom, flags)
        rc, out = _noalloc(lib, g, tp, om, grid)
        L.check(rc)
        ref = R.interp_fwd(geom, R.points_layout(geom, om), ob._tables(), grid)
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < TOL64


def test_noalloc_rejects_trajectories_beyond_its_array():
    from torchkbnufft_gb300 import _lib as L
    from torchkbnufft_gb300 import _runtime as R

    lib = L.load()
    im = (64, 64)
    geom = R.make_geom(torch.complex64, None, im, (6, 6), (1024, 1024), (32.0, 32.0))
    g = R.geom_struct(geom, 0)
    # real (small) device buffers; the size check rejects the call before any of them is used
    table = torch.zeros(6 * 1024 + 1, dtype=torch.complex64, device=DEV)
    om = torch.zeros((2, 16), device=DEV)
    grid = torch.zeros((1, 1) + im, dtype=torch.complex64, device=DEV)
    out = torch.zeros((1, 1, 16), dtype=torch.complex64, device=DEV)
    tp = L.ptr_array([table.data_ptr(), table.data_ptr()])
    rc = lib.tkbn_interp_fwd_noalloc(ctypes.byref(g), tp, om.data_ptr(), 4_000_000, grid.data_ptr(), 1, 1,
                                     out.data_ptr(), R.stream_handle(DEV))
    assert rc == L.TKBN_ERR_INVALID
    assert b"layout scratch" in lib.tkbn_last_error()
