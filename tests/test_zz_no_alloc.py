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
TOL128 = 1e-10  # relative L2, complex128


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


def _run(seed, im, B, C, M, cd):
    """One call of the entry point; returns its output, the workspace entry
    point's output and the oracle's, as numpy."""
    import torchkbnufft_gb300 as tkbn
    from oracle import kbnufft_oracle as O
    from torchkbnufft_gb300 import _lib as L
    from torchkbnufft_gb300 import _runtime as R

    lib = L.load()
    ob = tkbn.KbInterp(im_size=im, grid_size=im, dtype=cd, device=DEV)
    grid, om = _case(seed, im, B, C, M)
    grid = grid.to(cd)
    om = om.to(R.real_of(cd))
    geom = R.make_geom(cd, None, im, ob.numpoints, ob.table_oversamp, ob.n_shift)
    tables = ob._tables()
    tp, keep, flags = R.table_ptrs(tables, cd)
    g = R.geom_struct(geom, flags)
    rc, out = _noalloc(lib, g, tp, om, grid)
    L.check(rc)
    ws = R.interp_fwd(geom, R.points_layout(geom, om), tables, grid)
    torch.cuda.synchronize()
    want = O.interp_forward(grid.cpu().numpy(), om.cpu().numpy(), [t.cpu().numpy() for t in keep],
                            geom.n_shift, geom.numpoints, geom.table_oversamp)
    return out.cpu().numpy(), ws.cpu().numpy(), want


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls():
    # calls in a row with different sizes, dimension counts and dtypes: a large
    # one, a smaller one, then larger ones again, so leftover state in the
    # shared array (header, counts, lists past the previous size) would show
    for seed, im, B, C, M, cd in ((1, (64, 72), 2, 16, 20000, torch.complex64),
                                  (2, (48, 40), 1, 5, 7000, torch.complex64),
                                  (3, (24, 20, 28), 1, 3, 30000, torch.complex64),
                                  (4, (80, 64), 1, 2, 40000, torch.complex128),
                                  (5, (64, 72), 2, 16, 20000, torch.complex64)):
        out, ws, want = _run(seed, im, B, C, M, cd)
        tol = TOL64 if cd == torch.complex64 else TOL128
        assert rel_l2(out, ws) < tol
        assert rel_l2(out, want) < tol


def test_noalloc_empty_trajectory():
    out, ws, want = _run(6, (32, 32), 1, 4, 0, torch.complex64)
    assert out.shape == (1, 4, 0) and ws.shape == (1, 4, 0) and want.shape == (1, 4, 0)
    # and a call with points after it still matches the oracle
    out, ws, want = _run(7, (32, 32), 1, 4, 500, torch.complex64)
    assert rel_l2(out, want) < TOL64


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
