"""GPU parity of the FFT stages (fft_and_scale, ifft_and_scale, Toeplitz / fft_filter).

2D grids whose sizes factor into radices 2..15 run the fused row/column
passes; 3D grids whose sizes all have compile-time plans run the same passes
per dimension (x rows of the nonzero image rows, y columns of the nonzero
slices, z columns); other sizes (a prime factor above 5) and other 3D grids
run cuFFT between the pad and crop kernels. Both are checked against the oracle's numpy
restatement of torchkbnufft/_nufft/fft.py, with smaps (shared and per batch),
scaling coefficients and both norms.
"""

import numpy as np
import pytest
import torch

from oracle import kbnufft_oracle as O
from conftest import rel_l2

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL = {torch.complex64: 1e-5, torch.complex128: 1e-12}

# (im_size, grid_size): fused plans for 640 (10*8*8), 384 (8*8*6), 320 (8*8*5),
# 96 (12*8), 90 (15*6), 160 (10*4*4), 2048 (8*8*8*4); 77 and 98 (7, 11 factors)
# and the 3D shape go to cuFFT
SHAPES = [
    ((320, 320), (640, 640)),
    ((192, 160), (384, 320)),
    ((48, 45), (96, 90)),
    ((80, 7), (160, 16)),
    ((16, 1000), (24, 2048)),
    ((40, 49), (77, 98)),
    ((8, 12, 10), (16, 24, 20)),
]


def _rand(gen, shape, cd):
    return torch.view_as_complex(torch.randn(shape + (2,), generator=gen, dtype=torch.float64)).to(cd)


def _np(t):
    return t.detach().cpu().numpy()


def _geom(cd, im, gs):
    from torchkbnufft_gb300 import _runtime as R

    return R.make_geom(cd, im, gs, (1,) * len(im), (1,) * len(im), (0.0,) * len(im))


@pytest.mark.parametrize("cd", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("shape", range(len(SHAPES)))
@pytest.mark.parametrize("norm", [None, "ortho"])
def test_fft_and_scale_vs_oracle(shape, cd, norm):
    from torchkbnufft_gb300 import _runtime as R

    im, gs = SHAPES[shape]
    if cd == torch.complex64 and norm is None and shape == 0:
        B, C, sb = 2, 16, 1
    else:
        B, C, sb = 2, 3, 2
    gen = torch.Generator().manual_seed(7 + shape)
    x = _rand(gen, (B, 1) + im, cd)
    s = _rand(gen, (sb, C) + im, cd)
    sc = _rand(gen, im, cd)
    geom = _geom(cd, im, gs)
    grid = R.fft_and_scale(geom, x.to(DEV), s.to(DEV), sc.to(DEV), norm)
    ref = O.fft_and_scale(_np(x) * _np(s), _np(sc), im, gs, norm)
    assert rel_l2(_np(grid), ref) < TOL[cd]
    # without smaps: per-channel images
    xc = _rand(gen, (B, C) + im, cd)
    grid = R.fft_and_scale(geom, xc.to(DEV), None, None, norm)
    assert rel_l2(_np(grid), O.fft_and_scale(_np(xc), np.ones(im), im, gs, norm)) < TOL[cd]


@pytest.mark.parametrize("cd", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("shape", range(len(SHAPES)))
@pytest.mark.parametrize("norm", [None, "ortho"])
def test_ifft_and_scale_vs_oracle(shape, cd, norm):
    from torchkbnufft_gb300 import _runtime as R

    im, gs = SHAPES[shape]
    B, C, sb = (2, 16, 1) if shape == 0 else (3, 5, 3)
    gen = torch.Generator().manual_seed(70 + shape)
    g = _rand(gen, (B, C) + gs, cd)
    s = _rand(gen, (sb, C) + im, cd)
    sc = _rand(gen, im, cd)
    geom = _geom(cd, im, gs)
    img = R.ifft_and_scale(geom, g.to(DEV), s.to(DEV), sc.to(DEV), norm)
    per_coil = O.ifft_and_scale(_np(g), _np(sc), im, gs, norm)
    ref = np.sum(per_coil * np.conj(_np(s)), axis=1, keepdims=True)
    assert rel_l2(_np(img), ref) < TOL[cd]
    img = R.ifft_and_scale(geom, g.to(DEV), None, None, norm)
    assert rel_l2(_np(img), O.ifft_and_scale(_np(g), np.ones(im), im, gs, norm)) < TOL[cd]


@pytest.mark.parametrize("cd", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("shape", [0, 2, 4, 5])
@pytest.mark.parametrize("mode", ["shared", "batch", "channel"])
def test_toeplitz_and_filter_vs_oracle(shape, cd, mode):
    from torchkbnufft_gb300 import _runtime as R

    im, gs = SHAPES[shape]
    B, C = 2, 4
    gen = torch.Generator().manual_seed(700 + shape)
    x = _rand(gen, (B, 1) + im, cd)
    s = _rand(gen, (1, C) + im, cd)
    if mode == "shared":
        k = _rand(gen, gs, cd)
    elif mode == "batch":
        k = _rand(gen, (B,) + gs, cd)
    else:
        k = _rand(gen, (C,) + gs, cd)
    if mode != "channel":
        out = R.toep_apply(x.to(DEV), k.to(DEV), s.to(DEV), "ortho", mode)
        assert rel_l2(_np(out), O.toep_apply(_np(x), _np(k), _np(s), "ortho")) < TOL[cd]
    if mode != "batch":
        xc = _rand(gen, (B, C) + im, cd)
        out = R.toep_apply(xc.to(DEV), k.to(DEV), None, None, mode)
        ref = O.fft_filter(_np(xc), _np(k), None)
        assert rel_l2(_np(out), ref) < TOL[cd]


def test_fused_fft_is_deterministic():
    from torchkbnufft_gb300 import _runtime as R

    im, gs = SHAPES[0]
    gen = torch.Generator().manual_seed(5)
    g = _rand(gen, (1, 16) + gs, torch.complex64).to(DEV)
    s = _rand(gen, (1, 16) + im, torch.complex64).to(DEV)
    geom = _geom(torch.complex64, im, gs)
    a = R.ifft_and_scale(geom, g, s, None, None)
    b = R.ifft_and_scale(geom, g, s, None, None)
    assert torch.equal(a, b)


@pytest.mark.parametrize("cd", [torch.complex64, torch.complex128])
@pytest.mark.parametrize("norm", [None, "ortho"])
def test_fused_3d_stages_vs_oracle(cd, norm, tmp_path):
    """3D grid of 256^3 (the kooshball configuration's grid) with a smaller,
    non-cubic image: forward and inverse stages through the fused passes,
    with and without smaps, against the oracle."""
    import json

    from torch.profiler import ProfilerActivity, profile

    from torchkbnufft_gb300 import _runtime as R

    im, gs = (96, 128, 112), (256, 256, 256)
    B, C = 1, 2
    gen = torch.Generator().manual_seed(31)
    x = _rand(gen, (B, 1) + im, cd)
    s = _rand(gen, (1, C) + im, cd)
    sc = _rand(gen, im, cd)
    geom = _geom(cd, im, gs)
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        grid = R.fft_and_scale(geom, x.to(DEV), s.to(DEV), sc.to(DEV), norm)
        torch.cuda.synchronize()
    path = tmp_path / "trace.json"
    prof.export_chrome_trace(str(path))
    names = {e.get("name", "") for e in json.loads(path.read_text()).get("traceEvents", []) if e.get("cat") == "kernel"}
    if names:  # the profiler saw the launches: the fused passes, not the pad kernel and cuFFT
        assert any("k_fft_cols_io" in n for n in names) and not any("k_pad_scale" in n for n in names), names
    ref = O.fft_and_scale(_np(x) * _np(s), _np(sc), im, gs, norm)
    assert rel_l2(_np(grid), ref) < TOL[cd]
    del ref
    g = _rand(gen, (B, C) + gs, cd)
    img = R.ifft_and_scale(geom, g.to(DEV), s.to(DEV), sc.to(DEV), norm)
    per_coil = O.ifft_and_scale(_np(g), _np(sc), im, gs, norm)
    ref = np.sum(per_coil * np.conj(_np(s)), axis=1, keepdims=True)
    assert rel_l2(_np(img), ref) < TOL[cd]
    img = R.ifft_and_scale(geom, g.to(DEV), None, sc.to(DEV), norm)  # per-coil images, no coil sum
    assert rel_l2(_np(img), per_coil) < TOL[cd]


@pytest.mark.parametrize("mode", ["shared", "channel"])
def test_fused_3d_toeplitz_vs_oracle(mode):
    """The Toeplitz normal operator on a 256^3 grid (128^3 image) through the
    fused 3D passes: x rows, y columns of the nonzero slices, the z columns
    transformed, multiplied by the kernel and transformed back in one pass,
    then y columns and x rows inverse with the crop (and the coil sum)."""
    from torchkbnufft_gb300 import _runtime as R

    cd = torch.complex64
    im, gs = (128, 128, 128), (256, 256, 256)
    B, C = 1, 2
    gen = torch.Generator().manual_seed(37)
    if mode == "shared":
        x = _rand(gen, (B, 1) + im, cd)
        s = _rand(gen, (1, C) + im, cd)
        k = _rand(gen, gs, cd)
        out = R.toep_apply(x.to(DEV), k.to(DEV), s.to(DEV), "ortho", mode)
        assert rel_l2(_np(out), O.toep_apply(_np(x), _np(k), _np(s), "ortho")) < TOL[cd]
    else:
        xc = _rand(gen, (B, C) + im, cd)
        k = _rand(gen, (C,) + gs, cd)
        out = R.toep_apply(xc.to(DEV), k.to(DEV), None, None, mode)
        assert rel_l2(_np(out), O.fft_filter(_np(xc), _np(k), None)) < TOL[cd]
