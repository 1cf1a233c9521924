"""Pin the CPU oracle against the reference's golden vectors and live fixtures.

CPU-only: no GPU and no extension needed.
"""

import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import kbnufft_oracle as O


def _c(x):
    """real (..., 2) -> complex"""
    return x[..., 0] + 1j * x[..., 1]


@pytest.mark.parametrize("case", [0, 1, 2])
def test_reference_interp_pickle(case):
    """Reference golden ``interp_data.pkl`` (tests/test_interp.py:16-31), float64."""
    g = load_golden("ref_interp_data")
    image, ktraj, kdata = _c(g[f"image_{case}"]), g[f"ktraj_{case}"], _c(g[f"kdata_{case}"])
    im_size = image.shape[2:]
    op = O.Operator(im_size, grid_size=im_size, cdtype=np.complex128)
    out = op.interp(image, ktraj)
    # reference test uses torch.allclose (rtol 1e-5, atol 1e-8)
    assert np.allclose(out, kdata, rtol=1e-5, atol=1e-8)
    assert rel_l2(out, kdata) < 1e-12


@pytest.mark.parametrize("case", [0, 1])
def test_reference_nufft_pickle(case):
    """Reference golden ``nufft_data.pkl`` (tests/test_nufft.py:15-30), float64."""
    g = load_golden("ref_nufft_data")
    image, ktraj, kdata = _c(g[f"image_{case}"]), g[f"ktraj_{case}"], _c(g[f"kdata_{case}"])
    op = O.Operator(image.shape[2:], cdtype=np.complex128)
    out = op.forward(image, ktraj)
    assert np.allclose(out, kdata, rtol=1e-5, atol=1e-8)
    assert rel_l2(out, kdata) < 1e-12


@pytest.mark.parametrize("name", ["interp_1d", "interp_2d", "interp_2d_batched", "interp_3d", "interp_2d_c128"])
def test_live_interp(name):
    g = load_golden("live_" + name)
    cd = g["grid"].dtype
    im_size = g["grid"].shape[2:]
    op = O.Operator(im_size, grid_size=im_size, cdtype=cd)
    tol = 1e-6 if cd == np.complex64 else 1e-13
    assert rel_l2(op.interp(g["grid"], g["omega"]), g["kdata"]) < tol
    assert rel_l2(op.interp_adj(g["kdata_in"], g["omega"]), g["grid_adj"]) < tol


@pytest.mark.parametrize("name", ["nufft_1d", "nufft_2d", "nufft_2d_ortho", "nufft_2d_batched", "nufft_3d",
                                  "nufft_2d_grid", "nufft_2d_c128", "nufft_refparams_2d", "nufft_refparams_3d"])
def test_live_nufft(name):
    g = load_golden("live_" + name)
    cd = g["image"].dtype
    norm = str(g["norm"]) or None
    J = tuple(int(x) for x in g["numpoints"]) if "numpoints" in g else 6
    op = O.Operator(g["image"].shape[2:], grid_size=tuple(int(x) for x in g["grid_size"]), numpoints=J, cdtype=cd)
    tol = 2e-6 if cd == np.complex64 else 1e-12
    assert rel_l2(op.forward(g["image"], g["omega"], smaps=g["smaps"], norm=norm), g["kdata_sense"]) < tol
    assert rel_l2(op.adjoint(g["kdata_in"], g["omega"], smaps=g["smaps"], norm=norm), g["image_sense"]) < tol
    assert rel_l2(op.forward(g["image_coils"], g["omega"], norm=norm), g["kdata_plain"]) < tol
    assert rel_l2(op.adjoint(g["kdata_in"], g["omega"], norm=norm), g["image_plain"]) < tol


@pytest.mark.parametrize("name", ["toep_2d", "toep_2d_none", "toep_3d", "toep_2d_batched"])
def test_live_toeplitz(name):
    g = load_golden("live_" + name)
    norm = str(g["norm"]) or None
    im_size = g["image"].shape[2:]
    kern = O.toeplitz_kernel(g["omega"], im_size, weights=g["weights"], norm=norm)
    assert rel_l2(kern, g["kernel"]) < 2e-6
    assert rel_l2(O.toep_apply(g["image"], g["kernel"], smaps=g["smaps"], norm=norm), g["out_sense"]) < 2e-6
    assert rel_l2(O.toep_apply(g["image"], g["kernel"], norm=norm), g["out_plain"]) < 2e-6


@pytest.mark.parametrize("name", ["dcomp_2d", "dcomp_2d_batched"])
def test_live_dcomp(name):
    g = load_golden("live_" + name)
    out = O.density_compensation(g["omega"], tuple(int(x) for x in g["im_size"]))
    assert rel_l2(out, g["dcomp"]) < 1e-5


def test_ndft_matches_table_nufft():
    """The FP64 NDFT oracle agrees with the table NUFFT to the kernel's intrinsic error."""
    rng = np.random.default_rng(7)
    im = (rng.standard_normal((1, 1, 16, 16)) + 1j * rng.standard_normal((1, 1, 16, 16)))
    om = rng.uniform(-np.pi, np.pi, (2, 200))
    op = O.Operator((16, 16), cdtype=np.complex128)
    err = rel_l2(op.forward(im, om), O.ndft_forward(im, om))
    assert err < 2e-3
