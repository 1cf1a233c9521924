"""GPU parity of the Toeplitz path (K6, calc_toeplitz_kernel) and density compensation."""

import numpy as np
import pytest
import torch

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def tkbn():
    import torchkbnufft_gb300 as m

    return m


def _np(t):
    return t.detach().cpu().numpy()


def _rand(gen, shape, cd):
    return torch.view_as_complex(torch.randn(shape + (2,), generator=gen, dtype=torch.float64)).to(cd)


@pytest.mark.parametrize("name", ["toep_2d", "toep_2d_none", "toep_3d", "toep_2d_batched"])
def test_live_toeplitz_fixtures(name):
    g = load_golden("live_" + name)
    norm = str(g["norm"]) or None
    im_size = g["image"].shape[2:]
    t = lambda k: torch.tensor(g[k], device=DEV)
    kern = tkbn().calc_toeplitz_kernel(t("omega"), im_size, weights=t("weights"), norm=norm)
    assert rel_l2(_np(kern), g["kernel"]) < 1e-5
    toep = tkbn().ToepNufft()
    assert rel_l2(_np(toep(t("image"), t("kernel"), smaps=t("smaps"), norm=norm)), g["out_sense"]) < 1e-5
    assert rel_l2(_np(toep(t("image"), t("kernel"), norm=norm)), g["out_plain"]) < 1e-5


@pytest.mark.parametrize("shape, grid_size, M, norm, tol", [
    ([1, 3, 19], [57], 25, "ortho", 1e-2),
    ([1, 4, 32, 16], [64, 24], 83, None, 1e-2),
    ([3, 10, 13, 18, 12], [20, 26, 37], 112, None, 1e-2),
    ([2, 8, 40, 36], None, 2000, "ortho", 1e-4),
])
def test_toeplitz_matches_normal_operator(shape, grid_size, M, norm, tol):
    """ToepNufft ~= A^H A (reference tests/test_toep.py:20-60, 74-116), complex128."""
    gen = torch.Generator().manual_seed(123)
    im_size = tuple(shape[2:])
    x = _rand(gen, (shape[0], 1) + im_size, torch.complex128).to(DEV)
    s = _rand(gen, tuple(shape), torch.complex128).to(DEV)
    om = ((torch.rand((len(im_size), M), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    fwd = tkbn().KbNufft(im_size=im_size, grid_size=grid_size, dtype=torch.complex128, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, grid_size=grid_size, dtype=torch.complex128, device=DEV)
    kern = tkbn().calc_toeplitz_kernel(om, im_size, grid_size=grid_size, norm=norm)
    fbn = adj(fwd(x, om, smaps=s, norm=norm), om, smaps=s, norm=norm)
    fbt = tkbn().ToepNufft()(x, kern, smaps=s, norm=norm)
    assert (torch.linalg.vector_norm(fbn - fbt) / torch.linalg.vector_norm(fbn)).item() < tol


def test_toeplitz_backward_is_self_adjoint():
    gen = torch.Generator().manual_seed(2)
    im = (20, 24)
    x = _rand(gen, (2, 1) + im, torch.complex128).to(DEV).requires_grad_(True)
    s = _rand(gen, (2, 3) + im, torch.complex128).to(DEV)
    om = ((torch.rand((2, 500), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    kern = tkbn().calc_toeplitz_kernel(om, im, norm="ortho")
    toep = tkbn().ToepNufft()
    y = toep(x, kern, smaps=s, norm="ortho")
    (y.abs() ** 2 / 2).sum().backward()
    expect = toep(y.detach(), kern.conj(), smaps=s, norm="ortho")
    assert torch.allclose(x.grad, expect)


@pytest.mark.parametrize("name", ["dcomp_2d", "dcomp_2d_batched"])
def test_live_dcomp_fixtures(name):
    g = load_golden("live_" + name)
    out = tkbn().calc_density_compensation_function(torch.tensor(g["omega"], device=DEV),
                                                     tuple(int(x) for x in g["im_size"]))
    assert rel_l2(_np(out), g["dcomp"]) < 1e-5
