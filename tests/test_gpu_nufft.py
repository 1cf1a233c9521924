"""GPU parity of the full NUFFT (K2 pad/apodise/SENSE, cuFFT, K3/K4, K5 crop/coil-sum)."""

import numpy as np
import pytest
import torch

from conftest import load_golden, rel_l2
from oracle import kbnufft_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def tkbn():
    import torchkbnufft_gb300 as m

    return m


def _np(t):
    return t.detach().cpu().numpy()


def _rand(gen, shape, cd):
    return torch.view_as_complex(torch.randn(shape + (2,), generator=gen, dtype=torch.float64)).to(cd)


@pytest.mark.parametrize("case", [0, 1])
def test_reference_nufft_golden(case):
    """``tests/data/nufft_data.pkl`` through KbNufft in float64 (reference tests/test_nufft.py:15-30)."""
    g = load_golden("ref_nufft_data")
    image, ktraj, kdata = g[f"image_{case}"], g[f"ktraj_{case}"], g[f"kdata_{case}"]
    ob = tkbn().KbNufft(im_size=image.shape[2:-1], dtype=torch.float64, device=DEV)
    out = ob(torch.tensor(image, device=DEV), torch.tensor(ktraj, device=DEV))
    assert torch.allclose(out.cpu(), torch.tensor(kdata))
    assert rel_l2(_np(out), kdata) < 1e-10


@pytest.mark.parametrize("name", ["nufft_1d", "nufft_2d", "nufft_2d_ortho", "nufft_2d_batched", "nufft_3d",
                                  "nufft_2d_grid", "nufft_2d_c128"])
def test_live_nufft_fixtures(name):
    g = load_golden("live_" + name)
    cd = torch.complex64 if g["image"].dtype == np.complex64 else torch.complex128
    tol = 1e-5 if cd == torch.complex64 else 1e-10
    norm = str(g["norm"]) or None
    im_size = g["image"].shape[2:]
    gs = tuple(int(x) for x in g["grid_size"])
    fwd = tkbn().KbNufft(im_size=im_size, grid_size=gs, dtype=cd, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, grid_size=gs, dtype=cd, device=DEV)
    t = lambda k: torch.tensor(g[k], device=DEV)
    om = t("omega")
    assert rel_l2(_np(fwd(t("image"), om, smaps=t("smaps"), norm=norm)), g["kdata_sense"]) < tol
    assert rel_l2(_np(adj(t("kdata_in"), om, smaps=t("smaps"), norm=norm)), g["image_sense"]) < tol
    assert rel_l2(_np(fwd(t("image_coils"), om, norm=norm)), g["kdata_plain"]) < tol
    assert rel_l2(_np(adj(t("kdata_in"), om, norm=norm)), g["image_plain"]) < tol


@pytest.mark.parametrize("im_size, B, C, M, norm, smaps_batch", [
    ((64, 60), 2, 8, 12000, None, 2),
    ((48, 48), 3, 4, 6000, "ortho", 1),
    ((20, 18, 16), 1, 3, 5000, None, 1),
    ((120,), 2, 2, 800, "ortho", 2),
])
def test_sense_nufft_vs_oracle(im_size, B, C, M, norm, smaps_batch):
    gen = torch.Generator().manual_seed(sum(im_size) + C)
    x = _rand(gen, (B, 1) + im_size, torch.complex64)
    s = _rand(gen, (smaps_batch, C) + im_size, torch.complex64)
    om = ((torch.rand((len(im_size), M), generator=gen) * 2 - 1) * np.pi).float()
    y = _rand(gen, (B, C, M), torch.complex64)
    fwd = tkbn().KbNufft(im_size=im_size, dtype=torch.complex64, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, dtype=torch.complex64, device=DEV)
    op = O.Operator(im_size, cdtype=np.complex64)
    out = fwd(x.to(DEV), om.to(DEV), smaps=s.to(DEV), norm=norm)
    assert rel_l2(_np(out), op.forward(x.numpy(), om.numpy(), smaps=s.numpy(), norm=norm)) < 1e-5
    img = adj(y.to(DEV), om.to(DEV), smaps=s.to(DEV), norm=norm)
    assert rel_l2(_np(img), op.adjoint(y.numpy(), om.numpy(), smaps=s.numpy(), norm=norm)) < 1e-5


@pytest.mark.parametrize("shape, kdata_shape", [
    ([4, 3, 19], [4, 3, 25]), ([2, 4, 32, 16], [2, 4, 83]), ([3, 10, 13, 18, 12], [3, 10, 112]),
])
def test_sense_nufft_adjointness(shape, kdata_shape):
    """<A x, y> == <x, A^H y> with maps (reference tests/test_sense_nufft.py:78-116)."""
    gen = torch.Generator().manual_seed(123)
    im_size = tuple(shape[2:])
    x = _rand(gen, (shape[0], 1) + im_size, torch.complex128).to(DEV)
    s = _rand(gen, tuple(shape), torch.complex128).to(DEV)
    y = _rand(gen, tuple(kdata_shape), torch.complex128).to(DEV)
    om = ((torch.rand((len(im_size), kdata_shape[2]), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    fwd = tkbn().KbNufft(im_size=im_size, dtype=torch.complex128, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, dtype=torch.complex128, device=DEV)
    a = torch.vdot(y.flatten(), fwd(x, om, smaps=s).flatten())
    b = torch.vdot(adj(y, om, smaps=s).flatten(), x.flatten())
    assert torch.allclose(a, b)


def test_autograd_matches_adjoint_identity():
    """grad of 1/2||A x||^2 equals A^H A x (reference tests/conftest.py:56-87)."""
    gen = torch.Generator().manual_seed(11)
    im = (24, 20)
    x = _rand(gen, (2, 1) + im, torch.complex128).to(DEV).requires_grad_(True)
    s = _rand(gen, (2, 3) + im, torch.complex128).to(DEV)
    y = _rand(gen, (2, 3, 300), torch.complex128).to(DEV).requires_grad_(True)
    om = ((torch.rand((2, 300), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    fwd = tkbn().KbNufft(im_size=im, dtype=torch.complex128, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im, dtype=torch.complex128, device=DEV)
    yf = fwd(x, om, smaps=s)
    (yf.abs() ** 2 / 2).sum().backward()
    xa = adj(y, om, smaps=s)
    (xa.abs() ** 2 / 2).sum().backward()
    assert torch.allclose(x.grad, adj(yf.detach(), om, smaps=s))
    assert torch.allclose(y.grad, fwd(xa.detach(), om, smaps=s))


def test_smaps_gradient_matches_torch_composition():
    """Gradient w.r.t. smaps equals autograd through an explicit image*smaps product."""
    gen = torch.Generator().manual_seed(12)
    im = (16, 18)
    x = _rand(gen, (2, 1) + im, torch.complex128).to(DEV)
    s = _rand(gen, (2, 3) + im, torch.complex128).to(DEV).requires_grad_(True)
    om = ((torch.rand((2, 200), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    fwd = tkbn().KbNufft(im_size=im, dtype=torch.complex128, device=DEV)
    (fwd(x, om, smaps=s).abs() ** 2).sum().backward()
    g1 = s.grad.clone()
    s2 = s.detach().clone().requires_grad_(True)
    (fwd(x * s2, om).abs() ** 2).sum().backward()
    assert torch.allclose(g1, s2.grad)


def test_dtype_and_norm_errors():
    ob = tkbn().KbNufft(im_size=(8, 8), dtype=torch.complex64, device=DEV)
    x = torch.zeros((1, 1, 8, 8), dtype=torch.complex64, device=DEV)
    om = torch.zeros((2, 4), device=DEV)
    with pytest.raises(TypeError):
        ob(x, om, smaps=torch.zeros((1, 2, 8, 8), dtype=torch.complex128, device=DEV))
    with pytest.raises(ValueError):
        ob(x, om, norm="forward")
    with pytest.raises(ValueError):
        ob(torch.zeros((1, 1, 8, 8, 3), device=DEV), om)
    with pytest.raises(ValueError):
        ob(torch.zeros((2, 1, 8, 8), dtype=torch.complex64, device=DEV), torch.zeros((3, 2, 4), device=DEV))
    with pytest.raises(TypeError):
        ob(x, om, interp_mats=om)


def test_module_to_and_state_dict():
    ob = tkbn().KbNufft(im_size=(12, 10))
    assert ob.table_0.dtype == torch.complex64
    ob = ob.to(DEV).to(torch.complex128)
    assert ob.table_0.dtype == torch.complex128 and ob.n_shift.dtype == torch.float64
    assert ob.offsets.dtype == torch.long and ob.table_0.is_cuda
    names = set(ob.state_dict().keys())
    assert {"table_0", "table_1", "im_size", "grid_size", "n_shift", "numpoints", "offsets", "table_oversamp",
            "order", "alpha", "scaling_coef"} <= names
