"""Sparse-matrix interpolation (``interp_mats=``): matrix construction against
the reference's calc_tensor_spmatrix (fixtures written by the reference), and
the CUDA sparse interpolation / NUFFT against the reference's outputs.
"""

import numpy as np
import pytest
import torch

from conftest import load_golden, rel_l2

DEV = torch.device("cuda")


@pytest.mark.parametrize("name", ["spmat_2d", "spmat_3d"])
def test_calc_tensor_spmatrix_matches_reference(name):
    import torchkbnufft_gb300 as tkbn

    g = load_golden("live_" + name)
    im_size = g["image"].shape[2:]
    real, imag = tkbn.calc_tensor_spmatrix(torch.tensor(g["omega"]), im_size)
    assert real.shape == g["mat_real"].shape
    assert np.abs(real.to_dense().numpy() - g["mat_real"]).max() < 2e-6
    assert np.abs(imag.to_dense().numpy() - g["mat_imag"]).max() < 2e-6


@pytest.mark.parametrize("name", ["spmat_2d", "spmat_3d"])
def test_build_numpy_spmatrix_matches_reference(name):
    """``nufft_utils.build_numpy_spmatrix`` (the reference's complex scipy COO
    builder, same signature) holds the fixture's matrix as real + i imag."""
    import scipy.sparse

    import torchkbnufft_gb300 as tkbn

    g = load_golden("live_" + name)
    im_size = g["image"].shape[2:]
    om = torch.tensor(g["omega"])
    im, gs, J, ns, _, order, alpha, _, _ = tkbn.nufft_utils.validate_args(im_size, None, 6, None, 2**10, 2.34, 0.0,
                                                                          om.dtype, om.device)
    coo = tkbn.nufft_utils.build_numpy_spmatrix(om.numpy(), numpoints=J, im_size=im, grid_size=gs, n_shift=ns,
                                                order=order, alpha=alpha)
    assert scipy.sparse.issparse(coo) and coo.format == "coo" and coo.shape == g["mat_real"].shape
    dense = coo.toarray()
    assert np.abs(dense.real - g["mat_real"]).max() < 2e-6
    assert np.abs(dense.imag - g["mat_imag"]).max() < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["spmat_2d", "spmat_3d"])
def test_spmat_nufft_matches_reference(name):
    import torchkbnufft_gb300 as tkbn

    g = load_golden("live_" + name)
    im_size = tuple(g["image"].shape[2:])
    om = torch.tensor(g["omega"], device=DEV)
    mats = tkbn.calc_tensor_spmatrix(om, im_size)
    fwd = tkbn.KbNufft(im_size=im_size, device=DEV)
    adj = tkbn.KbNufftAdjoint(im_size=im_size, device=DEV)
    y = fwd(torch.tensor(g["image"], device=DEV), om, interp_mats=mats)
    assert rel_l2(y.cpu().numpy(), g["kdata"]) < 1e-5
    x = adj(torch.tensor(g["kdata_in"], device=DEV), om, interp_mats=mats)
    assert rel_l2(x.cpu().numpy(), g["image_adj"]) < 1e-5


@pytest.mark.gpu
def test_spmat_interp_is_the_matrix_product_and_adjoint():
    import torchkbnufft_gb300 as tkbn

    gen = torch.Generator().manual_seed(3)
    K = (20, 18)
    om = ((torch.rand((2, 300), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).to(DEV)
    mats = tkbn.calc_tensor_spmatrix(om, (10, 9), grid_size=K)
    A = (mats[0].to_dense() + 1j * mats[1].to_dense()).cpu()
    grid = torch.view_as_complex(torch.randn((2, 3) + K + (2,), generator=gen, dtype=torch.float64))
    y = tkbn.KbInterp(im_size=(10, 9), grid_size=K, dtype=torch.complex128, device=DEV)(grid.to(DEV), om,
                                                                                          interp_mats=mats)
    ref = (A @ grid.reshape(6, -1).T).T.reshape(2, 3, -1)
    assert rel_l2(y.cpu().numpy(), ref.numpy()) < 1e-12
    kin = torch.view_as_complex(torch.randn((2, 3, 300, 2), generator=gen, dtype=torch.float64))
    x = tkbn.KbInterpAdjoint(im_size=(10, 9), grid_size=K, dtype=torch.complex128, device=DEV)(
        kin.to(DEV), om, interp_mats=mats)
    ref = (A.conj().T @ kin.reshape(6, -1).T).T.reshape((2, 3) + K)
    assert rel_l2(x.cpu().numpy(), ref.numpy()) < 1e-12
    # autograd: the backward of the forward is the adjoint
    g2 = grid.to(DEV).requires_grad_(True)
    out = tkbn.functional.kb_spmat_interp(g2, mats)
    (out.abs() ** 2).sum().backward()
    expect = tkbn.functional.kb_spmat_interp_adjoint(2 * out.detach(), mats, torch.tensor(K))
    assert rel_l2(g2.grad.cpu().numpy(), expect.cpu().numpy()) < 1e-12
