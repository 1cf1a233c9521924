"""Trajectory (ktraj) gradients from the hand-written backward (K7).

The table operator is piecewise constant in omega (nearest table bin), so its
finite differences are meaningless; the gradient is that of the smooth KB
interpolation the table samples. It is checked against central finite
differences (h = 1e-4) of the exact-KB operator in complex128 (oracle), to a
relative L2 error of 1e-4.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import kbnufft_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
H = 1e-4
TOL = 1e-4


def tkbn():
    import torchkbnufft_gb300 as m

    return m


def _rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _away_from_edges(om, im_size, J=6, margin=2e-3):
    """Move coordinates whose footprint start is within `margin` cells of switching.

    There the truncated KB kernel jumps (KB(+-J/2) ~ 1e-5), so a central
    difference across the switch does not approximate the derivative.
    """
    om = om.copy()
    K = 2 * np.asarray(im_size, dtype=np.float64).reshape(-1, 1)
    tm = om / (2 * np.pi / K)
    f = (tm - J / 2) - np.floor(tm - J / 2)
    bad = np.minimum(f, 1 - f) < margin
    om = om + bad * (4 * margin) * (2 * np.pi / K)
    return om


def _fd(fun, om):
    g = np.zeros_like(om)
    for idx in np.ndindex(om.shape):
        p = om.copy()
        p[idx] += H
        m = om.copy()
        m[idx] -= H
        g[idx] = (fun(p) - fun(m)) / (2 * H)
    return g


@pytest.mark.parametrize("im_size, smaps, norm", [((12, 10), True, None), ((16,), False, "ortho"),
                                                   ((6, 8, 6), True, None)])
def test_forward_ktraj_grad_vs_fd(im_size, smaps, norm):
    rng = np.random.default_rng(0)
    M, C = 24, 2
    x = _rand(rng, (1, 1 if smaps else C) + im_size)
    s = _rand(rng, (1, C) + im_size) if smaps else None
    v = _rand(rng, (1, C, M))
    om = _away_from_edges(rng.uniform(-np.pi, np.pi, (len(im_size), M)), im_size)

    def loss(o):
        y = O.exact_nufft_forward(x, o, im_size, smaps=s, norm=norm)
        return float(np.real(np.vdot(v, y)))

    fd = _fd(loss, om)
    ob = tkbn().KbNufft(im_size=im_size, dtype=torch.complex128, device=DEV)
    omt = torch.tensor(om, device=DEV, requires_grad=True)
    y = ob(torch.tensor(x, device=DEV), omt, smaps=None if s is None else torch.tensor(s, device=DEV), norm=norm)
    torch.real(torch.vdot(torch.tensor(v, device=DEV).flatten(), y.flatten())).backward()
    assert rel_l2(omt.grad.cpu().numpy(), fd) < TOL


@pytest.mark.parametrize("im_size", [(10, 12), (6, 6, 8)])
def test_adjoint_ktraj_grad_vs_fd(im_size):
    rng = np.random.default_rng(1)
    M, C = 20, 2
    y = _rand(rng, (1, C, M))
    s = _rand(rng, (1, C) + im_size)
    u = _rand(rng, (1, 1) + im_size)
    om = _away_from_edges(rng.uniform(-np.pi, np.pi, (len(im_size), M)), im_size)

    def loss(o):
        return float(np.real(np.vdot(u, O.exact_nufft_adjoint(y, o, im_size, smaps=s))))

    fd = _fd(loss, om)
    ob = tkbn().KbNufftAdjoint(im_size=im_size, dtype=torch.complex128, device=DEV)
    omt = torch.tensor(om, device=DEV, requires_grad=True)
    x = ob(torch.tensor(y, device=DEV), omt, smaps=torch.tensor(s, device=DEV))
    torch.real(torch.vdot(torch.tensor(u, device=DEV).flatten(), x.flatten())).backward()
    assert rel_l2(omt.grad.cpu().numpy(), fd) < TOL


def test_normal_operator_loss_grad_vs_fd():
    """Loss ||A^H A x - x||^2 (batched), gradients w.r.t. ktraj and x.

    The loss is nonlinear, so the table operator's own values enter the
    gradient; a 2^16 table oversampling makes them agree with the exact-KB
    operator (nearest-bin error ~1e-8) so that the comparison with finite
    differences of the exact operator isolates the derivative itself.
    """
    rng = np.random.default_rng(2)
    im_size, M, C, B = (10, 10), 30, 2, 2
    x = _rand(rng, (B, 1) + im_size)
    s = _rand(rng, (B, C) + im_size) * 0.3
    om = _away_from_edges(rng.uniform(-np.pi, np.pi, (2, M)), im_size)

    def loss(o):
        r = O.exact_nufft_adjoint(O.exact_nufft_forward(x, o, im_size, smaps=s), o, im_size, smaps=s) - x
        return float(np.sum(np.abs(r) ** 2))

    fd = _fd(loss, om)
    fwd = tkbn().KbNufft(im_size=im_size, table_oversamp=2**16, dtype=torch.complex128, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, table_oversamp=2**16, dtype=torch.complex128, device=DEV)
    omt = torch.tensor(om, device=DEV, requires_grad=True)
    xt = torch.tensor(x, device=DEV, requires_grad=True)
    st = torch.tensor(s, device=DEV)
    r = adj(fwd(xt, omt, smaps=st), omt, smaps=st) - xt
    (r.abs() ** 2).sum().backward()
    assert rel_l2(omt.grad.cpu().numpy(), fd) < TOL
    # image gradient: 2 (A^H A - I)^H r with the table operator
    with torch.no_grad():
        rr = r.detach()
        expect = 2 * (adj(fwd(rr, omt, smaps=st), omt, smaps=st) - rr)
    assert torch.allclose(xt.grad, expect)


def test_interp_level_ktraj_grad_vs_fd():
    """KbInterp / KbInterpAdjoint (no FFT) ktraj gradients."""
    rng = np.random.default_rng(3)
    K, M, C = (16, 14), 25, 3
    grid = _rand(rng, (1, C) + K)
    v = _rand(rng, (1, C, M))
    om = _away_from_edges(rng.uniform(-np.pi, np.pi, (2, M)), tuple(k // 2 for k in K))

    def loss(o):
        return float(np.real(np.vdot(v, O.exact_kb_interp(grid, o, K))))

    fd = _fd(loss, om)
    ob = tkbn().KbInterp(im_size=K, grid_size=K, dtype=torch.complex128, device=DEV)
    omt = torch.tensor(om, device=DEV, requires_grad=True)
    y = ob(torch.tensor(grid, device=DEV), omt)
    torch.real(torch.vdot(torch.tensor(v, device=DEV).flatten(), y.flatten())).backward()
    assert rel_l2(omt.grad.cpu().numpy(), fd) < TOL

    g2 = _rand(rng, (1, C) + K)

    def loss2(o):
        return float(np.real(np.vdot(g2, O.exact_kb_interp_adjoint(v, o, K, K))))

    fd2 = _fd(loss2, om)
    ob2 = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex128, device=DEV)
    omt2 = torch.tensor(om, device=DEV, requires_grad=True)
    x = ob2(torch.tensor(v, device=DEV), omt2)
    torch.real(torch.vdot(torch.tensor(g2, device=DEV).flatten(), x.flatten())).backward()
    assert rel_l2(omt2.grad.cpu().numpy(), fd2) < TOL


def test_float32_ktraj_grad_close_to_float64():
    rng = np.random.default_rng(4)
    im, M, C = (32, 32), 500, 4
    x = _rand(rng, (1, 1) + im)
    s = _rand(rng, (1, C) + im)
    om = rng.uniform(-np.pi, np.pi, (2, M))
    grads = []
    for cd in (torch.complex64, torch.complex128):
        ob = tkbn().KbNufft(im_size=im, dtype=cd, device=DEV)
        rd = torch.float32 if cd == torch.complex64 else torch.float64
        omt = torch.tensor(om, dtype=rd, device=DEV, requires_grad=True)
        y = ob(torch.tensor(x, dtype=cd, device=DEV), omt, smaps=torch.tensor(s, dtype=cd, device=DEV))
        (y.abs() ** 2).sum().backward()
        grads.append(omt.grad.double().cpu().numpy())
    assert rel_l2(grads[0], grads[1]) < 1e-3


def test_image_grad_matches_reference_autograd():
    """The image gradient of the trajectory-optimisation loss ||A^H A x - x||^2
    (summed over the batch, spiral trajectory, coil maps) against the gradient
    the reference's own autograd wrote (``_autograd/interp.py:78-178`` plus
    torch's FFT backward; fixture ``live_grad_x_spiral``), complex64 bar."""
    from conftest import load_golden

    g = load_golden("live_grad_x_spiral")
    im_size = g["image"].shape[2:]
    fwd = tkbn().KbNufft(im_size=im_size, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, device=DEV)
    x = torch.tensor(g["image"], device=DEV, requires_grad=True)
    s = torch.tensor(g["smaps"], device=DEV)
    om = torch.tensor(g["omega"], device=DEV, requires_grad=True)
    loss = (adj(fwd(x, om, smaps=s), om, smaps=s) - x).abs().pow(2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) / float(g["loss"]) < 1e-5
    assert rel_l2(x.grad.cpu().numpy(), g["grad"]) < 1e-5
    # the trajectory gradient (which the reference does not provide) is finite
    assert torch.isfinite(om.grad).all()
