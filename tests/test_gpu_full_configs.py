"""GPU parity at every benchmark configuration, at its own size.

Each test builds the exact inputs that ``bench.py`` times (its seeded
generators) and compares the CUDA path, through the public modules, with the
CPU port of the reference table path (``oracle/cpu_baseline.py``: the C
restatement of ``torchkbnufft/_nufft/interp.py:88-203, 406-726`` plus
scipy FFTs, itself checked against fixtures written by the reference in
``test_cpu_port.py``). The bar is the complex64 parity bar, 1e-5 relative L2,
for the forward (k-space data) and the adjoint (image) separately; the
adjoint runs on the port's k-space data so that both sides see the same
input.

* single-coil radial: 256^2 image, 512^2 grid, 402 x 512 spokes, in full.
* SENSE: batch 4, 16 coils, 320^2, golden angle 404 x 640, in full; also the
  Toeplitz kernel, ToepNufft and the density compensation at that size.
* kooshball: 128^3, 8 coils, 20000 x 256 points. The GPU runs the full
  trajectory; the port evaluates a seeded 4096-point subset (the forward at
  those points; the adjoint of k-space data that is zero off the subset, so
  the GPU still walks every list entry of the full layout).
* spiral: batch 1, 16 coils, 256^2, 32 x 2048, in full.
* ragged: every problem of the 64-problem seeded draw, each against the port.
"""

import numpy as np
import pytest
import torch

import bench
from conftest import rel_l2
from oracle import cpu_baseline as P
from oracle import kbnufft_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL = 1e-5  # relative L2, complex64


def tkbn():
    import torchkbnufft_gb300 as m

    return m


def _np(t):
    return t.detach().cpu().numpy()


def _image(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _fwd_adj_parity(image, omega, smaps, im_size):
    """Forward and adjoint through KbNufft / KbNufftAdjoint against the port."""
    t = lambda a: None if a is None else torch.tensor(a, device=DEV)
    fwd = tkbn().KbNufft(im_size=im_size, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=im_size, device=DEV)
    om = t(omega)
    want_k = P.nufft_forward(image, omega, smaps)
    got_k = _np(fwd(t(image), om, smaps=t(smaps)))
    e_fwd = rel_l2(got_k, want_k)
    want_x = P.nufft_adjoint(want_k, omega, im_size, smaps)
    got_x = _np(adj(t(want_k), om, smaps=t(smaps)))
    e_adj = rel_l2(got_x, want_x)
    return e_fwd, e_adj


def test_single_coil_radial_full_size():
    rng = np.random.default_rng(1001)
    om = bench.radial_traj(402, 512)
    e_fwd, e_adj = _fwd_adj_parity(_image(rng, (1, 1, 256, 256)), om, None, (256, 256))
    assert e_fwd < TOL and e_adj < TOL, (e_fwd, e_adj)


def test_sense_full_size():
    """The headline workload: every kernel the bench times, at its size."""
    image, smaps, om = bench.make_inputs()
    e_fwd, e_adj = _fwd_adj_parity(image, om, smaps, (bench.N, bench.N))
    assert e_fwd < TOL and e_adj < TOL, (e_fwd, e_adj)


def test_sense_full_size_toeplitz_and_dcomp():
    image, smaps, om = bench.make_inputs()
    n = (bench.N, bench.N)
    t = lambda a: torch.tensor(a, device=DEV)
    dc = tkbn().calc_density_compensation_function(t(om), n)
    dc_ref = O.density_compensation(om, n, operator_cls=P.PortOperator)
    assert rel_l2(_np(dc), dc_ref) < TOL
    w = dc_ref[0]  # (1, M), as the reference's Toeplitz kernel takes it for a shared trajectory
    kern = tkbn().calc_toeplitz_kernel(t(om), n, weights=t(w))
    kern_ref = O.toeplitz_kernel(om, n, weights=w, operator_cls=P.PortOperator)
    assert rel_l2(_np(kern), kern_ref) < TOL
    out = tkbn().ToepNufft()(t(image), t(kern_ref), smaps=t(smaps))
    assert rel_l2(_np(out), O.toep_apply(image, kern_ref, smaps=smaps)) < TOL


def test_kooshball_subset():
    rng = np.random.default_rng(1003)
    om = bench.kooshball_traj(20000, 256)
    smaps = bench.smooth_maps_3d(8, 128, 3)
    image = _image(rng, (1, 1, 128, 128, 128))
    M = om.shape[1]
    sub = np.sort(rng.choice(M, 4096, replace=False))
    fwd = tkbn().KbNufft(im_size=(128,) * 3, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=(128,) * 3, device=DEV)
    om_d = torch.tensor(om, device=DEV)
    s_d = torch.tensor(smaps, device=DEV)
    y = fwd(torch.tensor(image, device=DEV), om_d, smaps=s_d)
    got_k = _np(y[..., torch.tensor(sub, device=DEV)])
    want_k = P.nufft_forward(image, om[:, sub], smaps)
    assert rel_l2(got_k, want_k) < TOL
    kfull = torch.zeros_like(y)
    kfull[..., torch.tensor(sub, device=DEV)] = torch.tensor(want_k, device=DEV)
    del y
    got_x = _np(adj(kfull, om_d, smaps=s_d))
    want_x = P.nufft_adjoint(want_k, om[:, sub], (128,) * 3, smaps)
    assert rel_l2(got_x, want_x) < TOL


def test_kooshball_full_size_adjointness():
    """<A x, y> = <x, A^H y> over the full 5.12M-point trajectory (no CPU work)."""
    gen = torch.Generator(device=DEV).manual_seed(5)
    om = torch.tensor(bench.kooshball_traj(20000, 256), device=DEV)
    s = torch.tensor(bench.smooth_maps_3d(8, 128, 3), device=DEV)
    x = torch.randn((1, 1) + (128,) * 3, dtype=torch.complex64, device=DEV, generator=gen)
    y = torch.randn((1, 8, om.shape[1]), dtype=torch.complex64, device=DEV, generator=gen)
    fwd = tkbn().KbNufft(im_size=(128,) * 3, device=DEV)
    adj = tkbn().KbNufftAdjoint(im_size=(128,) * 3, device=DEV)
    lhs = torch.vdot(fwd(x, om, smaps=s).flatten().to(torch.complex128), y.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), adj(y, om, smaps=s).flatten().to(torch.complex128))
    assert abs((lhs - rhs) / lhs).item() < TOL


def test_spiral_batch1_full_size():
    rng = np.random.default_rng(1004)
    om = bench.spiral_traj(32, 2048)
    smaps = bench.ring_smaps(16, 256, 1, 4)
    e_fwd, e_adj = _fwd_adj_parity(_image(rng, (1, 1, 256, 256)), om, smaps, (256, 256))
    assert e_fwd < TOL and e_adj < TOL, (e_fwd, e_adj)


def test_ragged_every_problem_against_port():
    """The 64-problem ragged draw, merged launches with autotuned layouts as the
    bench runs them; each problem's forward and adjoint against the port."""
    spec = bench.ragged_spec()
    rng = np.random.default_rng(7)
    probs, images = [], []
    for im, om, C in spec:
        probs.append((im, torch.tensor(om, device=DEV), C))
        images.append(_image(rng, (1, C) + im))
    rn = tkbn().RaggedNufft(probs, autotune_layout=True)
    ks = rn.forward([torch.tensor(x, device=DEV) for x in images])
    want_k = [P.nufft_forward(x, om, None) for x, (_, om, _) in zip(images, spec)]
    errs_k = [rel_l2(_np(a), b) for a, b in zip(ks, want_k)]
    xs = rn.adjoint([torch.tensor(k, device=DEV) for k in want_k])
    errs_x = [rel_l2(_np(a), P.nufft_adjoint(k, om, im, None)) for a, k, (im, om, _) in zip(xs, want_k, spec)]
    assert max(errs_k) < TOL, max(errs_k)
    assert max(errs_x) < TOL, max(errs_x)
