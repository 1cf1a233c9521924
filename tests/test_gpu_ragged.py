"""Ragged batches (K8): many problems with different image sizes, point counts
and coil counts in one launch per interpolation stage, and as one CUDA graph.

Each problem must give what a per-problem KbNufft / KbNufftAdjoint call gives
(the reference's way: one call per problem, torchkbnufft/modules/kbnufft.py).
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
# per-problem calls and the ragged launch agree to the complex64 parity bar:
# with linear-phase tables a per-problem 2D adjoint of 16 coils accumulates
# real kernel values and applies the phases per point and per cell, while the
# ragged launch multiplies the complex table factors
TOL = 1e-5


def _problems(seed, spec):
    gen = torch.Generator().manual_seed(seed)
    probs, images = [], []
    for im, M, C in spec:
        om = ((torch.rand((2, M), generator=gen) * 2 - 1) * np.pi).to(DEV)
        x = torch.view_as_complex(torch.randn((1, C) + im + (2,), generator=gen)).to(DEV)
        probs.append((im, om, C))
        images.append(x)
    return probs, images


# image sizes, point counts and coil counts as in a ragged batch: 16-coil
# problems take the register adjoint, the others the generic one; 17 coils
# make two coil chunks; the 24x24 image gives a 48x48 grid
SPEC = [((32, 32), 9000, 16), ((48, 40), 20000, 3), ((32, 32), 1500, 1), ((24, 24), 12000, 17),
        ((48, 40), 700, 16), ((32, 32), 30000, 5)]


def _reference(probs, images):
    import torchkbnufft_gb300 as tkbn

    out_k, out_x = [], []
    for (im, om, C), x in zip(probs, images):
        fwd = tkbn.KbNufft(im_size=im, device=DEV)
        adj = tkbn.KbNufftAdjoint(im_size=im, device=DEV)
        y = fwd(x, om)
        out_k.append(y)
        out_x.append(adj(y, om))
    return out_k, out_x


def test_ragged_matches_per_problem_calls():
    import torchkbnufft_gb300 as tkbn

    probs, images = _problems(3, SPEC)
    rk, rx = _reference(probs, images)
    rn = tkbn.RaggedNufft(probs)
    ks = rn.forward(images)
    for a, b in zip(ks, rk):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < TOL
    xs = rn.adjoint()
    for a, b in zip(xs, rx):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < TOL


def test_ragged_graph_replay_matches_eager():
    import torchkbnufft_gb300 as tkbn

    probs, images = _problems(4, SPEC)
    rn = tkbn.RaggedNufft(probs)
    rn.set_images(images)
    rn.forward_adjoint()
    torch.cuda.synchronize()
    eager = [rn.output_view(p).clone() for p in range(len(SPEC))]
    rn.capture()
    for p in range(len(SPEC)):
        rn.output_view(p).zero_()
    rn.replay()
    rn.replay()
    torch.cuda.synchronize()
    for p in range(len(SPEC)):
        assert rel_l2(rn.output_view(p).cpu().numpy(), eager[p].cpu().numpy()) < TOL
    # new inputs through the same graph
    _, images2 = _problems(5, SPEC)
    rn.set_images(images2)
    rn.replay()
    _, rx2 = _reference(probs, images2)
    for p in range(len(SPEC)):
        assert rel_l2(rn.output_view(p).cpu().numpy(), rx2[p].cpu().numpy()) < TOL


def test_ragged_with_autotuned_layouts():
    import torchkbnufft_gb300 as tkbn

    probs, images = _problems(6, SPEC[:3])
    rk, rx = _reference(probs, images)
    rn = tkbn.RaggedNufft(probs, autotune_layout=True)
    for (tile, chunk) in rn.tiles.values():
        assert tile is not None and chunk > 0
    ks = rn.forward(images)
    xs = rn.adjoint()
    for a, b in zip(ks, rk):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < TOL
    for a, b in zip(xs, rx):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < TOL


def test_ragged_rejects_batched_trajectories():
    import torchkbnufft_gb300 as tkbn

    om = torch.zeros((2, 2, 100), device=DEV)
    with pytest.raises(ValueError):
        tkbn.RaggedNufft([((16, 16), om, 1)])
