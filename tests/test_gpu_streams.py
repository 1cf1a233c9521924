"""Calls that share a cached trajectory layout from several CUDA streams.

The layout cache is keyed by the trajectory tensor, so calls on different
streams share one layout workspace. Its build must finish before another
stream reads it, and adjoints write per-point factor scratch into it, so
adjoints on different streams must not overlap. Each result is checked
against the oracle (complex64 bar, 1e-5 relative L2).
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import kbnufft_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL = 1e-5


def _cplx(gen, shape):
    return torch.view_as_complex(torch.randn(shape + (2,), generator=gen))


@pytest.mark.parametrize("C", [16, 3])
def test_adjoints_on_two_streams_share_a_layout(C):
    import torchkbnufft_gb300 as tkbn
    from torchkbnufft_gb300 import _runtime as R

    R.clear_caches()
    gen = torch.Generator().manual_seed(11 + C)
    im, M = (64, 64), 30000
    om = (torch.rand((2, M), generator=gen) * 2 - 1) * np.pi
    ks = [_cplx(gen, (1, C, M)) for _ in range(2)]
    adj = tkbn.KbNufftAdjoint(im_size=im, device=DEV)
    fwd = tkbn.KbNufft(im_size=im, device=DEV)
    omd = om.to(DEV)
    kd = [k.to(DEV) for k in ks]
    x = _cplx(gen, (1, C) + im)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    cur = torch.cuda.current_stream()
    for s in streams:
        s.wait_stream(cur)
    outs = [[], []]
    fouts = []
    # the first call (on the first stream) builds the layout; the second
    # stream then reads it, and the two streams' adjoints interleave
    for i in range(3):
        for j, s in enumerate(streams):
            with torch.cuda.stream(s):
                outs[j].append(adj(kd[j], omd))
                if i == 0 and j == 1:
                    fouts.append(fwd(x.to(DEV, non_blocking=False), omd))
    for s in streams:
        cur.wait_stream(s)
    torch.cuda.synchronize()
    op = O.Operator(im, cdtype=np.complex64)
    for j in range(2):
        want = op.adjoint(ks[j].numpy(), om.numpy())
        for o in outs[j]:
            assert rel_l2(o.cpu().numpy(), want) < TOL
    assert rel_l2(fouts[0].cpu().numpy(), op.forward(x.numpy(), om.numpy())) < TOL
