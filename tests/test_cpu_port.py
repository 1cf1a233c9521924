"""The CPU port timed as the CPU baseline (``oracle/cpu_baseline.py`` over the
C restatement ``oracle/interp_oracle.c``) computes the reference path: its
interpolation against fixtures written by the reference, its SENSE forward +
adjoint against the oracle's (itself pinned to the reference)."""

import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import cpu_baseline as P
from oracle import kbnufft_oracle as O


@pytest.mark.parametrize("name", ["interp_1d", "interp_2d", "interp_3d", "interp_2d_c128"])
def test_port_interp_matches_reference(name):
    g = load_golden("live_" + name)
    cd = g["grid"].dtype
    im_size = g["grid"].shape[2:]
    op = O.Operator(im_size, grid_size=im_size, cdtype=cd)
    tol = 1e-6 if cd == np.complex64 else 1e-12
    assert rel_l2(P.interp_forward(op, g["grid"], g["omega"]), g["kdata"]) < tol
    assert rel_l2(P.interp_adjoint(op, g["kdata_in"], g["omega"]), g["grid_adj"]) < tol


def test_port_sense_forward_adjoint_matches_oracle():
    g = load_golden("live_nufft_2d")
    image, smaps, om = g["image"], g["smaps"], g["omega"]
    op = O.Operator(image.shape[2:], cdtype=np.complex64)
    want = op.adjoint(op.forward(image, om, smaps=smaps), om, smaps=smaps)
    assert rel_l2(P.forward_adjoint(image, smaps, om), want) < 2e-6
