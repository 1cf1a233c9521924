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
    want_k = op.forward(image, om, smaps=smaps)
    want = op.adjoint(want_k, om, smaps=smaps)
    got_k, got = P.forward_adjoint(image, smaps, om)
    assert rel_l2(got_k, want_k) < 2e-6
    assert rel_l2(got, want) < 2e-6


@pytest.mark.parametrize("name", ["nufft_2d", "nufft_3d"])
def test_port_nufft_matches_reference_fixtures(name):
    """The port's NUFFT helpers (used by the full-configuration GPU parity
    tests and the bench) against outputs written by the reference (default
    norm, one shared trajectory)."""
    g = load_golden("live_" + name)
    tol = 1e-6
    im_size = g["image"].shape[2:]
    om = g["omega"]
    assert rel_l2(P.nufft_forward(g["image"], om, g["smaps"]), g["kdata_sense"]) < tol
    assert rel_l2(P.nufft_adjoint(g["kdata_in"], om, im_size, g["smaps"]), g["image_sense"]) < tol
    assert rel_l2(P.nufft_forward(g["image_coils"], om), g["kdata_plain"]) < tol
    assert rel_l2(P.nufft_adjoint(g["kdata_in"], om, im_size), g["image_plain"]) < tol


def test_port_operator_matches_oracle_toeplitz_and_dcomp():
    """The C-port operator hook gives the numpy oracle's Toeplitz kernel and
    density compensation (the full-size GPU tests use it)."""
    g = load_golden("live_toep_2d_none")
    om, w = g["omega"], g["weights"]
    im_size = g["image"].shape[2:]
    want = O.toeplitz_kernel(om, im_size, weights=w)
    assert rel_l2(O.toeplitz_kernel(om, im_size, weights=w, operator_cls=P.PortOperator), want) < 2e-6
    assert rel_l2(want, g["kernel"]) < 1e-5
    d = load_golden("live_dcomp_2d")
    im = tuple(int(v) for v in d["im_size"])
    got = O.density_compensation(d["omega"], im, operator_cls=P.PortOperator)
    assert rel_l2(got, d["dcomp"]) < 1e-5
