"""Host setup against the reference: every buffer of a KbNufft (the per-dim
interpolation tables, the scaling coefficients and the parsed arguments)
equals the reference module's for the same arguments (fixtures written by the
reference's own KbNufft in complex128, ``tests/golden/make_golden.py``).

This pins the inputs that the oracle and the CUDA kernels share: tables
(``torchkbnufft/_nufft/utils.py:122-179``), scaling coefficients
(``utils.py:182-254``) and ``validate_args`` (``utils.py:361-427``).
"""

import ast

import numpy as np
import pytest
import torch

from conftest import load_golden

CASES = ["setup_1d_default", "setup_2d", "setup_2d_custom", "setup_3d"]


def _module(g, dtype):
    import torchkbnufft_gb300 as tkbn

    return tkbn.KbNufft(dtype=dtype, **ast.literal_eval(str(g["kwargs"])))


@pytest.mark.parametrize("name", CASES)
def test_buffers_match_reference(name):
    g = load_golden("live_" + name)
    mine = {k: v.numpy() for k, v in _module(g, torch.complex128).state_dict().items()}
    ref = {k: v for k, v in g.items() if k != "kwargs" and not k.startswith("c64_")}
    assert set(mine) == set(ref)
    for k, want in ref.items():
        got = mine[k]
        assert got.shape == want.shape and got.dtype == want.dtype, (k, got.shape, want.shape, got.dtype, want.dtype)
        if np.issubdtype(want.dtype, np.complexfloating) or np.issubdtype(want.dtype, np.floating):
            scale = max(float(np.abs(want).max()), 1e-300)
            assert float(np.abs(got - want).max()) <= 1e-12 * scale, k
        else:
            assert np.array_equal(got, want), k


@pytest.mark.parametrize("name", CASES)
def test_complex64_buffers_match_reference(name):
    """The complex64 module's tables and scaling coefficients equal the
    reference's complex64 module's (bitwise in practice; a last-bit flip of a
    tiny tail entry is allowed)."""
    g = load_golden("live_" + name)
    sd = _module(g, torch.complex64).state_dict()
    keys = [k for k in g if k.startswith("c64_")]
    assert {k[4:] for k in keys} == {k for k, v in sd.items() if v.is_complex()}
    for k in keys:
        got, want = sd[k[4:]].numpy(), g[k]
        assert got.dtype == want.dtype == np.complex64 and got.shape == want.shape, k
        assert float(np.abs(got - want).max()) <= 1e-7 * float(np.abs(want).max()), k
        assert np.count_nonzero(got != want) <= max(1, want.size // 1000), k
