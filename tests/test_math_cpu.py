"""The complex helpers (``absolute``, ``complex_mult``, ``complex_sign``,
``conj_complex_mult``, ``imag_exp``, ``inner_product``) behave as
torchkbnufft's (``torchkbnufft/_math.py``; cases as ``tests/test_math.py``):
numpy products in the real (..., 2) layout at ``dim=-1`` and ``dim=2`` and in
the complex layout, plus the shapes, zero handling and errors of the others."""

import numpy as np
import pytest
import torch

import torchkbnufft_gb300 as tkbn


def _pair(z, dim=-1):
    return torch.stack((torch.tensor(np.real(z)), torch.tensor(np.imag(z))), dim)


def _unpair(t, dim=-1):
    t = t.numpy()
    return np.take(t, 0, axis=dim) + 1j * np.take(t, 1, axis=dim)


@pytest.fixture
def xy():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(8, 16, 10)) + 1j * rng.normal(size=(8, 16, 10))
    y = rng.normal(size=(8, 16, 10)) + 1j * rng.normal(size=(8, 16, 10))
    return x, y


@pytest.mark.parametrize("name, want", [("complex_mult", lambda x, y: x * y),
                                        ("conj_complex_mult", lambda x, y: x * np.conj(y))])
def test_products(name, want, xy):
    x, y = xy
    f = getattr(tkbn, name)
    assert np.allclose(_unpair(f(_pair(x), _pair(y))), want(x, y))
    assert np.allclose(_unpair(f(_pair(x, 2), _pair(y, 2), dim=2), 2), want(x, y))
    assert np.allclose(f(torch.tensor(x), torch.tensor(y)).numpy(), want(x, y))
    with pytest.raises(ValueError, match="different dtype"):
        f(torch.tensor(x), torch.tensor(y).to(torch.complex64))
    with pytest.raises(ValueError, match="dimension size 2"):
        f(torch.ones(3, 3), torch.ones(3, 3))


def test_absolute(xy):
    x, _ = xy
    r = tkbn.absolute(_pair(x, 2), dim=2)
    assert r.shape == (8, 16, 1, 10)  # the complex dim kept, size 1
    assert np.allclose(r[:, :, 0].numpy(), np.abs(x))
    assert np.allclose(tkbn.absolute(torch.tensor(x)).numpy(), np.abs(x))
    with pytest.raises(ValueError, match="dimension size 2"):
        tkbn.absolute(torch.ones(3, 3))


def test_complex_sign(xy):
    x, _ = xy
    x = x.copy()
    x[0, 0, :3] = 0
    want = np.exp(1j * np.arctan2(x.imag, x.real))  # 1 where x is 0
    c = tkbn.complex_sign(torch.tensor(x))
    assert c.is_complex() and np.allclose(c.numpy(), want)
    assert np.allclose(c.numpy()[0, 0, :3], 1.0)
    r = tkbn.complex_sign(_pair(x, 2), dim=2)
    assert r.shape == (8, 16, 10, 2)  # a real pair comes back on the last axis
    assert np.allclose(_unpair(r), want)


def test_imag_exp():
    t = torch.linspace(-7, 7, 101, dtype=torch.float64)
    assert np.allclose(tkbn.imag_exp(t).numpy(), np.exp(1j * t.numpy()))
    r = tkbn.imag_exp(t, return_complex=False)
    assert r.shape == (101, 2) and np.allclose(_unpair(r), np.exp(1j * t.numpy()))


def test_inner_product(xy):
    x, y = xy
    want = np.vdot(x, y)  # sum(conj(x) * y)
    assert np.allclose(tkbn.inner_product(torch.tensor(x), torch.tensor(y)).numpy(), want)
    r = tkbn.inner_product(_pair(x, 2), _pair(y, 2), dim=2)
    assert r.shape == (2,) and np.allclose(r[0] + 1j * r[1], want)
    with pytest.raises(ValueError, match="different dtype"):
        tkbn.inner_product(_pair(x), _pair(y).float())
