"""The trajectory-layout cache's policy, on the CPU with a stand-in layout
(building a real layout needs the GPU): in-place updates of omega keep one
entry, a freed trajectory leaves the cache, and the byte cap holds."""

import gc

import pytest
import torch

from torchkbnufft_gb300 import _runtime as R


class _FakeLayout:
    built = 0

    def __init__(self, geom, omega, tile, chunk, deterministic):
        _FakeLayout.built += 1
        self.nbytes = 1000


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(R, "PointsLayout", _FakeLayout)
    R._layout_cache.clear()
    _FakeLayout.built = 0
    yield
    R._layout_cache.clear()


GEOM = R.GeomKey(2, 0, (8, 8), (16, 16), (6, 6), (1024, 1024), (4.0, 4.0))


def test_in_place_updates_keep_one_entry(fake):
    om = torch.zeros((2, 100))
    for step in range(20):
        lay = R.points_layout(GEOM, om)
        assert R.points_layout(GEOM, om) is lay  # a hit while unchanged
        with torch.no_grad():
            om.add_(1e-3)  # an optimiser step in place
    assert _FakeLayout.built == 20
    assert R.layout_cache_info()[0] == 1


def test_freed_trajectory_leaves_the_cache(fake):
    om = torch.zeros((2, 100))
    R.points_layout(GEOM, om)
    other = torch.zeros((2, 50))
    R.points_layout(GEOM, other)
    assert R.layout_cache_info()[0] == 2
    del om
    gc.collect()
    assert R.layout_cache_info()[0] == 1


def test_byte_cap_keeps_the_newest(fake, monkeypatch):
    monkeypatch.setenv("TKBN_LAYOUT_CACHE_BYTES", "2500")
    keep = [torch.zeros((2, 10 + i)) for i in range(5)]
    for om in keep:
        R.points_layout(GEOM, om)
    n, nbytes = R.layout_cache_info()
    assert n == 2 and nbytes == 2000
    monkeypatch.setenv("TKBN_LAYOUT_CACHE_BYTES", "10")
    newest = torch.zeros((2, 3))
    R.points_layout(GEOM, newest)
    assert R.layout_cache_info()[0] == 1  # the newest layout stays even above the cap
