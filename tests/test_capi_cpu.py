"""The C-ABI library loads here (no GPU) and exports every declared entry point.

No compute calls: only functions that never touch the device are invoked.
"""

import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _header():
    with open(os.path.join(ROOT, "include", "tkbn_gb300.h")) as f:
        return f.read()


def _declared():
    src = _header()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(tkbn_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from torchkbnufft_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "tkbn_interp_fwd" in names and "tkbn_nufft_adj" in names and len(names) >= 16


def test_library_exports_every_declared_symbol(lib):
    from torchkbnufft_gb300 import _build

    out = subprocess.run(["nm", "-D", "--defined-only", _build.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(tkbn_\w+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    for n in _declared():
        assert getattr(lib, n) is not None


def test_python_binding_covers_header():
    from torchkbnufft_gb300 import _lib

    assert set(_declared()) == set(_lib.SIGNATURES)


def test_python_constants_match_header():
    """Every integer #define of the header has a Python constant of the same value."""
    from torchkbnufft_gb300 import _lib

    src = _header()
    defs = dict(re.findall(r"^#define\s+(TKBN_\w+)\s+\(?(-?\d+)\)?", src, re.M))
    assert "TKBN_ADJ_REUSE_FACTORS" in defs and "TKBN_TABLES_LINEAR_PHASE" in defs
    for name, value in defs.items():
        if name == "TKBN_GB300_H":
            continue
        assert getattr(_lib, name, None) == int(value), name


def test_abi_version(lib):
    assert lib.tkbn_abi_version() == 1


def test_host_side_argument_errors(lib):
    """Argument validation happens on the host before any CUDA call."""
    from torchkbnufft_gb300 import _lib

    g = _lib.Geometry()
    g.ndim = 4
    g.dtype = _lib.TKBN_C64
    n = ctypes.c_size_t(0)
    p = _lib.PointsDesc()
    p.npts, p.ntraj = 10, 1
    rc = lib.tkbn_points_workspace_size(ctypes.byref(g), ctypes.byref(p), ctypes.byref(n))
    assert rc == _lib.TKBN_ERR_UNSUPPORTED
    assert b"ndim" in lib.tkbn_last_error()
    g.ndim = 2
    g.dtype = 7
    rc = lib.tkbn_interp_fwd(ctypes.byref(g), ctypes.byref(p), None, None, None, 1, 1, None, None)
    assert rc == _lib.TKBN_ERR_UNSUPPORTED
    g.dtype = _lib.TKBN_C64
    for d in range(2):
        g.grid_size[d] = 0
    rc = lib.tkbn_interp_fwd(ctypes.byref(g), ctypes.byref(p), None, None, None, 1, 1, None, None)
    assert rc == _lib.TKBN_ERR_INVALID
    with pytest.raises(ValueError):
        _lib.check(rc)


def test_cpu_tensors_are_rejected():
    """No CPU fallback: the product path raises on CPU tensors."""
    import torch

    import torchkbnufft_gb300 as tkbn

    ob = tkbn.KbNufft(im_size=(8, 8))
    x = torch.randn(1, 1, 8, 8, dtype=torch.complex64)
    om = torch.rand(2, 10) * 2 - 1
    with pytest.raises(RuntimeError, match="CUDA"):
        ob(x, om)


def test_linear_phase_table_check():
    """The host sets TKBN_TABLES_LINEAR_PHASE only for tables of the form
    |h(u)| e^{icu}: the module's Kaiser-Bessel tables pass, a table with one
    entry's phase perturbed does not, and a magnitude change keeps the form."""
    import cmath

    import torch

    import torchkbnufft_gb300 as tk
    from torchkbnufft_gb300 import _runtime as R

    for im in [(320, 320), (40, 32, 48), (64,)]:
        m = tk.KbNufft(im_size=im)
        for d in range(len(im)):
            assert R._linear_phase(getattr(m, f"table_{d}"))
    t = tk.KbNufft(im_size=(320, 320)).table_0
    bad = t.clone()
    bad[3000] *= complex(cmath.exp(0.01j))
    assert not R._linear_phase(bad)
    scaled = t.clone()
    scaled[100] *= 1.01
    assert R._linear_phase(scaled)
    assert not R._linear_phase(t.to(torch.complex128))  # the linear-phase kernels are complex64


def test_factor_reuse_key():
    """A call reuses the layout's per-point factors only for tables with the
    contents (unmodified since) and table flags they were computed with."""
    import torch

    from torchkbnufft_gb300 import _runtime as R

    a, b = torch.ones(5, dtype=torch.complex64), torch.ones(5, dtype=torch.complex64)
    stored = ((a, b), (a._version, b._version), 9)
    assert R.factors_reusable(stored, [a, b], 9)
    assert not R.factors_reusable(None, [a, b], 9)
    assert not R.factors_reusable(stored, [a, b], 1)  # other table flags
    assert R.factors_reusable(stored, [a, b.clone()], 9)  # same contents, another tensor
    other = b.clone()
    other[0] = 2
    assert not R.factors_reusable(stored, [a, other], 9)  # other contents
    assert not R.factors_reusable(stored, [a, torch.ones(6, dtype=torch.complex64)], 9)
    assert not R.factors_reusable(stored, [a], 9)
    a.mul_(2)
    assert not R.factors_reusable(stored, [a, b], 9)  # changed in place


def test_missing_library_raises_instead_of_falling_back():
    """Without the CUDA library the package raises; there is no CPU path to fall back to."""
    import sys

    code = (
        "import torchkbnufft_gb300._build as B, torchkbnufft_gb300._lib as L\n"
        "B.lib_path = lambda: '/nonexistent/libtkbn_gb300.so'\n"
        "try:\n"
        "    L.load(build_if_missing=False)\n"
        "except RuntimeError as e:\n"
        "    print('raised:', e)\n"
        "try:\n"
        "    L.load(path='/nonexistent/libtkbn_gb300.so')\n"
        "except OSError:\n"
        "    print('raised: OSError')\n"
    )
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "raised: CUDA library not built" in out.stdout and "raised: OSError" in out.stdout, out.stdout


def test_factor_reuse_is_off_under_graph_capture(monkeypatch):
    """A call captured into a CUDA graph always carries the pre-pass and leaves
    no record (nothing ran at capture time); eager calls reuse as before."""
    import torch

    from torchkbnufft_gb300 import _lib as L
    from torchkbnufft_gb300 import _runtime as R

    lay = object.__new__(R.PointsLayout)  # the host logic only: no workspace
    lay.flags, lay.device, lay._factors = 0, torch.device("cuda", 0), None
    tabs = [torch.ones(5, dtype=torch.complex64)]
    seen = []
    capturing = [False]
    monkeypatch.setattr(R, "stream_capturing", lambda device: capturing[0])
    lay.factor_call(tabs, 9, seen.append)  # eager: computes, records
    lay.factor_call(tabs, 9, seen.append)  # eager: reuses
    capturing[0] = True
    lay.factor_call(tabs, 9, seen.append)  # captured: recomputes, no record
    capturing[0] = False
    lay.factor_call(tabs, 9, seen.append)  # eager after capture: recomputes
    lay.factor_call(tabs, 9, seen.append)  # and reuses again
    reuse = [bool(f & L.TKBN_ADJ_REUSE_FACTORS) for f in seen]
    assert reuse == [False, True, False, False, True]
    assert all(f & ~L.TKBN_ADJ_REUSE_FACTORS == 9 for f in seen)
