"""Generate the golden fixtures in this folder from the reference implementation.

Run where the reference (mmuckley/torchkbnufft) source tree is available,
giving its location as the argument or in ``TKBN_REFERENCE``::

    python tests/golden/make_golden.py <path to the reference source tree>

Two kinds of fixtures are written:

* ``ref_interp_data.npz`` / ``ref_nufft_data.npz`` — the reference's own
  golden vectors (``tests/data/interp_data.pkl``, ``tests/data/nufft_data.pkl``,
  float64, real ``(..., 2)`` layout), converted to numpy without change.
* ``live_*.npz`` — outputs of the reference's public API run here on seeded
  inputs, complex64 unless the name says c128. These pin the oracle and the
  CUDA path to the reference's table mode at the working precision.
  ``live_setup_*`` hold every buffer of a complex128 KbNufft and the complex
  buffers of a complex64 one (tables, scaling coefficients, parsed arguments).

The tests only read the ``.npz`` files; nothing at test time needs the reference.
``TKBN_GOLDEN_ONLY=<prefix>`` rewrites only the live fixtures with that prefix.
"""

from __future__ import annotations

import os
import pickle
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = None  # the reference source tree, from the command line or TKBN_REFERENCE


def _np(t):
    return t.detach().cpu().numpy()


def convert_reference_pickles():
    for name in ("interp_data", "nufft_data"):
        with open(os.path.join(REF, "tests", "data", name + ".pkl"), "rb") as f:
            cases = pickle.load(f)
        out = {}
        for i, (image, ktraj, kdata) in enumerate(cases):
            out[f"image_{i}"] = _np(image)
            out[f"ktraj_{i}"] = _np(ktraj)
            out[f"kdata_{i}"] = _np(kdata)
        out["ncases"] = np.array(len(cases))
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)


def _cplx(gen, shape, dtype):
    re = torch.randn(shape, generator=gen, dtype=torch.float64)
    im = torch.randn(shape, generator=gen, dtype=torch.float64)
    return torch.complex(re, im).to(dtype)


def _traj(gen, shape, rdtype):
    return (torch.rand(shape, generator=gen, dtype=torch.float64) * 2 * np.pi - np.pi).to(rdtype)


def live_cases():
    import torchkbnufft as tkbn

    torch.set_default_dtype(torch.float32)
    cases = {}

    def interp_case(name, shape, M, batched=False, cdtype=torch.complex64, seed=0):
        rdtype = torch.float32 if cdtype == torch.complex64 else torch.float64
        gen = torch.Generator().manual_seed(seed)
        im_size = shape[2:]
        grid = _cplx(gen, shape, cdtype)
        om = _traj(gen, (shape[0], len(im_size), M) if batched else (len(im_size), M), rdtype)
        kin = _cplx(gen, (shape[0], shape[1], M), cdtype)
        fwd = tkbn.KbInterp(im_size=im_size, grid_size=im_size, dtype=cdtype)
        adj = tkbn.KbInterpAdjoint(im_size=im_size, grid_size=im_size, dtype=cdtype)
        cases[name] = dict(grid=_np(grid), omega=_np(om), kdata_in=_np(kin), kdata=_np(fwd(grid, om)),
                           grid_adj=_np(adj(kin, om)))

    interp_case("interp_1d", (2, 2, 64), 100, seed=1)
    interp_case("interp_2d", (2, 3, 40, 36), 500, seed=2)
    interp_case("interp_2d_batched", (2, 2, 32, 30), 400, batched=True, seed=3)
    interp_case("interp_3d", (1, 2, 12, 14, 10), 300, seed=4)
    interp_case("interp_2d_c128", (1, 2, 24, 28), 300, cdtype=torch.complex128, seed=5)

    def nufft_case(name, B, C, im_size, M, norm, cdtype=torch.complex64, grid_size=None, seed=0, batched=False,
                   numpoints=6):
        rdtype = torch.float32 if cdtype == torch.complex64 else torch.float64
        gen = torch.Generator().manual_seed(seed)
        image = _cplx(gen, (B, 1) + im_size, cdtype)
        smaps = _cplx(gen, (B, C) + im_size, cdtype)
        om = _traj(gen, (B, len(im_size), M) if batched else (len(im_size), M), rdtype)
        kin = _cplx(gen, (B, C, M), cdtype)
        fwd = tkbn.KbNufft(im_size=im_size, grid_size=grid_size, numpoints=numpoints, dtype=cdtype)
        adj = tkbn.KbNufftAdjoint(im_size=im_size, grid_size=grid_size, numpoints=numpoints, dtype=cdtype)
        img_c = _cplx(gen, (B, C) + im_size, cdtype)
        cases[name] = dict(
            image=_np(image), smaps=_np(smaps), omega=_np(om), kdata_in=_np(kin), image_coils=_np(img_c),
            kdata_sense=_np(fwd(image, om, smaps=smaps, norm=norm)),
            image_sense=_np(adj(kin, om, smaps=smaps, norm=norm)),
            kdata_plain=_np(fwd(img_c, om, norm=norm)),
            image_plain=_np(adj(kin, om, norm=norm)),
            norm=np.array("ortho" if norm == "ortho" else ""),
            grid_size=np.array(grid_size if grid_size is not None else [2 * n for n in im_size]),
            numpoints=np.array(numpoints if isinstance(numpoints, tuple) else (numpoints,) * len(im_size)),
        )

    nufft_case("nufft_2d", 2, 4, (24, 20), 600, None, seed=10)
    nufft_case("nufft_2d_ortho", 1, 3, (32, 32), 700, "ortho", seed=11)
    nufft_case("nufft_2d_batched", 2, 2, (16, 18), 300, None, seed=12, batched=True)
    nufft_case("nufft_1d", 2, 2, (40,), 120, "ortho", seed=13)
    nufft_case("nufft_3d", 1, 3, (10, 12, 8), 400, None, seed=14)
    nufft_case("nufft_2d_grid", 1, 2, (20, 22), 300, None, grid_size=(30, 40), seed=15)
    nufft_case("nufft_2d_c128", 1, 2, (20, 22), 300, "ortho", cdtype=torch.complex128, seed=16)
    # the reference test suite's own shapes (tests/conftest.py test_params): batch 5, 4 coils,
    # 112 points, odd image sizes and per-dim numpoints
    nufft_case("nufft_refparams_2d", 5, 4, (33, 24), 112, None, seed=17, numpoints=(4, 6))
    nufft_case("nufft_refparams_3d", 5, 4, (11, 33, 24), 112, "ortho", seed=18, numpoints=(2, 4, 6))

    # Toeplitz kernel + normal operator
    for name, im_size, M, norm, batched, seed in (
        ("toep_2d", (16, 18), 800, "ortho", False, 20),
        ("toep_2d_none", (20, 16), 600, None, False, 21),
        ("toep_3d", (8, 10, 6), 500, "ortho", False, 22),
        ("toep_2d_batched", (12, 14), 400, "ortho", True, 23),
    ):
        gen = torch.Generator().manual_seed(seed)
        B, C = (2, 3)
        om = _traj(gen, (B, len(im_size), M) if batched else (len(im_size), M), torch.float32)
        w = torch.rand((B, 1, M) if batched else (1, M), generator=gen, dtype=torch.float32)
        kern = tkbn.calc_toeplitz_kernel(om, im_size, weights=w, norm=norm)
        image = _cplx(gen, (B, 1) + im_size, torch.complex64)
        smaps = _cplx(gen, (B, C) + im_size, torch.complex64)
        toep = tkbn.ToepNufft()
        cases[name] = dict(omega=_np(om), weights=_np(w), kernel=_np(kern), image=_np(image), smaps=_np(smaps),
                           out_sense=_np(toep(image, kern, smaps=smaps, norm=norm)),
                           out_plain=_np(toep(image, kern, norm=norm)),
                           norm=np.array("ortho" if norm == "ortho" else ""))

    # density compensation
    for name, im_size, shape_om, seed in (("dcomp_2d", (20, 20), (2, 400), 30), ("dcomp_2d_batched", (16, 16), (2, 2, 300), 31)):
        gen = torch.Generator().manual_seed(seed)
        om = _traj(gen, shape_om, torch.float32)
        cases[name] = dict(omega=_np(om), dcomp=_np(tkbn.calc_density_compensation_function(om, im_size)),
                           im_size=np.array(im_size))

    # sparse-matrix interpolation: the matrices (dense) and a NUFFT pair through them
    for name, im_size, M, seed in (("spmat_2d", (12, 10), 150, 40), ("spmat_3d", (6, 8, 6), 120, 41)):
        gen = torch.Generator().manual_seed(seed)
        om = _traj(gen, (len(im_size), M), torch.float32)
        real, imag = tkbn.calc_tensor_spmatrix(om, im_size)
        image = _cplx(gen, (2, 3) + im_size, torch.complex64)
        kin = _cplx(gen, (2, 3, M), torch.complex64)
        fwd = tkbn.KbNufft(im_size=im_size)
        adj = tkbn.KbNufftAdjoint(im_size=im_size)
        cases[name] = dict(omega=_np(om), mat_real=_np(real.to_dense()), mat_imag=_np(imag.to_dense()),
                           image=_np(image), kdata_in=_np(kin),
                           kdata=_np(fwd(image, om, interp_mats=(real, imag))),
                           image_adj=_np(adj(kin, om, interp_mats=(real, imag))))

    # host setup: every buffer of a complex128 KbNufft (tables, scaling
    # coefficients, parsed arguments), small table oversampling except the
    # default-argument 1D case
    for name, kw in (
        ("setup_1d_default", dict(im_size=(64,))),
        ("setup_2d", dict(im_size=(20, 24), table_oversamp=256)),
        ("setup_2d_custom", dict(im_size=(17, 12), grid_size=(30, 26), numpoints=(4, 5), table_oversamp=(128, 64),
                                 kbwidth=2.1, order=(0.0, 0.5))),
        ("setup_3d", dict(im_size=(6, 8, 5), numpoints=(2, 4, 6), table_oversamp=64)),
    ):
        mod = tkbn.KbNufft(dtype=torch.complex128, **kw)
        arrs = {k: _np(v) for k, v in mod.state_dict().items()}
        # the working-precision module's floating buffers (built in complex64, not cast)
        mod64 = tkbn.KbNufft(dtype=torch.complex64, **kw)
        arrs.update({"c64_" + k: _np(v) for k, v in mod64.state_dict().items() if v.is_complex()})
        arrs["kwargs"] = np.array(repr(kw))
        cases[name] = arrs

    # gradient of the trajectory-optimisation loss ||A^H A x - x||^2 (summed over
    # the batch) with respect to the image, through the reference's autograd
    # (its table interpolation Functions, _autograd/interp.py:78-178, and torch's
    # FFT backward); variable-density spiral k(t) = pi t^1.5 exp(i(2 pi 16 t + 2 pi j / nil))
    for name, B, C, im_size, nil, ns, seed in (("grad_x_spiral", 2, 4, (48, 48), 8, 384, 50),):
        gen = torch.Generator().manual_seed(seed)
        t = np.arange(ns) / ns
        k = np.concatenate([np.pi * t ** 1.5 * np.exp(1j * (2 * np.pi * 16 * t + 2 * np.pi * j / nil))
                            for j in range(nil)])
        om = torch.tensor(np.stack([k.imag, k.real]).astype(np.float32))
        image = _cplx(gen, (B, 1) + im_size, torch.complex64)
        smaps = _cplx(gen, (B, C) + im_size, torch.complex64) / 2
        fwd = tkbn.KbNufft(im_size=im_size)
        adj = tkbn.KbNufftAdjoint(im_size=im_size)
        x = image.clone().requires_grad_(True)
        y = adj(fwd(x, om, smaps=smaps), om, smaps=smaps)
        loss = (y - x).abs().pow(2).sum()
        loss.backward()
        cases[name] = dict(image=_np(image), smaps=_np(smaps), omega=_np(om), loss=_np(loss), grad=_np(x.grad))

    only = os.environ.get("TKBN_GOLDEN_ONLY")
    for name, arrs in cases.items():
        if only and not name.startswith(only):
            continue
        np.savez_compressed(os.path.join(HERE, f"live_{name}.npz"), **arrs)


if __name__ == "__main__":
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TKBN_REFERENCE")
    if not REF or not os.path.isdir(os.path.join(REF, "torchkbnufft")):
        sys.exit("usage: make_golden.py <reference source tree> (or set TKBN_REFERENCE)")
    sys.path.insert(0, REF)
    if not os.environ.get("TKBN_GOLDEN_ONLY"):
        convert_reference_pickles()
    live_cases()
    print("wrote fixtures to", HERE)
