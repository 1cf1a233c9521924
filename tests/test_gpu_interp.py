"""GPU parity of the interpolation kernels (K1 sort, K3 gather, K4 scatter).

Checked against the reference's golden vectors, live reference fixtures and
the CPU oracle. Tolerances: float64 paths at 1e-10 relative L2 (reference
tests use torch.allclose), complex64 at 1e-5 relative L2 (the parity bar).
"""

import numpy as np
import pytest
import torch

from conftest import load_golden, rel_l2
from oracle import kbnufft_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")
TOL64 = 1e-5
TOL128 = 1e-10


def tkbn():
    import torchkbnufft_gb300 as m

    return m


def _c(x):
    return x[..., 0] + 1j * x[..., 1]


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("case", [0, 1, 2])
def test_reference_interp_golden(case):
    """``tests/data/interp_data.pkl`` through KbInterp in float64, real (..., 2) layout."""
    g = load_golden("ref_interp_data")
    image, ktraj, kdata = g[f"image_{case}"], g[f"ktraj_{case}"], g[f"kdata_{case}"]
    im_size = image.shape[2:-1]
    ob = tkbn().KbInterp(im_size=im_size, grid_size=im_size, dtype=torch.float64, device=DEV)
    out = ob(torch.tensor(image, device=DEV), torch.tensor(ktraj, device=DEV))
    assert out.shape == kdata.shape
    assert torch.allclose(out.cpu(), torch.tensor(kdata))
    assert rel_l2(_np(out), kdata) < TOL128


@pytest.mark.parametrize("name", ["interp_1d", "interp_2d", "interp_2d_batched", "interp_3d", "interp_2d_c128"])
def test_live_interp_fixtures(name):
    g = load_golden("live_" + name)
    cd = torch.complex64 if g["grid"].dtype == np.complex64 else torch.complex128
    tol = TOL64 if cd == torch.complex64 else TOL128
    im_size = g["grid"].shape[2:]
    fwd = tkbn().KbInterp(im_size=im_size, grid_size=im_size, dtype=cd, device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=im_size, grid_size=im_size, dtype=cd, device=DEV)
    om = torch.tensor(g["omega"], device=DEV)
    assert rel_l2(_np(fwd(torch.tensor(g["grid"], device=DEV), om)), g["kdata"]) < tol
    assert rel_l2(_np(adj(torch.tensor(g["kdata_in"], device=DEV), om)), g["grid_adj"]) < tol


def _rand(gen, shape, cd):
    x = torch.randn(shape + (2,), generator=gen, dtype=torch.float64)
    return torch.view_as_complex(x).to(cd)


def _traj(gen, shape, scale=1.0):
    return (torch.rand(shape, generator=gen, dtype=torch.float64) * 2 - 1) * np.pi * scale


CASES = [
    # (grid_size, B, C, M, omega batched, numpoints, table_oversamp, omega scale)
    ((128, 128), 2, 5, 20000, False, 6, 1024, 1.0),
    ((96, 80), 3, 16, 7000, True, 6, 1024, 1.0),
    ((77, 93), 1, 17, 5000, False, 6, 1024, 1.0),   # odd grid, two coil chunks
    ((64, 48), 2, 3, 3000, False, (4, 6), 512, 1.0),  # per-dim numpoints, other table
    ((60, 64), 1, 1, 4000, False, 6, 1024, 3.0),  # omega outside [-pi, pi): periodic wrap
    ((200,), 2, 4, 3000, False, 6, 1024, 1.0),
    ((24, 20, 28), 1, 3, 4000, False, 6, 1024, 1.0),
    ((16, 18, 14), 2, 2, 1500, True, (4, 5, 6), 1024, 1.0),
    ((32, 24, 40), 1, 8, 30000, False, 6, 1024, 1.0),  # 3D register adjoint, 8 coils per job
    ((26, 21, 30), 2, 11, 9000, True, 6, 1024, 1.0),  # 3D, two coil chunks, edge tiles
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("cd", [torch.complex64, torch.complex128])
def test_interp_vs_oracle(case, cd):
    grid_size, B, C, M, batched, J, Lo, scale = CASES[case]
    gen = torch.Generator().manual_seed(100 + case)
    grid = _rand(gen, (B, C) + grid_size, cd)
    rd = torch.float32 if cd == torch.complex64 else torch.float64
    om = _traj(gen, (B, len(grid_size), M) if batched else (len(grid_size), M), scale).to(rd)
    kin = _rand(gen, (B, C, M), cd)
    fwd = tkbn().KbInterp(im_size=grid_size, grid_size=grid_size, numpoints=J, table_oversamp=Lo, dtype=cd,
                          device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=grid_size, grid_size=grid_size, numpoints=J, table_oversamp=Lo, dtype=cd,
                                 device=DEV)
    op = O.Operator(grid_size, grid_size, J, None, Lo, cdtype=np.complex64 if cd == torch.complex64 else np.complex128)
    tol = TOL64 if cd == torch.complex64 else TOL128
    y = fwd(grid.to(DEV), om.to(DEV))
    assert rel_l2(_np(y), op.interp(grid.numpy(), om.numpy())) < tol
    x = adj(kin.to(DEV), om.to(DEV))
    assert rel_l2(_np(x), op.interp_adj(kin.numpy(), om.numpy())) < tol


@pytest.mark.parametrize("shape, kdata_shape", [
    ([1, 1, 19], [1, 1, 25]), ([3, 1, 13], [3, 1, 18]), ([1, 1, 32, 16], [1, 1, 83]),
    ([5, 1, 15, 12], [5, 1, 83]), ([3, 2, 13, 18, 12], [3, 2, 112]), ([1, 2, 17, 19, 12], [1, 2, 112]),
])
def test_interp_adjointness(shape, kdata_shape):
    """<A x, y> == <x, A^H y> (reference tests/test_interp.py:34-70), complex128."""
    gen = torch.Generator().manual_seed(123)
    im_size = tuple(shape[2:])
    x = _rand(gen, tuple(shape), torch.complex128).to(DEV)
    y = _rand(gen, tuple(kdata_shape), torch.complex128).to(DEV)
    om = _traj(gen, (len(im_size), kdata_shape[2])).to(DEV)
    fwd = tkbn().KbInterp(im_size=im_size, grid_size=im_size, dtype=torch.complex128, device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=im_size, grid_size=im_size, dtype=torch.complex128, device=DEV)
    a = torch.vdot(y.flatten(), fwd(x, om).flatten())
    b = torch.vdot(adj(y, om).flatten(), x.flatten())
    assert torch.allclose(a, b)


def test_interp_batches_match_loop():
    """Batched omega equals a loop over batch items (reference tests/test_interp.py:283-328)."""
    gen = torch.Generator().manual_seed(5)
    im = (32, 16)
    x = _rand(gen, (4, 2) + im, torch.complex64).to(DEV)
    y = _rand(gen, (4, 2, 300), torch.complex64).to(DEV)
    om = _traj(gen, (4, 2, 300)).float().to(DEV)
    fwd = tkbn().KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    loop = torch.cat([fwd(x[i:i + 1], om[i]) for i in range(4)])
    assert torch.allclose(loop, fwd(x, om), rtol=1e-6, atol=1e-5)
    loop = torch.cat([adj(y[i:i + 1], om[i]) for i in range(4)])
    assert torch.allclose(loop, adj(y, om), rtol=1e-6, atol=1e-4)


def test_complex_real_layouts_match():
    gen = torch.Generator().manual_seed(9)
    im = (20, 22)
    x = _rand(gen, (2, 3) + im, torch.complex64).to(DEV)
    om = _traj(gen, (2, 200)).float().to(DEV)
    fwd = tkbn().KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    a = fwd(x, om)
    b = torch.view_as_complex(fwd(torch.view_as_real(x), om))
    assert torch.equal(a, b)


def test_edge_cases():
    """Single point, points on the grid boundary (+-pi), one coil, empty trajectory."""
    im = (16, 16)
    fwd = tkbn().KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    op = O.Operator(im, im, cdtype=np.complex64)
    gen = torch.Generator().manual_seed(3)
    x = _rand(gen, (1, 1) + im, torch.complex64)
    for om in (torch.tensor([[0.3], [-1.2]]), torch.tensor([[np.pi, -np.pi, 0.0], [-np.pi, np.pi, np.pi]])):
        om = om.float()
        y = fwd(x.to(DEV), om.to(DEV))
        assert rel_l2(_np(y), op.interp(x.numpy(), om.numpy())) < TOL64
        k = _rand(gen, (1, 1, om.shape[1]), torch.complex64)
        assert rel_l2(_np(adj(k.to(DEV), om.to(DEV))), op.interp_adj(k.numpy(), om.numpy())) < TOL64
    empty = torch.zeros((2, 0), device=DEV)
    assert fwd(x.to(DEV), empty).shape == (1, 1, 0)
    g = adj(torch.zeros((1, 1, 0), dtype=torch.complex64, device=DEV), empty)
    assert g.shape == (1, 1) + im and torch.count_nonzero(g) == 0


def test_nonfinite_omega_is_flagged():
    """A NaN coordinate gives NaN at that point, the others stay exact, and the status word is set."""
    from torchkbnufft_gb300 import _runtime

    im = (16, 16)
    fwd = tkbn().KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    gen = torch.Generator().manual_seed(4)
    x = _rand(gen, (1, 1) + im, torch.complex64)
    om = _traj(gen, (2, 50)).float()
    om[0, 7] = float("nan")
    _runtime.device_status(DEV)  # clear
    y = _np(fwd(x.to(DEV), om.to(DEV)))
    assert np.isnan(y[0, 0, 7])
    keep = np.ones(50, bool)
    keep[7] = False
    op = O.Operator(im, im, cdtype=np.complex64)
    ref = op.interp(x.numpy(), om.numpy()[:, keep])
    assert rel_l2(y[..., keep], ref) < TOL64
    assert _runtime.device_status(DEV) & 1
    assert _runtime.device_status(DEV) == 0


def test_repeated_calls_reuse_layout():
    from torchkbnufft_gb300 import _runtime

    im = (32, 32)
    fwd = tkbn().KbInterp(im_size=im, grid_size=im, dtype=torch.complex64, device=DEV)
    gen = torch.Generator().manual_seed(6)
    x = _rand(gen, (1, 2) + im, torch.complex64).to(DEV)
    om = _traj(gen, (2, 500)).float().to(DEV)
    a = fwd(x, om)
    n = len(_runtime._layout_cache)
    b = fwd(x, om)
    assert len(_runtime._layout_cache) == n and torch.equal(a, b)
    om.mul_(0.5)  # in-place change must invalidate the cached layout
    c = fwd(x, om)
    op = O.Operator(im, im, cdtype=np.complex64)
    assert rel_l2(_np(c), op.interp(_np(x), _np(om))) < TOL64


@pytest.mark.parametrize("C", [16, 5, 3, 1])
def test_adjoint_owned_tiles_deterministic(C):
    """Grids with K >= T + J - 1 use the owned-tile adjoint; tiles that are not split
    over several sub-jobs are accumulated without atomics (with fewer than 16 coils,
    warp groups' partial tiles are summed in a fixed order), so the result is bitwise
    repeatable."""
    gen = torch.Generator().manual_seed(21)
    K = (160, 144)
    y = _rand(gen, (2, C, 30000), torch.complex64)
    om = _traj(gen, (2, 30000)).float()
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    a = adj(y.to(DEV), om.to(DEV))
    b = adj(y.to(DEV), om.to(DEV))
    assert torch.equal(a, b)
    op = O.Operator(K, K, cdtype=np.complex64)
    assert rel_l2(_np(a), op.interp_adj(y.numpy(), om.numpy())) < TOL64


@pytest.mark.parametrize("batched", [False, True])
def test_adjoint_split_heavy_tiles_match_oracle(batched):
    """Points clustered at the k-space centre make tiles heavy enough to be split
    over several sub-jobs (accumulated into pre-zeroed tiles)."""
    gen = torch.Generator().manual_seed(22)
    K = (160, 144)
    B, C, M = 2, 16, 30000
    y = _rand(gen, (B, C, M), torch.complex64)
    om = _traj(gen, (B, 2, M) if batched else (2, M)).float()
    om[..., :8000] *= 0.03
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    fwd = tkbn().KbInterp(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    op = O.Operator(K, K, cdtype=np.complex64)
    assert rel_l2(_np(adj(y.to(DEV), om.to(DEV))), op.interp_adj(y.numpy(), om.numpy())) < TOL64
    g = _rand(gen, (B, C) + K, torch.complex64)
    assert rel_l2(_np(fwd(g.to(DEV), om.to(DEV))), op.interp(g.numpy(), om.numpy())) < TOL64


def test_adjoint_deterministic_layout_is_bitwise_repeatable():
    """With torch's deterministic-algorithms setting (or deterministic=True), the layout
    has no split output tiles, so even k-space-centre-heavy trajectories give bitwise
    repeatable adjoints."""
    from torchkbnufft_gb300 import _runtime

    gen = torch.Generator().manual_seed(23)
    K = (160, 144)
    y = _rand(gen, (2, 16, 30000), torch.complex64).to(DEV)
    om = _traj(gen, (2, 30000)).float()
    om[..., :8000] *= 0.03
    om = om.to(DEV)
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    torch.use_deterministic_algorithms(True)
    try:
        a = adj(y, om)
        b = adj(y, om)
    finally:
        torch.use_deterministic_algorithms(False)
    assert torch.equal(a, b)
    op = O.Operator(K, K, cdtype=np.complex64)
    assert rel_l2(_np(a), op.interp_adj(_np(y), _np(om))) < TOL64
    lay = _runtime.points_layout(_runtime.make_geom(torch.complex64, K, K, (6, 6), (1024, 1024), (0.0, 0.0)), om,
                                 deterministic=True)
    assert lay.flags == 2


@pytest.mark.parametrize("C", [8, 3, 1])
def test_adjoint_3d_owned_tiles_deterministic(C):
    """3D owned tiles (4 x 8 x 8, register accumulators): bitwise repeatable, and
    equal to the oracle, with points concentrated at the k-space centre."""
    gen = torch.Generator().manual_seed(31)
    K = (40, 32, 48)
    M = 20000
    y = _rand(gen, (1, C, M), torch.complex64)
    om = _traj(gen, (3, M)).float()
    om[..., :5000] *= 0.1
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    torch.use_deterministic_algorithms(True)
    try:
        a = adj(y.to(DEV), om.to(DEV))
        b = adj(y.to(DEV), om.to(DEV))
    finally:
        torch.use_deterministic_algorithms(False)
    assert torch.equal(a, b)
    op = O.Operator(K, K, cdtype=np.complex64)
    assert rel_l2(_np(a), op.interp_adj(y.numpy(), om.numpy())) < TOL64
    c = adj(y.to(DEV), om.to(DEV))  # split heavy tiles (default layout)
    assert rel_l2(_np(c), op.interp_adj(y.numpy(), om.numpy())) < TOL64


def _kernels_launched(fn, tmp_path):
    """Names of the CUDA kernels that fn launches (the profiler's kernel trace)."""
    import json

    from torch.profiler import ProfilerActivity, profile

    torch.cuda.synchronize()
    # the process's first profiling session can miss kernel records while the
    # activity tracer starts up: run one throwaway session first
    with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]):
        torch.ones(8, device=DEV).sum()
        torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]) as prof:
        fn()
        torch.cuda.synchronize()
    path = tmp_path / "trace.json"
    prof.export_chrome_trace(str(path))
    events = json.loads(path.read_text()).get("traceEvents", [])
    return {e.get("name", "") for e in events if e.get("cat") == "kernel"}


@pytest.mark.parametrize("case", ["2d16", "2d4", "3d8"])
def test_specialised_kernels_are_selected(case, tmp_path):
    """The benchmark shapes run the register-accumulator adjoint and the coil-pair
    gather (a layout or eligibility regression would silently fall back to the
    generic kernels, which are also correct)."""
    from torchkbnufft_gb300 import _runtime as R

    gen = torch.Generator().manual_seed(31)
    if case == "3d8":
        im, C = (16, 16, 16), 8
    else:
        im, C = (40, 40), 16 if case == "2d16" else 4
    gs = tuple(2 * n for n in im)
    M = 3000
    om = ((torch.rand((len(im), M), generator=gen, dtype=torch.float64) * 2 - 1) * np.pi).float().to(DEV)
    mod = tkbn().KbNufft(im_size=im, device=DEV)
    geom = mod._geom(torch.complex64)
    tables = mod._tables()
    lay = R.points_layout(geom, om)
    grid = torch.randn((1, C) + gs, dtype=torch.complex64, generator=torch.Generator().manual_seed(3)).to(DEV)
    kdata = R.interp_fwd(geom, lay, tables, grid)
    names = _kernels_launched(lambda: R.interp_adj(geom, lay, tables, kdata), tmp_path)
    want = "k_interp_adj_reg3" if case == "3d8" else "k_interp_adj_reg<"
    assert any(want in n for n in names), names
    # the linear-phase gathers
    names = _kernels_launched(lambda: R.interp_fwd(geom, lay, tables, grid), tmp_path)
    if case != "3d8":
        assert any("k_interp_fwd_pairs<" in n and "true>" in n for n in names), names
    else:
        assert any("k_interp_fwd_lp3<" in n for n in names), names


def _bins_mismatched(om, op, K):
    """Per dim, the points whose table bins do not step by exactly L from tap to
    tap (the reference's fl(tm - g) rounds), in the oracle's arithmetic."""
    rdt = np.float32
    tm = O.normalized_freq(om, K, rdt)
    base = O.point_indices(tm, op.numpoints, rdt)
    out = []
    for d in range(len(K)):
        L, J = op.table_oversamp[d], op.numpoints[d]
        bins = np.stack([np.rint((tm[d] - (base[d] + j).astype(rdt)) * rdt(L)) for j in range(J)]).astype(np.int64)
        out.append(np.any(bins != bins[0] - np.arange(J)[:, None] * L, axis=0))
    return out


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("subset", ["centre_heavy", "left_out_only"])
def test_linear_phase_adjoint_exact_pass(ndim, subset, tmp_path):
    """Points within a few cells of tm = 0 (the k-space centre) can have table
    bins that do not step by exactly L (the reference's fl(tm - g) rounds);
    the linear-phase register adjoint leaves them to an exact atomic pass.
    Cases: 3/4 of the points near the centre, and only the left-out points
    (with a mismatch in every dimension among them)."""
    from torchkbnufft_gb300 import _runtime as R

    gen = torch.Generator().manual_seed(41)
    K, C, M = ((160, 144), 16, 30000) if ndim == 2 else ((40, 32, 48), 8, 20000)
    y = _rand(gen, (1, C, M), torch.complex64)
    om = _traj(gen, (ndim, M)).float()
    om[..., : 3 * M // 4] *= 0.01
    op = O.Operator(K, K, cdtype=np.complex64)
    if subset == "left_out_only":
        per_dim = _bins_mismatched(om.numpy(), op, K)
        assert all(m.any() for m in per_dim), [int(m.sum()) for m in per_dim]
        keep = torch.tensor(np.any(per_dim, axis=0))
        y, om = y[..., keep].contiguous(), om[:, keep].contiguous()
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    assert R.table_ptrs(adj._tables(), torch.complex64)[2] & 8  # linear-phase tables
    names = _kernels_launched(lambda: adj(y.to(DEV), om.to(DEV)), tmp_path)
    assert any("k_adj_lp_fix" in n for n in names), names
    assert rel_l2(_np(adj(y.to(DEV), om.to(DEV))), op.interp_adj(y.numpy(), om.numpy())) < TOL64


@pytest.mark.parametrize("ndim", [2, 3])
def test_adjoint_factor_reuse_follows_the_tables(ndim, tmp_path):
    """The register adjoints keep their per-point table factors in the layout's
    workspace between calls (they depend on the trajectory and the tables
    only). The same tables again skip the pre-pass; another table set on the
    same layout (same geometry, other kbwidth) or a table changed in place
    recomputes it. Every result matches the oracle for its own tables."""
    gen = torch.Generator().manual_seed(47)
    K, C, M = ((96, 84), 4, 6000) if ndim == 2 else ((40, 32, 48), 4, 6000)
    y = _rand(gen, (1, C, M), torch.complex64)
    om = _traj(gen, (ndim, M)).float()
    a1 = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, device=DEV)
    a2 = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, kbwidth=2.0, device=DEV)
    o1 = O.Operator(K, K, cdtype=np.complex64)
    ref1 = o1.interp_adj(y.numpy(), om.numpy())
    ref2 = O.Operator(K, K, kbwidth=2.0, cdtype=np.complex64).interp_adj(y.numpy(), om.numpy())
    ref1b = O.interp_adjoint(y.numpy(), om.numpy(), [o1.tables[0] * 2] + list(o1.tables[1:]), o1.n_shift,
                             o1.numpoints, o1.table_oversamp, K)
    yd, omd = y.to(DEV), om.to(DEV)

    def run(mod):
        return _np(mod(yd, omd))

    def prepass_launched(mod):
        names = _kernels_launched(lambda: mod(yd, omd), tmp_path)
        assert any(("k_interp_adj_reg<" if ndim == 2 else "k_interp_adj_reg3<") in n for n in names), names
        return any(("k_point_factors2" if ndim == 2 else "k_point_factors3") in n for n in names)

    assert rel_l2(run(a1), ref1) < TOL64
    assert not prepass_launched(a1)
    assert rel_l2(run(a1), ref1) < TOL64
    assert prepass_launched(a2)
    assert rel_l2(run(a2), ref2) < TOL64
    assert prepass_launched(a1)
    assert rel_l2(run(a1), ref1) < TOL64
    with torch.no_grad():
        a1.table_0.mul_(2)
    assert prepass_launched(a1)
    assert rel_l2(run(a1), ref1b) < TOL64


@pytest.mark.parametrize("case", ["2d16", "2d4", "3d8", "3d3"])
@pytest.mark.parametrize("subset", ["centre_heavy", "left_out_only"])
def test_linear_phase_gather_exact_pass(case, subset, tmp_path):
    """The linear-phase gathers (2D coil pairs, 3D one lane per coil) work with
    real kernel values on a patch multiplied by the E tables; points whose
    table bins do not step by exactly L get their exact values from a second
    pass (k_fwd_lp_fix, k_fwd_lp_fix3). Cases: 3/4 of the points near the
    k-space centre, and only the left-out points (with a mismatch in every
    dimension among them)."""
    ndim, C = (2 if case.startswith("2d") else 3), int(case[2:])
    gen = torch.Generator().manual_seed(43)
    K, M = ((160, 144), 30000) if ndim == 2 else ((40, 32, 48), 20000)
    if ndim == 2:
        grid = _rand(gen, (2, C) + K, torch.complex64)
        om = _traj(gen, (ndim, M)).float()
    else:  # the trajectory first, so that it does not depend on the coil count
        om = _traj(gen, (ndim, M)).float()
        grid = _rand(gen, (2, C) + K, torch.complex64)
    om[..., : 3 * M // 4] *= 0.01
    op = O.Operator(K, K, cdtype=np.complex64)
    if subset == "left_out_only":
        per_dim = _bins_mismatched(om.numpy(), op, K)
        assert all(m.any() for m in per_dim), [int(m.sum()) for m in per_dim]
        om = om[:, torch.tensor(np.any(per_dim, axis=0))].contiguous()
    fwd = tkbn().KbInterp(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    gd, omd = grid.to(DEV), om.to(DEV)
    names = _kernels_launched(lambda: fwd(gd, omd), tmp_path)
    if ndim == 2:
        assert any("k_fwd_lp_fix" in n for n in names), names
        assert any("k_interp_fwd_pairs<" in n and "true>" in n for n in names), names
    else:
        assert any("k_fwd_lp_fix3" in n for n in names), names
        assert any("k_interp_fwd_lp3<" in n for n in names), names
    assert rel_l2(_np(fwd(gd, omd)), op.interp(grid.numpy(), om.numpy())) < TOL64


def test_factor_reuse_between_forward_and_adjoint(tmp_path):
    """Forward and adjoint calls on one layout share its per-point factor
    scratch: whichever runs first fills it, the other reuses it for the same
    tables, and another table set (or a table changed in place) recomputes it.
    Every result matches the oracle for its own tables."""
    from torchkbnufft_gb300 import _runtime as R

    gen = torch.Generator().manual_seed(53)
    K, C, M = (96, 84), 4, 6000
    grid = _rand(gen, (1, C) + K, torch.complex64)
    y = _rand(gen, (1, C, M), torch.complex64)
    om = _traj(gen, (2, M)).float()
    f1 = tkbn().KbInterp(im_size=K, grid_size=K, device=DEV)
    a1 = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, device=DEV)
    f2 = tkbn().KbInterp(im_size=K, grid_size=K, kbwidth=2.0, device=DEV)
    o1 = O.Operator(K, K, cdtype=np.complex64)
    o2 = O.Operator(K, K, kbwidth=2.0, cdtype=np.complex64)
    gd, yd, omd = grid.to(DEV), y.to(DEV), om.to(DEV)
    R._layout_cache.clear()

    def prepass(fn):
        names = _kernels_launched(fn, tmp_path)
        return any("k_point_factors2" in n for n in names)

    assert prepass(lambda: f1(gd, omd))  # a new layout: the forward fills the scratch
    assert rel_l2(_np(f1(gd, omd)), o1.interp(grid.numpy(), om.numpy())) < TOL64
    assert not prepass(lambda: a1(yd, omd))  # the adjoint reuses the forward's factors
    assert rel_l2(_np(a1(yd, omd)), o1.interp_adj(y.numpy(), om.numpy())) < TOL64
    assert prepass(lambda: f2(gd, omd))  # other tables on the same layout
    assert rel_l2(_np(f2(gd, omd)), o2.interp(grid.numpy(), om.numpy())) < TOL64
    assert prepass(lambda: a1(yd, omd))
    assert not prepass(lambda: f1(gd, omd))
    assert rel_l2(_np(f1(gd, omd)), o1.interp(grid.numpy(), om.numpy())) < TOL64
    with torch.no_grad():
        f1.table_0.mul_(2)
    assert prepass(lambda: f1(gd, omd))
    want = O.interp_forward(grid.numpy(), om.numpy(), [o1.tables[0] * 2, o1.tables[1]], o1.n_shift, o1.numpoints,
                            o1.table_oversamp)
    assert rel_l2(_np(f1(gd, omd)), want) < TOL64


def test_linear_phase_factors_beyond_one_pass_of_the_prepass_grid():
    """The per-point factor pre-pass runs a grid-stride loop; with more points
    than its grid has threads (152 * 16 blocks of 256), threads take several
    points, some of them left out (near the k-space centre). Forward and
    adjoint against the oracle at 700k points."""
    gen = torch.Generator().manual_seed(59)
    K, C, M = (160, 144), 2, 700_000
    grid = _rand(gen, (1, C) + K, torch.complex64)
    y = _rand(gen, (1, C, M), torch.complex64)
    om = _traj(gen, (2, M)).float()
    om[..., ::4] *= 0.01  # every fourth point near the centre, spread over the sorted order
    op = O.Operator(K, K, cdtype=np.complex64)
    fwd = tkbn().KbInterp(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    adj = tkbn().KbInterpAdjoint(im_size=K, grid_size=K, dtype=torch.complex64, device=DEV)
    omd = om.to(DEV)
    assert rel_l2(_np(fwd(grid.to(DEV), omd)), op.interp(grid.numpy(), om.numpy())) < TOL64
    assert rel_l2(_np(adj(y.to(DEV), omd)), op.interp_adj(y.numpy(), om.numpy())) < TOL64
