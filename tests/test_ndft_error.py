"""The table NUFFT's intrinsic error per benchmark configuration, against the
complex128 NDFT ``y_m = sum_n x[n] exp(-i omega_m . (n - N//2))``.

The NUFFT side is the oracle in complex128 (the reference's table path,
which the CUDA complex128 path matches to 1e-10). Each configuration uses
its benchmark trajectory, subsampled to 4096 seeded points, and an image
with i.i.d. N(0,1) real and imaginary parts. J = 6 at 2x oversampling has
an intrinsic error near 1e-3 relative L2, so this states the error rather
than gating parity; the assertion only catches a broken geometry.
"""

import numpy as np
import pytest

from conftest import rel_l2
from oracle import kbnufft_oracle as O


def _configs():
    import bench

    return {
        "single-coil radial 256^2 (402 x 512)": ((256, 256), bench.radial_traj(402, 512)),
        "SENSE golden-angle 320^2 (404 x 640)": ((320, 320), bench.golden_angle_traj(404, 640)),
        "kooshball 128^3 (20000 x 256)": ((128, 128, 128), bench.kooshball_traj(20000, 256)),
        "spiral 256^2 (32 x 2048)": ((256, 256), bench.spiral_traj(32, 2048)),
    }


@pytest.mark.parametrize("name", ["single-coil radial 256^2 (402 x 512)", "SENSE golden-angle 320^2 (404 x 640)",
                                  "kooshball 128^3 (20000 x 256)", "spiral 256^2 (32 x 2048)"])
def test_nufft_vs_ndft_error(name):
    im_size, traj = _configs()[name]
    rng = np.random.default_rng(2024)
    om = traj[:, rng.choice(traj.shape[1], 4096, replace=False)].astype(np.float64)
    x = rng.standard_normal(im_size) + 1j * rng.standard_normal(im_size)
    y_nufft = O.Operator(im_size, cdtype=np.complex128).forward(x[None, None], om)[0, 0]
    y_ndft = O.ndft_forward_separable(x, om)
    err = rel_l2(y_nufft, y_ndft)
    print(f"{name}: NUFFT vs NDFT relative L2 {err:.2e}")
    assert err < 3e-3, err
