"""Host restatements of the learned warm start's data kernels (no GPU): the
slice-wise Poiseuille prior the network corrects and the masked smoothing
of predictions.  They are the checkers of lbm_ws_prior / lbm_ws_smooth
(tests/test_gpu_nn.py); here their own properties are pinned."""
import numpy as np

from helpers import poiseuille_prior, slice_distance, smooth_masked


def _tube(D=48, H=24, W=24, R=8.3, cx=11.6, cy=11.4):
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    m = ((x - cx) ** 2 + (y - cy) ** 2 < R ** 2).astype(np.uint8)
    m[0] = 0  # caps
    m[-1] = 0
    return m


def test_slice_distance_of_a_square_duct():
    m = np.zeros((3, 9, 9), np.uint8)
    m[:, 2:7, 2:7] = 1  # 5 x 5 fluid square
    d = slice_distance(m)
    assert d[1, 2, 2] == 0.5 and d[1, 2, 4] == 0.5
    assert d[1, 3, 3] == 1.5 and d[1, 4, 4] == 2.5
    assert np.all(d[m == 0] == 0.0)


def test_poiseuille_prior_flux_and_gradient():
    mask = _tube()
    U, tau = 0.02, 0.8
    drho, uz = poiseuille_prior(mask, U, tau)
    fl = mask > 0
    flux = [uz[z][fl[z]].sum() for z in range(1, mask.shape[0] - 1)]
    # the same profile on every section of a straight tube
    assert np.std(flux) < 1e-9 * np.mean(flux) + 1e-12
    inlet = uz[1][fl[1]]
    assert abs(inlet.max() / U - 1.0) < 0.15
    # density falls linearly along z to 1 on the last fluid slice
    means = np.array([drho[z][fl[z]].mean() for z in range(1, mask.shape[0] - 1)])
    assert abs(means[-1]) < 1e-15
    d = np.diff(means)
    assert np.all(d < 0) and np.std(d) < 1e-9 * abs(d.mean())


def test_smoothing_kills_checkerboard_keeps_linear():
    mask = np.ones((12, 10, 8), np.uint8)
    z, y, x = np.meshgrid(*[np.arange(n) for n in mask.shape], indexing="ij")
    lin = 0.3 * z + 0.1 * y - 0.2 * x
    chk = (-1.0) ** (x + y + z)
    out = smooth_masked(mask, lin + 0.05 * chk, rounds=1)
    inner = (slice(1, -1),) * 3
    assert np.max(np.abs(out[inner] - lin[inner])) < 1e-12
    # restricted to the fluid: solid voxels stay zero, a constant stays constant
    mask[:, :, :3] = 0
    c = smooth_masked(mask, np.full(mask.shape, 2.0), rounds=2)
    assert np.all(c[mask == 0] == 0.0) and np.allclose(c[mask > 0], 2.0)
