"""The compact step kernel (per-warp node metadata, launch variants 6, 7)
against the flat step kernel (variant 0): the same arithmetic on the same
loads, so the distributions and the wall-shear-stress accumulators must be
bit-identical, for every storage format, both lattices, both collisions,
with velocity / pressure boundary rules and walls."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COMPACT = (6, 7)


def _tube(capi, Q, prec, variant, collision, steps=37):
    from pv_dec_original_gb300 import geometry as G
    surf = G.stenosed_tube(6.0, 60.0, 0.5, 0.25, center=(8.3, 8.1), z0=1.6, h=1.4, seed=5)
    surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (17.0, 17.0, 64.0))
    tri = surf.tri12()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    s = capi.Solver(Q, prec, capi.LBM_PHYSICS, 0.6, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0, collision=collision)
    s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, 8.3, 8.1, 6.0),
                          capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
    s.set_normals(tri)
    s.set_inlet_table(0.04 * (1 + 0.5 * np.sin(2 * np.pi * np.arange(50) / 50)))
    s.set_variant(variant)
    s.step(steps)
    return s


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("prec", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("collision", [0, 1])
def test_compact_kernel_bit_identical_to_flat(gpu_lib, Q, prec, collision):
    ref = _tube(gpu_lib, Q, prec, 0, collision)
    f0, w0 = ref.distributions(), ref.wss()
    ref.close()
    for v in COMPACT:
        s = _tube(gpu_lib, Q, prec, v, collision)
        f, w = s.distributions(), s.wss()
        s.close()
        assert np.array_equal(f, f0), f"variant {v}: max |diff| {np.abs(f - f0).max():.3g}"
        for k in ("wss", "acc", "acc_mag", "tawss"):
            assert np.array_equal(w[k], w0[k]), (v, k)


def test_compact_kernel_ragged_and_crowded_warps(gpu_lib):
    """A lattice of scattered solid points: many warps hold several pull
    segments and many wall lanes, and the active-node count is neither a
    multiple of 32 nor of the block (the last warp's metadata is zero past
    the last node)."""
    capi = gpu_lib
    rng = np.random.default_rng(11)
    mask = np.zeros((9, 7, 13), np.uint8)
    mask[1:8, 1:6, 1:12] = 1
    mask[rng.random(mask.shape) < 0.15] = 0
    if int(mask.sum()) % 32 == 0:
        mask[tuple(np.argwhere(mask > 0)[-1])] = 0
    n = int(mask.sum())
    assert n % 32 != 0 and n % 128 != 0
    out = []
    for v in (0,) + COMPACT:
        s = capi.Solver(19, "f32", capi.LBM_PHYSICS, 0.7, 1.0, (0.0, 0.0, 0.0), 1.0, 1.0)
        s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", 7, 1.002)])
        s.set_variant(v)
        s.step(15)
        out.append(s.distributions())
        s.close()
    for k in range(1, len(out)):
        assert np.array_equal(out[0], out[k]), (0, COMPACT[k - 1])
