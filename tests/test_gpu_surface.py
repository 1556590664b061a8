"""Surface read-out: WSS, OSI and TAWSS at STL vertices from the nearest
next-to-wall node (the reference's commented-out FindClosestLatticePoint /
InterpolateAttributesToSTLVertices, OutputFile.cpp:431-488).  The device's
expanding-cube search must return exactly the brute-force nearest node."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tube(capi):
    from pv_dec_original_gb300 import geometry as G
    surf = G.stenosed_tube(6.0, 40.0, 0.5, 0.2, center=(9.3, 9.1), z0=1.6, h=1.2, seed=3)
    surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (18.0, 18.0, 44.0))
    tri = surf.tri12()
    mask, vd = capi.voxelize(tri, 1.0)
    bb = np.array(vd.bbox[:])
    origin = (bb[0], bb[2], bb[4])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    s = capi.Solver(19, "f32", capi.LBM_PHYSICS, 0.6, 1.0, origin, 1.0, 1.0)
    s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, 9.3, 9.1, 6.0),
                          capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
    s.set_normals(tri)
    s.set_inlet_table([0.02])
    return s, tri, mask, np.array(origin)


def _brute(s, mask, origin, xyz):
    nz, ny, nx = mask.shape
    pt = s.wss()["pt"]
    ijk = np.stack([pt % nx, (pt // nx) % ny, pt // (nx * ny)], 1).astype(np.float64)
    g = (xyz - origin) / 1.0
    d2 = ((ijk[None, :, :] - g[:, None, :]) ** 2).sum(-1)
    idx = np.argmin(d2, 1)  # first (lowest index) minimum
    return idx, np.sqrt(d2[np.arange(len(g)), idx])


def test_gpu_nearest_next_to_wall_matches_brute_force(gpu_lib):
    s, tri, mask, origin = _tube(gpu_lib)
    s.step(50)
    xyz = np.unique(tri[:, :9].reshape(-1, 3), axis=0)
    rng = np.random.default_rng(0)
    xyz = np.concatenate([xyz, xyz[:200] + rng.normal(0.0, 0.7, (200, 3))])
    idx, dist = s.nearest_next_to_wall(xyz)
    ref, rd = _brute(s, mask, origin, xyz)
    assert np.array_equal(idx, ref)
    np.testing.assert_allclose(dist, rd, rtol=1e-12, atol=1e-12)
    a = s.wss_at_points(xyz)
    w = s.wss()
    for k in ("wss", "osi", "tawss"):
        np.testing.assert_array_equal(a[k], w[k][ref])
    assert np.all(np.isfinite(a["tawss"])) and np.all(a["tawss"] > 0)


def test_gpu_nearest_next_to_wall_out_of_reach(gpu_lib):
    s, tri, mask, origin = _tube(gpu_lib)
    far = origin[None, :] + np.array([[-40.0, -40.0, -40.0]])
    idx, dist = s.nearest_next_to_wall(far, max_radius=2)
    assert idx[0] == -1 and dist[0] == -1.0
    idx, _ = s.nearest_next_to_wall(far, max_radius=128)
    ref, _ = _brute(s, mask, origin, far)
    assert idx[0] == ref[0]
    with pytest.raises(gpu_lib.LbmError):
        s.nearest_next_to_wall(far, max_radius=0)
