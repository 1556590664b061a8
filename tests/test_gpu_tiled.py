"""The tiled step kernel (launch variant 5: bulk copies stage each 256-node
tile's sources in shared memory) computes exactly what the one-node-per-
thread kernel computes: the same populations are read and the same
arithmetic runs, so distributions and wall shear stress are bit-identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILED = 5


def _run(capi, mask, bcs, tri, Q, prec, variant, nsteps, amp, tau=0.6):
    s = capi.Solver(Q, prec, capi.LBM_PHYSICS, tau, 1.0, (0.0, 0.0, 0.0), 1.0, 1.0)
    s.set_geometry(mask, bcs)
    s.set_normals(tri)
    s.set_inlet_table(amp)
    s.set_variant(variant)
    s.step(nsteps)
    return s


@pytest.mark.parametrize("Q,prec", [(19, "f32"), (19, "f16"), (19, "bf16"), (27, "f32"), (27, "f16"), (19, "f64")])
def test_gpu_tiled_matches_flat_stenosed_tube(gpu_lib, Q, prec):
    from pv_dec_original_gb300 import geometry as G
    capi = gpu_lib
    surf = G.stenosed_tube(7.0, 60.0, 0.5, 0.2, center=(10.3, 10.1), z0=1.6, h=1.4, seed=5)
    surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (20.0, 20.0, 64.0))
    tri = surf.tri12()
    mask, _ = capi.voxelize(tri, 1.0)
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    bcs = [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, 10.3, 10.1, 7.0),
           capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)]
    amp = 0.03 * (1 + 0.5 * np.sin(2 * np.pi * np.arange(40) / 40))
    a = _run(capi, mask, bcs, tri, Q, prec, 0, 37, amp)
    b = _run(capi, mask, bcs, tri, Q, prec, TILED, 37, amp)
    assert np.array_equal(a.distributions(), b.distributions())
    wa, wb = a.wss(), b.wss()
    for k in ("acc", "acc_mag", "wss"):
        assert np.array_equal(wa[k], wb[k]), k


def test_gpu_tiled_matches_flat_bifurcation(gpu_lib):
    """The full 256x192x512 bifurcation: many tiles, segment rows beyond the
    shared-memory cap fall back to global reads; 21 steps (one stress-ring
    fold) through a captured graph."""
    from pv_dec_original_gb300 import geometry as G
    capi = gpu_lib
    surf = G.config_c2_bifurcation()
    tri = surf.tri12()
    mask, _ = capi.voxelize(tri, 1.0)
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    cx, cy = surf.meta["center"]
    bcs = [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, cx, cy, 24.0),
           capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)]
    out = []
    for v in (0, TILED):
        s = capi.Solver(19, "f32", capi.LBM_PHYSICS, 0.55, 1.0, (0.0, 0.0, 0.0), 1.0, 1.0)
        s.set_geometry(mask, bcs)
        s.set_normals(tri)
        s.set_inlet_table([0.03])
        s.set_variant(v)
        s.set_graph_steps(4)
        s.step(21)
        out.append((s.distributions(), s.wss()["acc_mag"]))
        s.close()
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0])
        assert np.array_equal(out[0][1], o[1])
