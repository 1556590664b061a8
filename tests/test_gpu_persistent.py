"""Persistent stepping (lbm_set_persistent): one cooperative launch runs
several steps with a bounded grid barrier between them.  Every format, both
modes, D3Q27, interpolated walls, graph replay and a packed ensemble of
uneven vessels must give bit-identical distributions and wall-shear outputs
to one launch per step; a barrier that never completes must end the launch
with an error status and leave the handle usable after re-initialisation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 53  # crosses the stress-ring folds at steps 16, 32, 48 and leaves a remainder


def _tube(capi, Q=19, prec=None, mode=None, tau=0.7, walls=False):
    from pv_dec_original_gb300 import geometry as G, waveform
    prec = capi.LBM_F32 if prec is None else prec
    mode = capi.LBM_PHYSICS if mode is None else mode
    surf = G.stenosed_tube(5.0, 30.0, 0.5, 0.2, center=(7.3, 7.1), z0=1.6, h=1.4, seed=3)
    surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (14.0, 14.0, 34.0))
    tri = surf.tri12()
    mask, vd = capi.voxelize(tri, 1.0)
    bb = np.array(vd.bbox[:])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    s = capi.Solver(Q, prec, mode, tau, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0)
    s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, 7.3, 7.1, 5.0),
                          capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
    s.set_normals(tri)
    if walls:
        s.set_wall_distances(tri)
    s.set_inlet_table(waveform.sinusoid_table(0.03, 40.0))
    return s


def _same(a, b):
    fa, fb = a.distributions(), b.distributions()
    assert np.array_equal(fa, fb), f"distributions differ (max {np.abs(fa - fb).max():.3g})"
    wa, wb = a.wss(), b.wss()
    for k in wa:
        assert np.array_equal(np.asarray(wa[k]), np.asarray(wb[k]), equal_nan=True), k


@pytest.mark.parametrize("prec", ["f32", "f16", "bf16", "f64"])
@pytest.mark.parametrize("graph", [0, 16])
def test_gpu_persistent_matches_flat(gpu_lib, prec, graph):
    capi = gpu_lib
    P = {"f32": capi.LBM_F32, "f16": capi.LBM_F16, "bf16": capi.LBM_BF16, "f64": capi.LBM_F64}[prec]
    flat, pers = _tube(capi, prec=P), _tube(capi, prec=P)
    pers.set_persistent(4)
    if graph:
        flat.set_graph_steps(graph)
        pers.set_graph_steps(graph)
    n0 = pers.launches()
    flat.step(STEPS)
    pers.step(STEPS)
    if not graph:
        assert pers.launches() - n0 == STEPS // 4 + STEPS % 4
    _same(flat, pers)


@pytest.mark.parametrize("case", ["q27", "walls", "parity"])
def test_gpu_persistent_variants(gpu_lib, case):
    capi = gpu_lib
    kw = {"q27": dict(Q=27), "walls": dict(walls=True),
          "parity": dict(prec=capi.LBM_F64, mode=capi.LBM_PARITY)}[case]
    flat, pers = _tube(capi, **kw), _tube(capi, **kw)
    pers.set_persistent(16)
    flat.step(STEPS)
    pers.step(STEPS)
    _same(flat, pers)


def test_gpu_persistent_ensemble(gpu_lib):
    from pv_dec_original_gb300 import geometry as G
    from pv_dec_original_gb300.ensemble import Ensemble
    members = []
    for m, (r, length, mean, period) in enumerate([(5.0, 40.0, 0.03, 400.0), (7.0, 56.0, 0.02, 700.0),
                                                    (4.2, 33.0, 0.04, 300.0)]):
        nxy, nz = int(np.ceil(2 * r + 6)), int(np.ceil(length + 6))
        cx, cy = 0.5 * (nxy - 1) + 0.173, 0.5 * (nxy - 1) + 0.061
        s = G.stenosed_tube(r, length, 0.4, 0.1, center=(cx, cy), z0=2.7, seed=200 + m, h=1.4)
        meta = dict(s.meta)
        s = G.add_bbox_anchors(s, (0.0, 0.0, 0.0), (nxy - 1.0, nxy - 1.0, float(nz)))
        s.meta = meta
        members.append({"surface": s, "radius": r, "center": (cx, cy), "inlet_mean": mean, "period": period})
    flat = Ensemble(members, 19, "f16", 0.6)
    pers = Ensemble(members, 19, "f16", 0.6)
    pers.solver.set_persistent(8)
    pers.solver.set_graph_steps(32)
    flat.step(77)
    pers.step(77)
    _same(flat.solver, pers.solver)


def test_gpu_persistent_arguments(gpu_lib):
    capi = gpu_lib
    s = _tube(capi)
    for bad in (-2, 1, 3):
        with pytest.raises(capi.LbmError):
            s.set_persistent(bad)
    s.set_persistent(4)
    with pytest.raises(capi.LbmError):
        s.set_graph_steps(6)  # not a multiple of 4
    s.set_graph_steps(8)
    with pytest.raises(capi.LbmError):
        s.set_persistent(6)  # 8 is not a multiple of 6
    s.set_persistent(0)
    s.step(3)


def test_gpu_persistent_barrier_timeout(gpu_lib):
    """A barrier that waits for more arrivals than there are blocks: every
    block's bounded wait gives up, the status reports it, and the handle
    steps correctly again after re-initialisation."""
    capi = gpu_lib
    s = _tube(capi)
    s.set_persistent(4)
    s.preset_barrier(0x40000000)
    with pytest.raises(capi.LbmError, match="bounded wait"):
        s.step(4)
    s.init_equilibrium()
    s.step(STEPS)
    ref = _tube(capi)
    ref.step(STEPS)
    _same(ref, s)
