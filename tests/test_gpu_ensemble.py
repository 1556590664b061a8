"""Packed ensemble: several stenosed tubes of different sizes and inlet
waveforms advanced as one lattice must reproduce, member by member, the
same tubes run as separate lattices (no link joins two members; every
member keeps its own inlet/outlet planes, profile, waveform and normals)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members():
    from pv_dec_original_gb300 import geometry as G
    out = []
    specs = [(5.0, 40.0, 0.5, 0.2, 0.03, 400.0), (7.0, 56.0, 0.3, 0.0, 0.02, 700.0), (4.2, 33.0, 0.6, 0.3, 0.04, 300.0)]
    for m, (r, length, sev, ecc, mean, period) in enumerate(specs):
        nxy = int(np.ceil(2 * r + 6))
        nz = int(np.ceil(length + 6))
        cx, cy = 0.5 * (nxy - 1) + 0.173, 0.5 * (nxy - 1) + 0.061
        s = G.stenosed_tube(r, length, sev, ecc, center=(cx, cy), z0=2.7, seed=100 + m, h=1.4)
        meta = dict(s.meta)
        s = G.add_bbox_anchors(s, (0.0, 0.0, 0.0), (nxy - 1.0, nxy - 1.0, float(nz)))
        s.meta = meta
        out.append({"surface": s, "radius": r, "center": (cx, cy), "inlet_mean": mean, "period": period})
    return out


def _single(capi, m, prec, tau):
    from pv_dec_original_gb300 import waveform
    tri = m["surface"].tri12()
    mask, vd = capi.voxelize(tri, 1.0)
    bb = np.array(vd.bbox[:])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    s = capi.Solver(19, prec, capi.LBM_PHYSICS, tau, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0)
    s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, m["center"][0], m["center"][1],
                                       m["radius"]),
                          capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
    s.set_normals(tri)
    s.set_inlet_table(waveform.sinusoid_table(m["inlet_mean"], m["period"]))
    return s


@pytest.mark.parametrize("prec", ["f32", "f16"])
def test_gpu_ensemble_matches_separate_lattices(gpu_lib, prec):
    from pv_dec_original_gb300.ensemble import Ensemble
    members = _members()
    tau = 0.6
    ens = Ensemble(members, 19, prec, tau)
    singles = [_single(gpu_lib, m, prec, tau) for m in members]
    cnt = ens.counts
    assert cnt["active"] == sum(s.counts()["active"] for s in singles)
    assert cnt["next_to_wall"] == sum(s.counts()["next_to_wall"] for s in singles)
    for b, s in enumerate(singles):  # inlet and outlet node counts per member
        assert cnt["bc"][2 * b] == s.counts()["bc"][0]
        assert cnt["bc"][2 * b + 1] == s.counts()["bc"][1]
    ens.step(37)
    for s in singles:
        s.step(37)
    rho, u, mem = ens.macro()
    w = ens.wss()
    for m, s in enumerate(singles):
        r1, u1 = s.macro()
        np.testing.assert_allclose(rho[mem == m], r1, rtol=0, atol=1e-6)
        np.testing.assert_allclose(u[mem == m], u1, rtol=0, atol=1e-6)
        w1 = s.wss()
        sel = w["member"] == m
        np.testing.assert_allclose(w["normal"][sel], w1["normal"], atol=1e-12)
        err = np.linalg.norm(w["tawss"][sel] - w1["tawss"]) / np.linalg.norm(w1["tawss"])
        assert err < 1e-5, err
    # flux: each member's inlet and outlet carry that member's own flux
    _, _, fl = ens.solver.conservation()
    for m, s in enumerate(singles):
        _, _, f1 = s.conservation()
        np.testing.assert_allclose(fl[2 * m:2 * m + 2], f1, rtol=1e-5, atol=1e-9)


def test_gpu_grouped_ensemble_matches_one_packed_lattice(gpu_lib):
    """The members packed into two lattices advanced concurrently on their own
    streams give every member what one packed lattice gives it."""
    from pv_dec_original_gb300.ensemble import Ensemble, GroupedEnsemble
    members = _members()
    tau = 0.6
    one = Ensemble(members, 19, "f16", tau)
    grp = GroupedEnsemble(members, 2, 19, "f16", tau)
    assert len(grp.groups) == 2 and grp.active == one.active
    grp.set_graph_steps(8)
    one.step(37)
    grp.step(37)
    rho, u, mem = one.macro()
    rho2, u2, mem2 = grp.macro()
    assert np.array_equal(mem, mem2)
    np.testing.assert_allclose(rho2, rho, rtol=0, atol=1e-6)
    np.testing.assert_allclose(u2, u, rtol=0, atol=1e-6)
    w, w2 = one.wss(), grp.wss()
    assert np.array_equal(w["member"], w2["member"])
    for m in range(len(members)):
        sel = w["member"] == m
        err = np.linalg.norm(w2["tawss"][sel] - w["tawss"][sel]) / np.linalg.norm(w["tawss"][sel])
        assert err < 1e-5, err
    _, _, fl = one.solver.conservation()
    _, _, fl2 = grp.conservation()
    np.testing.assert_allclose(fl2, fl, rtol=1e-5, atol=1e-9)
    grp.close()
