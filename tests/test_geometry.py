"""Synthetic geometry generators: closed surfaces, outward normals, lattice
sizing through bbox anchors."""
import numpy as np
import pytest

from pv_dec_original_gb300 import geometry as G


def _edges_closed(surf):
    """Every directed edge (a->b) of a closed, consistently oriented surface
    appears reversed (b->a) exactly once."""
    v = np.round(surf.v, 9)
    keys = {}
    for t in range(surf.ntri):
        for k in range(3):
            a, b = tuple(v[t, k]), tuple(v[t, (k + 1) % 3])
            keys[(a, b)] = keys.get((a, b), 0) + 1
    return all(keys.get((b, a), 0) == n for (a, b), n in keys.items())


def _enclosed_volume(surf):
    v = surf.v
    return float(np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])).sum() / 6.0)


@pytest.mark.parametrize("maker", [
    lambda: G.capped_cylinder(10.0, 100.0, 48),
    lambda: G.elbow(radius=4.0, leg=12.0, h=1.5, exit="z-"),
    lambda: G.elbow(radius=4.0, leg=12.0, h=1.5, exit="y+"),
    lambda: G.stenosed_tube(5.0, 30.0, 0.5, 0.2, h=1.2),
    lambda: G.y_bifurcation(6.0, 4.25, 30.0, z_in=1.3, z_out=60.6, z_split=38.0, h=1.5),
], ids=["cylinder", "elbow_z", "elbow_y", "stenosis", "bifurcation"])
def test_surfaces_closed_and_outward(maker):
    s = maker()
    assert s.ntri > 0
    assert _edges_closed(s)
    assert _enclosed_volume(s) > 0  # outward orientation
    # file normals agree with the vertex winding
    n = np.cross(s.v[:, 1] - s.v[:, 0], s.v[:, 2] - s.v[:, 0])
    assert np.all((n * s.n).sum(axis=1) > 0)


def test_cylinder_volume_close_to_analytic():
    s = G.capped_cylinder(10.0, 100.0, 48)
    vol = _enclosed_volume(s)
    poly = 0.5 * 48 * 10.0 ** 2 * np.sin(2 * np.pi / 48) * 100.0
    assert abs(vol - poly) < 1e-6 * poly


def test_stenosis_removes_requested_area():
    s = G.stenosed_tube(10.0, 80.0, 0.5, 0.0, h=0.8)
    # the SDF throat radius is r (1 - k) with k = 1 - sqrt(1 - severity)
    z = s.v[..., 2]
    throat = s.v[np.abs(z - 40.0) < 0.5]
    r = np.hypot(throat[:, 0], throat[:, 1]).max()
    assert abs(r - 10.0 * np.sqrt(0.5)) < 0.8


@pytest.mark.parametrize("cfg,dims", [(G.config_c1_cylinder, (24, 24, 104))])
def test_anchor_lattice(cfg, dims):
    s = cfg()
    bb, d = G.reference_lattice_dims(s.tri12(), 1.0)
    assert d == dims


def test_c2_lattice_and_stl_round_trip(tmp_path):
    s = G.config_c2_bifurcation()
    _, d = G.reference_lattice_dims(s.tri12(), 1.0)
    assert d == (256, 192, 512)
    p = str(tmp_path / "c2.stl")
    G.write_stl_ascii(p, s)
    assert np.array_equal(G.read_stl_ascii(p), s.tri12())


def test_ensemble_members_seeded():
    a = G.config_c4_ensemble(3, seed=7)
    b = G.config_c4_ensemble(3, seed=7)
    for x, y in zip(a, b):
        assert np.array_equal(x["surface"].v, y["surface"].v)
        assert 8 <= x["radius"] <= 20 and 120 <= x["length"] <= 400
        assert 0.2 <= x["severity"] <= 0.7 and 0 <= x["eccentricity"] <= 0.3
        assert 2000 <= x["period"] <= 6000 and 0.01 <= x["inlet_mean"] <= 0.04


def test_ensemble_groups_split_contiguously_and_balanced():
    """GroupedEnsemble's split: contiguous runs covering every member once,
    none empty, each run's total near an equal share."""
    from pv_dec_original_gb300.ensemble import split_balanced
    rng = np.random.default_rng(3)
    for n, g in ((64, 4), (64, 8), (5, 5), (7, 3), (3, 8), (1, 1)):
        sizes = rng.integers(50_000, 400_000, n)
        cuts = split_balanced(sizes, g)
        assert len(cuts) == min(g, n)
        assert cuts[0][0] == 0 and cuts[-1][1] == n
        assert all(a < b for a, b in cuts)
        assert all(cuts[k][1] == cuts[k + 1][0] for k in range(len(cuts) - 1))
        if n >= 4 * g:
            share = sizes.sum() / g
            for a, b in cuts:  # off an equal share by at most the largest member
                assert abs(sizes[a:b].sum() - share) <= sizes.max()
    assert split_balanced([5, 5, 5, 5], 2) == [(0, 2), (2, 4)]
    assert split_balanced([1, 1, 1, 10], 2) == [(0, 3), (3, 4)]


def test_grouped_ensemble_bookkeeping_on_the_host(monkeypatch):
    """GroupedEnsemble's host logic with stand-in groups (no device): the
    groups are contiguous member runs balanced by fluid voxels, every call
    reaches every group, and read-outs come back in member order with global
    member indices."""
    from pv_dec_original_gb300 import ensemble as E
    sizes = [5, 9, 4, 7, 6, 8, 3]
    calls = []

    class FakeSolver:
        def __init__(self, g):
            self.g = g

        def stream(self):
            return 1000 + self.g

        def autotune(self, n):
            calls.append(("tune", self.g, n))
            return 6, []

        def set_graph_steps(self, n):
            calls.append(("graph", self.g, n))

        def sync(self):
            calls.append(("sync", self.g))

        def check_status(self):
            calls.append(("status", self.g))

        def launches(self):
            return 10 + self.g

        def conservation(self):
            n = len(groups[self.g])
            return 1.0, np.ones(3), np.arange(2 * n, dtype=float) + 100 * self.g

        def close(self):
            calls.append(("close", self.g))

    groups = []

    class FakeEnsemble:
        def __init__(self, members, Q, precision, tau, parts=None, **kw):
            self.g = len(groups)
            groups.append(members)
            self.solver = FakeSolver(self.g)
            self.n = [int(np.count_nonzero(p[1])) for p in parts]
            self.active = sum(self.n)

        def step_async(self, n):
            calls.append(("step", self.g, n))

        def macro(self):
            mem = np.repeat(np.arange(len(self.n)), self.n)
            return np.full(self.active, float(self.g)), np.zeros((self.active, 3)), mem

        def wss(self):
            mem = np.repeat(np.arange(len(self.n)), 2)
            return {"pt": np.arange(len(mem)), "tawss": np.full(len(mem), float(self.g)), "member": mem}

        def close(self):
            self.solver.close()

    parts = [(None, np.ones(s, np.uint8), None) for s in sizes]
    monkeypatch.setattr(E, "voxelize_members", lambda members: parts)
    monkeypatch.setattr(E, "Ensemble", FakeEnsemble)
    members = [{"k": k} for k in range(len(sizes))]
    grp = E.GroupedEnsemble(members, 3, 19, "f16", 0.55)
    assert [len(m) for m in groups] == [2, 2, 3]  # 14 / 11 / 17 of 42 fluid voxels (targets 14, 28)
    assert grp.first == [0, 2, 4] and grp.active == sum(sizes)
    assert [m["k"] for g in groups for m in g] == list(range(len(sizes)))
    grp.set_graph_steps(32)
    grp.step(7)
    assert [c for c in calls if c[0] == "step"] == [("step", g, 7) for g in range(3)]
    assert {c[1] for c in calls if c[0] == "sync"} == {0, 1, 2}
    rho, u, mem = grp.macro()
    assert np.array_equal(mem, np.repeat(np.arange(len(sizes)), sizes))
    assert np.array_equal(rho, np.repeat([0.0, 1.0, 2.0], [14, 11, 17]))
    w = grp.wss()
    assert np.array_equal(w["member"], np.repeat(np.arange(len(sizes)), 2)) and "pt" not in w
    mass, mom, flux = grp.conservation()
    assert mass == 3.0 and np.array_equal(mom, np.full(3, 3.0)) and len(flux) == 2 * len(sizes)
    assert grp.launches() == 33
    grp.close()
    assert {c[1] for c in calls if c[0] == "close"} == {0, 1, 2}
