"""The CPU oracle against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py from the reference compiled unchanged)."""
import numpy as np
import pytest

from helpers import classify, fixtures, golden_mask, load, sha, sim_bcs, wss_C


@pytest.mark.parametrize("path", fixtures("vox"), ids=lambda p: p.split("/")[-1])
@pytest.mark.parametrize("culled", [False, True])
def test_oracle_mask_matches_reference(oracle_lib, path, culled):
    O = oracle_lib
    d = load(path)
    bb, dims = O.bbox_dims(d["tri12"], float(d["spacing"]))
    assert tuple(dims) == tuple(d["dims"])
    assert np.array_equal(bb, d["bbox"])
    mask, _, _ = O.voxelize(d["tri12"], float(d["spacing"]), culled=culled)
    ref = golden_mask(d)
    assert int(mask.sum()) == int(d["nfluid"])
    assert np.array_equal(mask, ref)


@pytest.mark.parametrize("path", fixtures("vox"), ids=lambda p: p.split("/")[-1])
def test_oracle_boundary_points_match_reference(oracle_lib, path):
    d = load(path)
    b = oracle_lib.find_boundary(golden_mask(d), 19)
    ijk = np.argwhere(b.transpose(2, 1, 0) > 0).astype(np.int32)  # reference order: i, j, k loops
    assert len(ijk) == int(d["nboundary"])
    assert sha(ijk) == str(d["boundary_ijk_sha"])


def _oracle_parity_run(O, d):
    mask, bb, dims = O.voxelize(d["tri12"], float(d["spacing"]))
    bcs = sim_bcs(d)
    cls = classify(mask, [(axis, spec["plane"]) for axis, spec in bcs])
    sim = O.Sim(19, O.PARITY, cls, (bb[0], bb[2], bb[4]), float(d["spacing"]), float(d["tau"]),
                [spec for _, spec in bcs])
    sim.set_amplitude(d["amp"])
    sim.set_wss(wss_C(float(d["dt"]), float(d["spacing"])), 0.9)
    sim.compute_normals(d["tri12"])
    sim.step(int(d["nsteps"]))
    return sim, cls


@pytest.mark.parametrize("path", fixtures("sim"), ids=lambda p: p.split("/")[-1])
def test_oracle_step_bit_exact_vs_reference(oracle_lib, path):
    d = load(path)
    sim, cls = _oracle_parity_run(oracle_lib, d)
    pt, c = sim.active()
    assert np.array_equal(pt, d["active_pt"])
    assert np.array_equal(c, d["active_cls"])
    f, fnew, feq = sim.f()
    assert sha(f) == str(d["f_sha"])
    assert sha(fnew) == str(d["fnew_sha"])
    assert sha(feq) == str(d["feq_sha"])
    rho, u = sim.macro()
    assert np.array_equal(rho, d["rho"]) and np.array_equal(u, d["u"])
    nw = sim.nw()
    assert np.array_equal(nw["pt"], d["nw_pt"])
    for k in ("normal", "wss", "acc", "acc_mag", "osi", "tawss"):
        assert np.array_equal(nw[k], d["nw_" + k]), k


def _pv_fixture():
    from helpers import GOLDEN
    d = load(GOLDEN + "/pv_stl.npz")
    tri = np.concatenate([d["verts"][d["faces"]].reshape(-1, 9), d["normals"]], axis=1)
    return d, np.ascontiguousarray(tri)


def test_oracle_pv_mask_pin(oracle_lib):
    """PV.stl at spacing 0.05: the binned oracle's mask is the pinned one,
    and the brute-force oracle (every triangle for every point, the
    reference's loop) agrees with it on 12x12 columns of the pinned block."""
    O = oracle_lib
    d, tri = _pv_fixture()
    sp = float(d["spacing"])
    bb, dims = O.bbox_dims(tri, sp)
    assert tuple(dims) == tuple(int(v) for v in d["dims"]) and np.array_equal(bb, d["bbox"])
    mask, _, _ = O.voxelize(tri, sp)
    assert int(mask.sum()) == int(d["nfluid"])
    assert sha(mask.reshape(-1)) == str(d["mask_sha"])
    i0, j0, n = (int(v) for v in d["brute_block"])
    i0, j0 = i0 + n // 2 - 6, j0 + n // 2 - 6
    org = (bb[0] + i0 * sp, bb[2] + j0 * sp, bb[4])
    sub, _, _ = O.voxelize(tri, sp, bbox=bb, origin=org, dims=(12, 12, dims[2]), culled=False)
    assert sub.any() and np.array_equal(sub, mask[:, j0:j0 + 12, i0:i0 + 12])


def test_pv_windows_pin_from_reference_rule(oracle_lib):
    """The reference's PV windows (ComplexGeometry.cpp:1369-1429, long
    double) on the pinned mask's boundary points give the pinned lists."""
    import importlib.util
    from helpers import GOLDEN
    spec = importlib.util.spec_from_file_location("make_pv_fixture", GOLDEN + "/make_pv_fixture.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    O = oracle_lib
    d, tri = _pv_fixture()
    sp = float(d["spacing"])
    nx, ny, nz = (int(v) for v in d["dims"])
    bb = d["bbox"]
    mask, _, _ = O.voxelize(tri, sp)
    bidx = np.flatnonzero(O.find_boundary(mask, 19).reshape(-1))
    assert len(bidx) == int(d["nboundary"])
    coords = np.stack([bb[0] + (bidx % nx) * sp, bb[2] + ((bidx // nx) % ny) * sp, bb[4] + (bidx // (nx * ny)) * sp],
                      axis=1)
    win = mk.classify_windows(coords)
    for w in range(4):
        assert int((win == w).sum()) == int(d["window_count"][w])
        assert sha(bidx[win == w].astype(np.int64)) == str(d["window_sha"][w])
    assert int((win < 0).sum()) == int(d["nwall"])


def test_waveform_matches_reference():
    from helpers import GOLDEN
    from pv_dec_original_gb300 import waveform
    d = load(GOLDEN + "/pulse.npz")
    tab = waveform.reference_table(float(d["dt"]), int(d["n"]))
    got = tab[d["idx"]]
    # libm pow may differ by an ulp across platforms; on the fixture's own
    # platform the table is bit-identical
    np.testing.assert_allclose(got, d["v"], rtol=1e-14, atol=1e-15)
    t = np.cumsum(np.r_[0.0, np.full(int(d["n"]) - 1, float(d["dt"]))])
    assert np.all(np.abs(tab) < 2.0)
    assert tab[0] == 0.1423
