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
