"""The reference's PV case on the GPU: the PV coordinate-window classifier
(ComplexGeometry.cpp:1369-1429) against the reference's long double rule,
and the full PV.stl lattice (752x583x472 points at spacing 0.05) against the
pins of tests/golden/pv_stl.npz (tests/golden/make_pv_fixture.py)."""
import hashlib
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu

# (plane axis, centre as the reference's long double literal, transverse
# open intervals in x < y < z order, the rule's face), ComplexGeometry.cpp:1378-1408
WINDOWS = [
    (0, "-16.9538", (-191.0, -187.0), (-118.0, -114.0), "x-"),
    (1, "-170.016", (2.0, 5.0), (-109.0, -106.0), "y+"),
    (2, "-110.0", (-27.0, -25.0), (-198.0, -195.0), "z-"),
    (2, "-123", (-33.0, -30.0), (-189.0, -186.0), "z-"),
]
TOL = 1e-2


def _sha(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def pv_rules(capi):
    """The PV preset (Geometry::UsePVPreset): the reference's inlet and three
    outlets as region rules, in the reference's order."""
    kinds = [capi.LBM_BC_REF_INLET, capi.LBM_BC_REF_OUTLET_YMAX, capi.LBM_BC_REF_OUTLET_ZMIN,
             capi.LBM_BC_REF_OUTLET_ZMIN]
    return [capi.bc_spec(k, face, -1, 1.0, region=(float(c), TOL, t1, t2))
            for k, (axis, c, t1, t2, face) in zip(kinds, WINDOWS)]


def reference_window(coords, w):
    """The reference's test of window w, in long double (numpy's longdouble:
    the platform's long double, as the reference's compiler gives it)."""
    ld = np.longdouble
    axis, c, (a0, a1), (b0, b1), _ = WINDOWS[w]
    t1, t2 = [a for a in range(3) if a != axis]
    x = coords.astype(ld)
    return (np.abs(x[:, axis] - ld(c)) <= ld(TOL)) & (ld(a0) < x[:, t1]) & (x[:, t1] < ld(a1)) & \
        (ld(b0) < x[:, t2]) & (x[:, t2] < ld(b1))


def fp64_window(coords, w):
    axis, c, (a0, a1), (b0, b1), _ = WINDOWS[w]
    t1, t2 = [a for a in range(3) if a != axis]
    return (np.abs(coords[:, axis] - float(c)) <= TOL) & (a0 < coords[:, t1]) & (coords[:, t1] < a1) & \
        (b0 < coords[:, t2]) & (coords[:, t2] < b1)


@pytest.mark.parametrize("w", range(4))
@pytest.mark.parametrize("shift", [0.0, 2e-12, -2e-12])
def test_pv_window_classifier_matches_reference_rule(gpu_lib, w, shift):
    """A lattice of spacing 0.01 around window w: on the plane axis from
    centre - 0.04 to centre + 0.04 (points on both edges of the +-0.01 band
    and beyond), on the transverse axes 0.03 past both ends of the open
    intervals (points on each end).  The origin moves by `shift` on every
    axis, which puts the edge points just inside or just outside.  The mask
    is a checkerboard, so every fluid point is a boundary point; both
    parities are run.  Every point must get the class the reference's rule
    gives, except where FP64 and long double disagree within rounding of an
    edge (|distance - 0.01| < 1e-12), the documented deviation."""
    capi = gpu_lib
    axis, c, (a0, a1), (b0, b1), _ = WINDOWS[w]
    t1, t2 = [a for a in range(3) if a != axis]
    s = 0.01
    lo, n = [0.0] * 3, [0] * 3
    lo[axis], n[axis] = float(c) - 0.04, 9
    lo[t1], n[t1] = a0 - 0.03, int(round((a1 - a0 + 0.06) / s)) + 1
    lo[t2], n[t2] = b0 - 0.03, int(round((b1 - b0 + 0.06) / s)) + 1
    org = tuple(v + shift for v in lo)
    nx, ny, nz = n
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    coords = np.stack([org[0] + I.reshape(-1) * s, org[1] + J.reshape(-1) * s, org[2] + K.reshape(-1) * s], axis=1)
    ref = reference_window(coords, w)
    f64 = fp64_window(coords, w)
    dist = np.abs(coords[:, axis] - float(c))
    edge = np.abs(dist - TOL) < 1e-12
    assert np.array_equal(ref[~edge], f64[~edge])
    if shift != 0.0:
        assert not edge.any()
    for parity in (0, 1):
        mask = (((I + J + K) % 2) == parity).astype(np.uint8)
        sol = capi.Solver(19, capi.LBM_F32, capi.LBM_PHYSICS, 0.8, s, org, 1.0, 0.9)
        sol.set_geometry(mask, pv_rules(capi))
        cls = (sol.classes().reshape(-1) & 0x7F).astype(np.int64)
        sol.close()
        fl = mask.reshape(-1) > 0
        want = np.where(ref, 3 + w, 2)
        got = cls[fl]
        bad = (got != want[fl]) & ~edge[fl]
        assert not bad.any(), f"window {w}: {int(bad.sum())} points classified unlike the reference"
        assert np.array_equal(got[edge[fl]] == 3 + w, f64[fl][edge[fl]])
        assert (got == 3 + w).sum() > 0


def _pv():
    path = os.path.join(GOLDEN, "pv_stl.npz")
    d = dict(np.load(path, allow_pickle=False))
    tri = np.concatenate([d["verts"][d["faces"]].reshape(-1, 9), d["normals"]], axis=1)
    return d, np.ascontiguousarray(tri)


def test_pv_mask_and_windows_match_pins(gpu_lib):
    """PV.stl: the GPU voxel mask equals the pinned mask bit for bit, and the
    PV preset puts exactly the pinned boundary points in each of the
    reference's inlet / outlet lists."""
    capi = gpu_lib
    d, tri = _pv()
    sp = float(d["spacing"])
    mask, desc = capi.voxelize(tri, sp)
    assert tuple(mask.shape[::-1]) == tuple(int(v) for v in d["dims"])
    assert int(mask.sum()) == int(d["nfluid"])
    assert _sha(mask.reshape(-1)) == str(d["mask_sha"]), "PV voxel mask differs from the pin"
    bb = np.array(desc.bbox[:])
    np.testing.assert_array_equal(bb, d["bbox"])
    s = capi.Solver(19, capi.LBM_F32, capi.LBM_PHYSICS, 1.5, sp, (bb[0], bb[2], bb[4]), 1.0, 0.9)
    s.set_geometry(mask, pv_rules(capi))
    cls = s.classes().reshape(-1) & 0x7F
    for w in range(4):
        pts = np.flatnonzero(cls == 3 + w).astype(np.int64)
        assert len(pts) == int(d["window_count"][w]), (w, len(pts))
        assert _sha(pts) == str(d["window_sha"][w]), f"window {w} point set differs from the pin"
    assert int((cls == 2).sum()) == int(d["nwall"])
    s.close()
