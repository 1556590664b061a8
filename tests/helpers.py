"""Shared test helpers: golden fixtures, plane-rule classification."""
import glob
import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def fixtures(prefix):
    return sorted(glob.glob(os.path.join(GOLDEN, prefix + "_*.npz")))


def load(path):
    d = dict(np.load(path, allow_pickle=False))
    return d


def golden_mask(d):
    nx, ny, nz = (int(v) for v in d["dims"])
    return np.unpackbits(d["mask_bits"])[: nx * ny * nz].reshape(nz, ny, nx)


def classify(mask, rules, Q=19):
    """Plane rules (first match wins, remaining boundary points are walls)."""
    from oracle import oracle as O
    b = O.find_boundary(mask, Q)
    cls = np.where(mask > 0, 1, 0).astype(np.uint8)
    nz, ny, nx = mask.shape
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    idx = [I, J, K]
    taken = np.zeros(mask.shape, bool)
    for r, (axis, plane) in enumerate(rules):
        sel = (b > 0) & ~taken & (idx[axis] == plane)
        cls[sel] = 3 + r
        taken |= sel
    cls[(b > 0) & ~taken] = 2
    return cls


REF_KIND = {"inlet": 1, "outlet1": 2, "outlet2": 3, "outlet3": 3}
REF_FACE = {"inlet": 0, "outlet1": 3, "outlet2": 4, "outlet3": 4}


def sim_bcs(d):
    """Boundary specs (as dicts) of a golden parity run."""
    out = []
    prof = d["profile"]
    for key, (axis, plane) in zip(d["rule_keys"], d["rules"]):
        key = str(key)
        spec = dict(kind=REF_KIND[key], face=2 * int(axis) + REF_FACE[key] % 2, plane=int(plane), value=1.0)
        if key == "inlet" and bool(d["has_profile"]):
            spec.update(profile=1, c1=float(prof[0]), c2=float(prof[1]), R=float(prof[2]))
        out.append((int(axis), spec))
    return out


def wss_C(dt, spacing):
    # ComputeWallShearStress's constant, in its evaluation order (Simulation.cpp:880-881)
    return 1060.0 * (dt * dt) / ((spacing * spacing) * 1e-6)


# ------------------------------------------------------- warm-start checkers
def slice_distance(mask):
    """In-slice distance (flow along z) of every fluid voxel to the nearest
    fluid voxel with a solid (or out-of-box) in-plane 4-neighbour, + 0.5;
    0 on solid.  Exact (brute force per slice): the checker of the jump
    flooding in lbm_ws_prior."""
    D, H, W = mask.shape
    out = np.zeros(mask.shape, np.float64)
    fl = mask > 0
    pad = np.pad(fl, ((0, 0), (1, 1), (1, 1)))
    inner = pad[:, 1:-1, 1:-1]
    seed = inner & ~(pad[:, 2:, 1:-1] & pad[:, :-2, 1:-1] & pad[:, 1:-1, 2:] & pad[:, 1:-1, :-2])
    yy, xx = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    for z in range(D):
        sy, sx = np.nonzero(seed[z])
        if sy.size == 0:
            continue
        fy, fx = np.nonzero(fl[z])
        d2 = (fy[:, None] - sy[None, :]) ** 2 + (fx[:, None] - sx[None, :]) ** 2
        out[z, fy, fx] = np.sqrt(d2.min(1)) + 0.5
    return out


def poiseuille_prior(mask, inlet, tau, s=None):
    """Slice-wise Hagen-Poiseuille prior, FP64 (the checker of
    lbm_ws_prior) from the in-slice distance s (slice_distance when None):
    returns (rho - 1, u_z) voxel arrays."""
    import math
    D = mask.shape[0]
    fl = mask > 0
    s = slice_distance(mask) if s is None else np.asarray(s, np.float64)
    R = s.reshape(D, -1).max(1)
    zs = np.nonzero(R > 0)[0]
    if zs.size == 0:
        return np.zeros(mask.shape), np.zeros(mask.shape)
    Q = math.pi * R[zs[0]] ** 2 * inlet / 2.0
    nu = (tau - 0.5) / 3.0
    Rs = np.maximum(R, 1.0)
    peak = 2.0 * Q / (math.pi * Rs ** 2)
    prof = np.clip(1.0 - (Rs[:, None, None] - s) ** 2 / Rs[:, None, None] ** 2, 0.0, 1.0)
    uz = np.where(fl, peak[:, None, None] * prof, 0.0)
    drho = np.where(R > 0, 3.0 * 8.0 * nu * Q / (math.pi * Rs ** 4), 0.0)
    tail = np.concatenate([np.cumsum(drho[::-1])[::-1][1:], [0.0]])  # sum over the slices downstream
    return np.where(fl, tail[:, None, None], 0.0), uz


def smooth_masked(mask, v, rounds=2):
    """[1, 2, 1] / 4 filter along z, y, x restricted to fluid voxels
    (weights renormalised where a neighbour is solid or outside the box),
    FP64: the checker of lbm_ws_smooth."""
    fl = mask > 0
    v = np.where(fl, v, 0.0)
    w = fl.astype(np.float64)
    for _ in range(rounds):
        for a in range(3):
            num, den = 2.0 * v, 2.0 * w
            for sh in (1, -1):
                e = np.ones(mask.shape[a])
                e[0 if sh == 1 else -1] = 0.0
                e = e.reshape([-1 if k == a else 1 for k in range(3)])
                num = num + np.roll(v * w, sh, axis=a) * e
                den = den + np.roll(w, sh, axis=a) * e
            v = np.where(fl, num / np.maximum(den, 1e-30), 0.0)
    return v
