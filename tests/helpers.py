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
