"""Golden fixture of the reference's own workload, PV.stl (spacing 0.05).

    python tests/golden/make_pv_fixture.py [--ref DIR] [--threads N]

Reads PV.stl from the reference's tree (--ref, else $LBM_REFERENCE_DIR, else
the REF default of oracle/Makefile) and writes tests/golden/pv_stl.npz:

* the surface: unique vertices, per-facet vertex indices and the file's facet
  normals (the voxelizer uses the file normals), from which the (T, 12)
  triangle rows are rebuilt exactly;
* the lattice by the reference's bounding-box rule (ComplexGeometry.cpp:133-214)
  and the SHA-256 of the voxel mask from the oracle's binned voxelizer (the
  reference's ray test for every point against the triangles of its column,
  ComplexGeometry.cpp:620-674, 803-1053), with its fluid count;
* a block of columns voxelized by the oracle's brute force (every triangle
  for every point, as the reference does), which must equal the binned mask
  there -- the reference's own run over all 207M points is out of reach;
* the classification of the boundary points (ComplexGeometry.cpp:1259-1300)
  by the reference's PV windows (ComplexGeometry.cpp:1369-1429), evaluated in
  long double as the reference does: per window the count and the SHA-256
  of the sorted point indices n = (k ny + j) nx + i, and the wall count.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from pv_dec_original_gb300 import geometry as G  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pv_stl.npz")
SPACING = 0.05
# (plane axis, centre, (lo, hi) on the first transverse axis, (lo, hi) on the
# second, x < y < z order), ComplexGeometry.cpp:1378-1408
WINDOWS = [
    (0, "-16.9538", (-191.0, -187.0), (-118.0, -114.0)),   # inlet
    (1, "-170.016", (2.0, 5.0), (-109.0, -106.0)),         # outlet 1
    (2, "-110.0", (-27.0, -25.0), (-198.0, -195.0)),       # outlet 2
    (2, "-123", (-33.0, -30.0), (-189.0, -186.0)),         # outlet 3
]
# brute-force block: 48 x 48 columns through the vessel's middle, every z
BRUTE_COLS = 48


def sha(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def classify_windows(coords):
    """Index of the first PV window each point lies in (-1: none), with the
    reference's long double comparisons: |c - centre| <= 1e-2 on the plane
    axis, open intervals on the two others."""
    ld = np.longdouble
    out = np.full(len(coords), -1, np.int64)
    for w, (axis, centre, (a0, a1), (b0, b1)) in enumerate(WINDOWS):
        t1, t2 = [a for a in range(3) if a != axis]
        c = coords.astype(ld)
        hit = (np.abs(c[:, axis] - ld(centre)) <= ld(1e-2)) & (ld(a0) < c[:, t1]) & (c[:, t1] < ld(a1)) & \
              (ld(b0) < c[:, t2]) & (c[:, t2] < ld(b1))
        out[(out < 0) & hit] = w
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=O.reference_dir())
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    path = os.path.join(a.ref, "PV.stl")
    if not os.path.exists(path):
        sys.exit(f"PV.stl not found under {a.ref}")
    tri = G.read_stl_ascii(path)
    verts, inv = np.unique(tri[:, :9].reshape(-1, 3), axis=0, return_inverse=True)
    faces = inv.reshape(-1, 3).astype(np.int32)
    normals = tri[:, 9:].copy()
    rebuilt = np.concatenate([verts[faces].reshape(-1, 9), normals], axis=1)
    assert np.array_equal(rebuilt, tri)

    bb, dims = O.bbox_dims(tri, SPACING)
    nx, ny, nz = dims
    t0 = time.perf_counter()
    mask, _, _ = O.voxelize(tri, SPACING, nthreads=a.threads)
    t_bin = time.perf_counter() - t0
    print(f"binned oracle: dims {dims}, fluid {int(mask.sum())}, {t_bin:.1f} s")

    # brute force on a block of columns: same bbox (the ray depends on it),
    # origin shifted to the block
    fl = np.argwhere(mask > 0)
    j0 = int(np.median(fl[:, 1])) - BRUTE_COLS // 2
    i0 = int(np.median(fl[:, 2])) - BRUTE_COLS // 2
    org = np.array([bb[0] + i0 * SPACING, bb[2] + j0 * SPACING, bb[4]])
    t0 = time.perf_counter()
    sub, _, _ = O.voxelize(tri, SPACING, bbox=bb, origin=org, dims=(BRUTE_COLS, BRUTE_COLS, nz), culled=False,
                           nthreads=a.threads)
    t_brute = time.perf_counter() - t0
    assert np.array_equal(sub, mask[:, j0:j0 + BRUTE_COLS, i0:i0 + BRUTE_COLS]), "brute force != binned"
    print(f"brute-force block {BRUTE_COLS}x{BRUTE_COLS} columns at (i0, j0) = ({i0}, {j0}): "
          f"{int(sub.sum())} fluid, equal to the binned mask ({t_brute:.1f} s)")

    b = O.find_boundary(mask, 19).reshape(-1)
    bidx = np.flatnonzero(b)
    i = bidx % nx
    j = (bidx // nx) % ny
    k = bidx // (nx * ny)
    # point coordinates as generatePointsInSubBox forms them (ComplexGeometry.cpp:338-340)
    coords = np.stack([bb[0] + i * SPACING, bb[2] + j * SPACING, bb[4] + k * SPACING], axis=1)
    win = classify_windows(coords)
    wcount = np.array([int((win == w).sum()) for w in range(len(WINDOWS))], np.int64)
    wsha = np.array([sha(bidx[win == w].astype(np.int64)) for w in range(len(WINDOWS))])
    print(f"boundary points {len(bidx)}, windows {wcount.tolist()}, walls {int((win < 0).sum())}")

    np.savez_compressed(
        OUT, verts=verts, faces=faces, normals=normals, spacing=SPACING, dims=np.array(dims), bbox=bb,
        mask_sha=sha(mask.reshape(-1)), nfluid=int(mask.sum()), nboundary=len(bidx),
        brute_block=np.array([i0, j0, BRUTE_COLS]), brute_fluid=int(sub.sum()),
        window_count=wcount, window_sha=wsha, nwall=int((win < 0).sum()))
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
