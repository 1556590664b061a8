"""Seeded synthetic vessel geometries written as ASCII STL.

The reference reads one patient STL (``PV.stl``) through
``Reader::readSTLASCII`` (GeometryReader.cpp:33-117) and voxelizes it with a
+z ray-parity test (ComplexGeometry.cpp:978-1053).  These generators make the
closed, outward-oriented triangle surfaces used by the benchmark and test
workloads:

* :func:`capped_cylinder` -- straight tube with fan caps (48 facets around).
* :func:`y_bifurcation`   -- parent tube splitting into two daughters.
* :func:`stenosed_tube`   -- tube with a cosine stenosis and eccentricity.
* :func:`elbow`           -- tube entering along +x and leaving along -z.

Curved unions are meshed with marching tetrahedra over a signed distance
function (six tetrahedra per grid cube, all sharing the cube's main diagonal,
so neighbouring cubes split their shared faces the same way and the surface
is watertight).

The lattice of the reference is derived from the STL bounding box
(ComplexGeometry.cpp:145-165: ``nx = ceil(dx/s)+1``, ``ny = ceil(dy/s)+1``,
``nz = ceil(dz/s)``; the y/z extremes ignore each facet's third vertex).  To
place a vessel inside a lattice of a prescribed size, :func:`add_bbox_anchors`
adds two tiny closed tetrahedra at opposite corners of the wanted box.  No
lattice ray can meet them: the rays of the extreme columns are moved 0.02
inwards (ComplexGeometry.cpp:853-884) and the anchors are 0.01 wide.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Surface", "write_stl_ascii", "read_stl_ascii", "capped_cylinder", "y_bifurcation",
    "stenosed_tube", "elbow", "add_bbox_anchors", "marching_tetrahedra", "reference_lattice_dims",
    "config_c1_cylinder", "config_c1_cylinder_x", "config_c2_bifurcation", "config_c4_ensemble",
]


@dataclass
class Surface:
    """Triangle soup: ``v`` is (T, 3, 3) float64 vertices, ``n`` (T, 3) unit normals."""
    v: np.ndarray
    n: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def ntri(self) -> int:
        return int(self.v.shape[0])

    def tri12(self) -> np.ndarray:
        """(T, 12) float64 rows ``x1 y1 z1 x2 y2 z2 x3 y3 z3 nx ny nz`` (Struct.h:117-125 order)."""
        return np.ascontiguousarray(np.concatenate([self.v.reshape(-1, 9), self.n], axis=1))

    def concat(self, other: "Surface") -> "Surface":
        return Surface(np.concatenate([self.v, other.v]), np.concatenate([self.n, other.n]),
                       dict(self.meta))


def _unit_normals(v: np.ndarray) -> np.ndarray:
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return n / ln


def write_stl_ascii(path: str, surf: Surface, name: str = "vessel") -> None:
    """Write ASCII STL with ``%.17g`` so every double round-trips exactly."""
    lines = [f"solid {name}"]
    for t in range(surf.ntri):
        n = surf.n[t]
        lines.append(f"  facet normal {n[0]:.17g} {n[1]:.17g} {n[2]:.17g}")
        lines.append("    outer loop")
        for k in range(3):
            p = surf.v[t, k]
            lines.append(f"      vertex {p[0]:.17g} {p[1]:.17g} {p[2]:.17g}")
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append(f"endsolid {name}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_stl_ascii(path: str) -> np.ndarray:
    """Parse ASCII STL into (T, 12) float64 rows, following readSTLASCII's rules.

    A facet counts only when the ``facet normal``, ``outer loop``, three
    ``vertex``, ``endloop`` and ``endfacet`` lines appear in order
    (GeometryReader.cpp:50-110); Python's ``float`` rounds correctly, like the
    ``istream >> double`` of the reference.
    """
    out = []
    with open(path) as f:
        lines = f.read().split("\n")
    i, n = 0, len(lines)
    while i < n:
        tok = lines[i].split()
        i += 1
        if len(tok) < 5 or tok[0] != "facet" or tok[1] != "normal":
            continue
        try:
            nrm = [float(tok[2]), float(tok[3]), float(tok[4])]
        except ValueError:
            continue
        if i >= n:
            break
        tok = lines[i].split(); i += 1
        if len(tok) < 2 or tok[0] != "outer" or tok[1] != "loop":
            continue
        verts = []
        for _ in range(3):
            if i >= n:
                break
            tok = lines[i].split(); i += 1
            if len(tok) < 4 or tok[0] != "vertex":
                break
            verts.append([float(tok[1]), float(tok[2]), float(tok[3])])
        if len(verts) < 3:
            # the reference keeps the previous facet's values for missing
            # vertices; malformed facets are simply dropped here
            continue
        if i >= n:
            break
        tok = lines[i].split(); i += 1
        if not tok or tok[0] != "endloop":
            continue
        if i >= n:
            break
        tok = lines[i].split(); i += 1
        if not tok or tok[0] != "endfacet":
            continue
        out.append(verts[0] + verts[1] + verts[2] + nrm)
    return np.asarray(out, dtype=np.float64).reshape(-1, 12)


def reference_lattice_dims(tri12: np.ndarray, spacing: float):
    """Bounding box and lattice size by the reference rule (ComplexGeometry.cpp:145-165)."""
    t = np.asarray(tri12)
    min_x = min(t[:, 0].min(), t[:, 3].min(), t[:, 6].min())
    max_x = max(t[:, 0].max(), t[:, 3].max(), t[:, 6].max())
    min_y = min(t[:, 1].min(), t[:, 4].min())
    max_y = max(t[:, 1].max(), t[:, 4].max())
    min_z = min(t[:, 2].min(), t[:, 5].min())
    max_z = max(t[:, 2].max(), t[:, 5].max())
    nx = int(math.ceil((max_x - min_x) / spacing)) + 1
    ny = int(math.ceil((max_y - min_y) / spacing)) + 1
    nz = int(math.ceil((max_z - min_z) / spacing))
    return (min_x, max_x, min_y, max_y, min_z, max_z), (nx, ny, nz)


# ---------------------------------------------------------------------------
# analytic capped cylinder

def capped_cylinder(radius: float, length: float, n_around: int = 48, center=(0.0, 0.0),
                    z0: float = 0.0, phase: float = 0.5) -> Surface:
    """Cylinder along +z with fan caps; ``phase`` rotates the polygon by a
    fraction of one facet so no lattice column runs along a fan edge."""
    th = 2.0 * math.pi * (np.arange(n_around) + phase) / n_around
    cx, cy = center
    ring = np.stack([cx + radius * np.cos(th), cy + radius * np.sin(th)], axis=1)
    z1 = z0 + length
    tris = []
    for a in range(n_around):
        b = (a + 1) % n_around
        pa0 = [ring[a, 0], ring[a, 1], z0]
        pb0 = [ring[b, 0], ring[b, 1], z0]
        pa1 = [ring[a, 0], ring[a, 1], z1]
        pb1 = [ring[b, 0], ring[b, 1], z1]
        tris.append([pa0, pb0, pb1])        # side, outward
        tris.append([pa0, pb1, pa1])
        tris.append([[cx, cy, z0], pb0, pa0])  # bottom cap, normal -z
        tris.append([[cx, cy, z1], pa1, pb1])  # top cap, normal +z
    v = np.asarray(tris, dtype=np.float64)
    return Surface(v, _unit_normals(v), {"kind": "cylinder", "radius": radius, "length": length})


# ---------------------------------------------------------------------------
# marching tetrahedra over a signed distance function

_CUBE = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0],
                  [0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]], dtype=np.int64)
_TETS = np.array([[0, 1, 3, 7], [0, 3, 2, 7], [0, 2, 6, 7],
                  [0, 6, 4, 7], [0, 4, 5, 7], [0, 5, 1, 7]], dtype=np.int64)


def marching_tetrahedra(sdf, lo, hi, h: float) -> Surface:
    """Mesh the zero level set of ``sdf`` (negative inside) on a grid of step ``h``.

    Vertices on a grid edge are interpolated from the lower to the higher
    flattened grid index, so two tetrahedra sharing an edge produce the same
    point bit for bit.
    """
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    dims = np.maximum(np.ceil((hi - lo) / h).astype(np.int64) + 1, 2)
    gx = lo[0] + h * np.arange(dims[0])
    gy = lo[1] + h * np.arange(dims[1])
    gz = lo[2] + h * np.arange(dims[2])
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    P = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    V = np.asarray(sdf(P), dtype=np.float64)
    nyz = dims[1] * dims[2]

    def gid(ijk):
        return ijk[..., 0] * nyz + ijk[..., 1] * dims[2] + ijk[..., 2]

    ci = np.stack(np.meshgrid(np.arange(dims[0] - 1), np.arange(dims[1] - 1), np.arange(dims[2] - 1),
                              indexing="ij"), axis=-1).reshape(-1, 3)
    # cull cubes whose 8 corners share one sign
    corner_ids = gid(ci[:, None, :] + _CUBE[None, :, :])  # (C, 8)
    cv = V[corner_ids] < 0.0
    mixed = cv.any(axis=1) & ~cv.all(axis=1)
    corner_ids = corner_ids[mixed]

    out = []

    def edge_point(a, b):
        swap = a > b
        lo_id = np.where(swap, b, a)
        hi_id = np.where(swap, a, b)
        va, vb = V[lo_id], V[hi_id]
        t = va / (va - vb)
        return P[lo_id] + t[:, None] * (P[hi_id] - P[lo_id])

    for tet in _TETS:
        ids = corner_ids[:, tet]  # (C, 4)
        inside = V[ids] < 0.0
        code = (inside * np.array([1, 2, 4, 8])).sum(axis=1)
        for case in range(1, 15):
            sel = code == case
            if not sel.any():
                continue
            T = ids[sel]
            ins = [k for k in range(4) if case & (1 << k)]
            outs = [k for k in range(4) if not case & (1 << k)]
            pin = P[T[:, ins]].mean(axis=1)
            pout = P[T[:, outs]].mean(axis=1)
            grad = pout - pin
            if len(ins) == 1 or len(outs) == 1:
                lone = ins[0] if len(ins) == 1 else outs[0]
                others = [k for k in range(4) if k != lone]
                p = [edge_point(T[:, lone], T[:, o]) for o in others]
                tris = [np.stack(p, axis=1)]
            else:
                i1, i2 = ins
                o1, o2 = outs
                e11 = edge_point(T[:, i1], T[:, o1])
                e12 = edge_point(T[:, i1], T[:, o2])
                e22 = edge_point(T[:, i2], T[:, o2])
                e21 = edge_point(T[:, i2], T[:, o1])
                tris = [np.stack([e11, e12, e22], axis=1), np.stack([e11, e22, e21], axis=1)]
            for tv in tris:
                nrm = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
                flip = (nrm * grad).sum(axis=1) < 0.0
                tv = tv.copy()
                tv[flip, 1], tv[flip, 2] = tv[flip, 2].copy(), tv[flip, 1].copy()
                out.append(tv)
    v = np.concatenate(out) if out else np.zeros((0, 3, 3))
    # drop zero-area facets (interpolation landing on a grid vertex)
    area2 = np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1)
    v = v[area2 > 1e-12]
    return Surface(v, _unit_normals(v))


def _capsule(p, a, b, r):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ab = b - a
    t = np.clip(((p - a) @ ab) / (ab @ ab), 0.0, 1.0)
    q = a + t[:, None] * ab
    return np.linalg.norm(p - q, axis=1) - r


def y_bifurcation(parent_radius: float = 24.0, daughter_radius: float = 17.0, angle_deg: float = 30.0,
                  z_in: float = 0.0, z_out: float = 500.0, z_split: float = 300.0,
                  center=(0.0, 0.0), seed: int = 0, h: float = 2.0) -> Surface:
    """Parent tube along +z splitting at ``z_split`` into two daughters at
    +/-``angle_deg`` in the x-z plane; flat inlet cut at ``z_in`` and flat
    outlet cut at ``z_out``.  ``seed`` jitters the meshing grid."""
    rng = np.random.default_rng(seed)
    cx, cy = center
    ang = math.radians(angle_deg)
    B = np.array([cx, cy, z_split])
    L = (z_out - z_split) / math.cos(ang) + 2 * daughter_radius
    D1 = B + L * np.array([math.sin(ang), 0.0, math.cos(ang)])
    D2 = B + L * np.array([-math.sin(ang), 0.0, math.cos(ang)])
    P0 = np.array([cx, cy, z_in - 2 * parent_radius])

    def sdf(p):
        d = np.minimum(_capsule(p, P0, B, parent_radius),
                       np.minimum(_capsule(p, B, D1, daughter_radius), _capsule(p, B, D2, daughter_radius)))
        d = np.maximum(d, z_in - p[:, 2])
        return np.maximum(d, p[:, 2] - z_out)

    spread = (z_out - z_split) * math.tan(ang) + daughter_radius / math.cos(ang) + 2 * h
    rad = max(parent_radius, daughter_radius) + 2 * h
    jitter = rng.uniform(0.11, 0.37, size=3) * h
    lo = np.array([cx - max(spread, rad), cy - rad, z_in - 2 * h]) - jitter
    hi = np.array([cx + max(spread, rad), cy + rad, z_out + 2 * h])
    s = marching_tetrahedra(sdf, lo, hi, h)
    s.meta = {"kind": "y_bifurcation", "parent_radius": parent_radius, "daughter_radius": daughter_radius,
              "angle_deg": angle_deg, "z_in": z_in, "z_out": z_out, "center": (cx, cy), "seed": seed}
    return s


def stenosed_tube(radius: float, length: float, severity: float, eccentricity: float = 0.0,
                  center=(0.0, 0.0), z0: float = 0.0, stenosis_len: float | None = None,
                  h: float = 1.5, seed: int = 0) -> Surface:
    """Tube along +z with a cosine stenosis removing ``severity`` of the lumen
    area at its throat; the throat centre moves by ``eccentricity * radius``."""
    rng = np.random.default_rng(seed)
    cx, cy = center
    zc = z0 + 0.5 * length
    ls = stenosis_len if stenosis_len is not None else 4.0 * radius
    k = 1.0 - math.sqrt(1.0 - severity)  # radius reduction at the throat

    def sdf(p):
        z = p[:, 2]
        w = np.where(np.abs(z - zc) < ls / 2, 0.5 * (1.0 + np.cos(2.0 * math.pi * (z - zc) / ls)), 0.0)
        r = radius * (1.0 - k * w)
        off = eccentricity * radius * k * w
        d = np.hypot(p[:, 0] - (cx + off), p[:, 1] - cy) - r
        d = np.maximum(d, z0 - z)
        return np.maximum(d, z - (z0 + length))

    jitter = rng.uniform(0.11, 0.37, size=3) * h
    lo = np.array([cx - radius - 2 * h, cy - radius - 2 * h, z0 - 2 * h]) - jitter
    hi = np.array([cx + radius + 2 * h, cy + radius + 2 * h, z0 + length + 2 * h])
    s = marching_tetrahedra(sdf, lo, hi, h)
    s.meta = {"kind": "stenosed_tube", "radius": radius, "length": length, "severity": severity,
              "eccentricity": eccentricity, "center": (cx, cy), "z0": z0}
    return s


def elbow(radius: float = 6.0, leg: float = 30.0, h: float = 1.25, seed: int = 0, exit: str = "z-") -> Surface:
    """Tube entering along +x through a flat cut at x=0 and leaving either
    along -z through a flat cut at z=0 (``exit="z-"``) or along +y through a
    flat cut at y=leg+radius (``exit="y+"``): the x-min inlet and the z-min /
    y-max outlets are the faces whose Zou-He formulas the reference implements
    (Boundary.cpp:157-185, Simulation.cpp:628-838)."""
    rng = np.random.default_rng(seed)
    if exit == "z-":
        A = np.array([-2 * radius, 0.0, leg])
        B = np.array([leg, 0.0, leg])
        C = np.array([leg, 0.0, -2 * radius])
        cut_lo = lambda p: -p[:, 2]
        lo = np.array([-2 * h, -radius - 2 * h, -2 * h])
        hi = np.array([leg + radius + 2 * h, radius + 2 * h, leg + radius + 2 * h])
    elif exit == "y+":
        top = leg + radius
        A = np.array([-2 * radius, 0.0, 0.0])
        B = np.array([leg, 0.0, 0.0])
        C = np.array([leg, top + 2 * radius, 0.0])
        cut_lo = lambda p: p[:, 1] - top
        lo = np.array([-2 * h, -radius - 2 * h, -radius - 2 * h])
        hi = np.array([leg + radius + 2 * h, top + 2 * h, radius + 2 * h])
    else:
        raise ValueError("exit must be 'z-' or 'y+'")

    def sdf(p):
        d = np.minimum(_capsule(p, A, B, radius), _capsule(p, B, C, radius))
        d = np.maximum(d, -p[:, 0])
        return np.maximum(d, cut_lo(p))

    jitter = rng.uniform(0.11, 0.37, size=3) * h
    s = marching_tetrahedra(sdf, lo - jitter, hi, h)
    s.meta = {"kind": "elbow", "radius": radius, "leg": leg, "exit": exit}
    return s


def add_bbox_anchors(surf: Surface, lo, hi, size: float = 0.01) -> Surface:
    """Append two tiny closed tetrahedra so that the reference's bounding box
    becomes exactly [lo, hi]; each anchor's extreme vertex is listed first in
    its facets (the bbox rule ignores third vertices for y and z)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    tris = []
    for corner, sgn in ((lo, 1.0), (hi, -1.0)):
        a = corner
        b = corner + sgn * np.array([size, 0.0, 0.0])
        c = corner + sgn * np.array([0.0, size, 0.0])
        d = corner + sgn * np.array([0.0, 0.0, size])
        tet = [[a, c, b], [a, b, d], [a, d, c], [b, c, d]]
        tv = np.asarray(tet)
        cen = (a + b + c + d) / 4.0
        nrm = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
        outward = ((tv.mean(axis=1) - cen) * nrm).sum(axis=1)
        for t in range(4):
            if outward[t] < 0:
                tv[t, [1, 2]] = tv[t, [2, 1]]
        tris.append(tv)
    v = np.concatenate(tris)
    out = surf.concat(Surface(v, _unit_normals(v)))
    out.meta["anchors"] = (lo.tolist(), hi.tolist())
    return out


# ---------------------------------------------------------------------------
# benchmark / test workloads

def config_c1_cylinder(lattice=(24, 24, 104)) -> Surface:
    """Capped z-cylinder, r=10 lu, L=100 lu, 48 facets, centred in a
    24x24x104 lattice (spacing 1) through bbox anchors."""
    nx, ny, nz = lattice
    cx, cy = 0.5 * (nx - 1) + 0.137, 0.5 * (ny - 1) + 0.071
    z0 = 0.5 * (nz - 100.0) + 0.29
    s = capped_cylinder(10.0, 100.0, 48, center=(cx, cy), z0=z0)
    s = add_bbox_anchors(s, (0.0, 0.0, 0.0), (nx - 1.0, ny - 1.0, float(nz)))
    s.meta.update({"kind": "cylinder", "radius": 10.0, "center": (cx, cy), "z0": z0, "length": 100.0})
    return s


def config_c1_cylinder_x() -> Surface:
    """The C1 cylinder turned to lie along +x (coordinates cycled (x, y, z)
    -> (z, x, y), a rotation), so its inflow face is the x-min face on which
    the reference's velocity inlet formula acts (Boundary.cpp:129-157)."""
    s = config_c1_cylinder()
    v = s.v[:, :, [2, 0, 1]].copy()
    n = s.n[:, [2, 0, 1]].copy()
    cx, cy = s.meta["center"]
    meta = dict(s.meta)
    meta.update({"kind": "cylinder_x", "center": (cx, cy), "axis": "x"})
    return Surface(v, n, meta)


def config_c2_bifurcation(lattice=(256, 192, 512), seed: int = 0, h: float = 3.0) -> Surface:
    """Y-bifurcation (parent r=24 lu, daughters r=17 lu at +/-30 deg) inside a
    256x192x512 lattice (spacing 1).  Inlet cut at z=3.3, outlet cut at z=508.6;
    the split height keeps the daughters 6 lu inside the x extent."""
    nx, ny, nz = lattice
    cx, cy = 0.5 * (nx - 1) + 0.213, 0.5 * (ny - 1) + 0.087
    z_in, z_out = 3.3, nz - 3.4
    # daughters reach x = cx +/- (dz*tan30 + r_d/cos30): keep 6 lu of margin
    ang = math.radians(30.0)
    reach = 0.5 * (nx - 1) - 6.0 - 17.0 / math.cos(ang)
    z_split = z_out - reach / math.tan(ang)
    s = y_bifurcation(24.0, 17.0, 30.0, z_in=z_in, z_out=z_out, z_split=z_split, center=(cx, cy),
                      seed=seed, h=h)
    meta = dict(s.meta)
    s = add_bbox_anchors(s, (0.0, 0.0, 0.0), (nx - 1.0, ny - 1.0, float(nz)))
    s.meta = meta
    return s


def config_c4_ensemble(n: int = 64, seed: int = 0):
    """Seeded stenosed-tube ensemble members: radius U[8,20], length U[120,400],
    area severity U[0.2,0.7], eccentricity U[0,0.3], inlet mean U[0.01,0.04],
    period U[2000,6000] steps.  Returns a list of dicts (surface + parameters)."""
    rng = np.random.default_rng(seed)
    members = []
    for m in range(n):
        r = float(rng.uniform(8.0, 20.0))
        length = float(rng.uniform(120.0, 400.0))
        sev = float(rng.uniform(0.2, 0.7))
        ecc = float(rng.uniform(0.0, 0.3))
        mean = float(rng.uniform(0.01, 0.04))
        period = float(rng.uniform(2000.0, 6000.0))
        nxy = int(math.ceil(2 * r + 6))
        nz = int(math.ceil(length + 6))
        cx = 0.5 * (nxy - 1) + 0.173
        cy = 0.5 * (nxy - 1) + 0.061
        s = stenosed_tube(r, length, sev, ecc, center=(cx, cy), z0=2.7, seed=seed * 1000 + m,
                          h=max(1.5, r / 8.0))
        meta = dict(s.meta)
        s = add_bbox_anchors(s, (0.0, 0.0, 0.0), (nxy - 1.0, nxy - 1.0, float(nz)))
        s.meta = meta
        members.append({"surface": s, "radius": r, "length": length, "severity": sev,
                        "eccentricity": ecc, "inlet_mean": mean, "period": period,
                        "lattice": (nxy, nxy, nz), "center": (cx, cy)})
    return members
