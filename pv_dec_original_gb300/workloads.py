"""The benchmark's named workloads, shared by bench.py and the tests.

* the Y-bifurcation (parent radius 24 lu, daughters radius 17 lu at +/-30
  deg, seed 0) in a 256x192x512 lattice, and the same vessel in a
  384x288x768 lattice for the storage-precision comparison;
* D3Q19 / D3Q27 physics mode, tau = 0.55, a parabolic Zou-He velocity inlet
  on the z-min fluid layer driven by u(t) = 0.03 (1 + 0.5 sin(2 pi t / 4000)
  + 0.2 sin(4 pi t / 4000)), a Zou-He density outlet rho = 1 on the z-max
  fluid layer, half-way bounce-back walls and wall shear stress on every
  next-to-wall node each step.

Geometry comes from the seeded generators of ``geometry``; nothing is read
from disk.
"""
from __future__ import annotations

import numpy as np

TAU = 0.55
U_MEAN = 0.03
PERIOD = 4000.0
C2_LATTICE = (256, 192, 512)
C3_LATTICE = (384, 288, 768)


def bifurcation(capi, lattice=C2_LATTICE):
    """(surface, triangles, mask, origin) of the bifurcation in `lattice`."""
    from . import geometry as G
    surf = G.config_c2_bifurcation(lattice=lattice)
    tri = surf.tri12()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    return surf, tri, mask, (bb[0], bb[2], bb[4])


def bifurcation_bcs(capi, surf, mask):
    """Velocity inlet on the lowest fluid layer along z, density outlet on
    the highest; returns (specs, (inlet plane, outlet plane))."""
    fl = np.argwhere(mask > 0)  # (k, j, i)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    cx, cy = surf.meta["center"]
    return [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, cx, cy, surf.meta["parent_radius"]),
            capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)], (kin, kout)


def bifurcation_solver(capi, mask, surf, tri, Q, prec, origin, device=0, collision=0):
    """A solver on the bifurcation with the benchmark's boundary rules,
    normals and inlet waveform; returns (solver, (inlet plane, outlet plane))."""
    from . import waveform
    s = capi.Solver(Q, prec, capi.LBM_PHYSICS, TAU, 1.0, origin, 1.0, PERIOD, device, collision=collision)
    bcs, planes = bifurcation_bcs(capi, surf, mask)
    s.set_geometry(mask, bcs)
    s.set_normals(tri)
    s.set_inlet_table(waveform.sinusoid_table(U_MEAN, PERIOD))
    return s, planes


def pressure_drop(rho, mask, planes):
    """Mean density on the inlet layer minus the outlet layer, over 3."""
    fl = np.argwhere(mask > 0)
    kin, kout = planes
    return (rho[fl[:, 0] == kin].mean() - rho[fl[:, 0] == kout].mean()) / 3.0


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
