"""Batched ensemble: many vessels advanced by one lattice, one launch per step.

Members (each a closed surface along +z, e.g. the seeded stenosed tubes of
``geometry.config_c4_ensemble``) are voxelized one by one with the
reference's bbox rule, then stacked along z into one lattice, with ``gap``
solid layers between neighbours so that no lattice link joins two members.
Stacking along the slowest axis keeps every member's active nodes
contiguous in the lattice's active-node order, so a member's pull sources
lie as close in memory as in a lattice of its own.  The packed lattice is
an ordinary handle of the C ABI: the step kernel sweeps the active nodes of
every member in one launch (uneven members cost nothing extra: only active
nodes are stored and updated), and a captured CUDA graph replays many steps
per call.

Per member the packing adds
  * a velocity inlet rule on the member's z-min fluid layer and a density
    outlet rule on its z-max fluid layer (plane rules: no other member has
    fluid on those layers),
  * a parabolic inlet profile about the member's axis and its own inlet
    waveform (``lbm_set_waveform``),
  * next-to-wall normals from the member's own surface only
    (``lbm_set_normals_from_surface_box``).

The reference holds one vessel per run; this module has no counterpart there.
"""
from __future__ import annotations

import numpy as np

from . import capi
from . import waveform


class Ensemble:
    def __init__(self, members, Q=19, precision="f16", tau=0.55, gap=1, tawss_div=1.0, device=0, periods=None,
                 steady=False, collision=0):
        """members: dicts with "surface" (geometry.Surface), "center" (tube axis
        x, y in surface coordinates), "radius", "inlet_mean", "period".
        collision: capi.LBM_COLLISION_BGK or LBM_COLLISION_REGULARIZED.
        steady: a constant inlet at each member's mean instead of its waveform."""
        self.members = members
        parts = []
        for m in members:
            tri = m["surface"].tri12()
            mask, vd = capi.voxelize(tri, 1.0)
            bb = np.array(vd.bbox[:])
            parts.append((tri, mask, np.array([bb[0], bb[2], bb[4]])))
        X = max(p[1].shape[2] for p in parts)
        Y = max(p[1].shape[1] for p in parts)
        Z = sum(p[1].shape[0] + gap for p in parts)
        packed = np.zeros((Z, Y, X), np.uint8)
        self.z0, self.z1, self.shift, self.tri = [], [], [], []
        bcs = []
        oz = 0
        for idx, ((tri, mask, org), m) in enumerate(zip(parts, members)):
            nz, ny, nx = mask.shape
            packed[oz:oz + nz, :ny, :nx] = mask
            # packed coordinates = member coordinates + shift (packed origin 0, spacing 1)
            shift = np.array([0.0, 0.0, oz]) - org
            t = tri.copy()
            for c in range(3):
                t[:, c::3][:, :3] += shift[c]
            fl = np.argwhere(mask > 0)
            kin, kout = int(fl[:, 0].min()) + oz, int(fl[:, 0].max()) + oz
            cx, cy = m["center"][0] + shift[0], m["center"][1] + shift[1]
            bcs.append(capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, cx, cy, m["radius"], wave=idx))
            bcs.append(capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0))
            self.z0.append(oz)
            self.z1.append(oz + nz)
            self.shift.append(shift)
            self.tri.append(t)
            oz += nz + gap
        self.mask = packed
        self.member_masks = [p[1] for p in parts]
        self.solver = capi.Solver(Q, precision, capi.LBM_PHYSICS, tau, 1.0, (0.0, 0.0, 0.0), 1.0, tawss_div, device,
                                  collision=collision)
        self.solver.set_geometry(packed, bcs)
        for idx, (t, m) in enumerate(zip(self.tri, members)):
            lo = (-1e30, -1e30, self.z0[idx] - 0.5)
            hi = (1e30, 1e30, self.z1[idx] - 0.5)
            self.solver.set_normals_box(t, lo, hi)
            if steady:
                self.solver.set_waveform(idx, [m["inlet_mean"]])
            else:
                n = None if periods is None else int(round(periods * m["period"]))
                self.solver.set_waveform(idx, waveform.sinusoid_table(m["inlet_mean"], m["period"], n))
        self.counts = self.solver.counts()

    @property
    def active(self) -> int:
        return self.counts["active"]

    def step(self, n=1):
        self.solver.step(n)

    def step_async(self, n=1):
        self.solver.step_async(n)

    def member_mask(self, k):
        """Member k's own mask ([z][y][x], as voxelized alone)."""
        return self.member_masks[k]

    def member_of_z(self, k):
        """Member index of lattice layer z = k (-1 in a gap)."""
        k = np.asarray(k)
        out = np.full(k.shape, -1, np.int64)
        for m, (a, b) in enumerate(zip(self.z0, self.z1)):
            out[(k >= a) & (k < b)] = m
        return out

    def macro(self):
        """rho, u per active node and the member of each node."""
        rho, u = self.solver.macro()
        fl = np.argwhere(self.mask > 0)
        return rho, u, self.member_of_z(fl[:, 0])

    def wss(self):
        w = self.solver.wss()
        nxy = self.mask.shape[1] * self.mask.shape[2]
        w["member"] = self.member_of_z(w["pt"] // nxy)
        return w
