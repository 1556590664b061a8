"""Batched ensemble: many vessels advanced by one lattice, one launch per step.

Members (each a closed surface along +z, e.g. the seeded stenosed tubes of
``geometry.config_c4_ensemble``) are voxelized one by one with the
reference's bbox rule, then packed side by side along x into one lattice,
with ``gap`` solid columns between neighbours so that no lattice link joins
two members.  The packed lattice is an ordinary handle of the C ABI: the step
kernel sweeps the active nodes of every member in one launch (uneven members
cost nothing extra: only active nodes are stored and updated), and a captured
CUDA graph replays many steps per call.

Per member the packing adds
  * a velocity inlet rule on the member's z-min fluid layer and a density
    outlet rule on its z-max fluid layer, both region rules restricted to the
    member's x/y box (so members of different lengths keep their own planes),
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
                 steady=False):
        """members: dicts with "surface" (geometry.Surface), "center" (tube axis
        x, y in surface coordinates), "radius", "inlet_mean", "period".
        steady: a constant inlet at each member's mean instead of its waveform."""
        self.members = members
        parts = []
        for m in members:
            tri = m["surface"].tri12()
            mask, vd = capi.voxelize(tri, 1.0)
            bb = np.array(vd.bbox[:])
            parts.append((tri, mask, np.array([bb[0], bb[2], bb[4]])))
        X = sum(p[1].shape[2] + gap for p in parts)
        Y = max(p[1].shape[1] for p in parts)
        Z = max(p[1].shape[0] for p in parts)
        packed = np.zeros((Z, Y, X), np.uint8)
        self.x0, self.x1, self.shift, self.tri = [], [], [], []
        bcs = []
        ox = 0
        for idx, ((tri, mask, org), m) in enumerate(zip(parts, members)):
            nz, ny, nx = mask.shape
            packed[:nz, :ny, ox:ox + nx] = mask
            # packed coordinates = member coordinates + shift (packed origin 0, spacing 1)
            shift = np.array([ox, 0.0, 0.0]) - org
            t = tri.copy()
            for c in range(3):
                t[:, c::3][:, :3] += shift[c]
            fl = np.argwhere(mask > 0)
            kin, kout = float(fl[:, 0].min()), float(fl[:, 0].max())
            xr = (ox - 0.5, ox + nx - 0.5)
            yr = (-0.5, ny - 0.5)
            cx, cy = m["center"][0] + shift[0], m["center"][1] + shift[1]
            bcs.append(capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", -1, 1.0, 1, cx, cy, m["radius"],
                                    region=(kin, 0.01, xr, yr), wave=idx))
            bcs.append(capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", -1, 1.0, region=(kout, 0.01, xr, yr)))
            self.x0.append(ox)
            self.x1.append(ox + nx)
            self.shift.append(shift)
            self.tri.append(t)
            ox += nx + gap
        self.mask = packed
        self.member_masks = [p[1] for p in parts]
        self.solver = capi.Solver(Q, precision, capi.LBM_PHYSICS, tau, 1.0, (0.0, 0.0, 0.0), 1.0, tawss_div, device)
        self.solver.set_geometry(packed, bcs)
        for idx, (t, m) in enumerate(zip(self.tri, members)):
            lo = (self.x0[idx] - 0.5, -1e30, -1e30)
            hi = (self.x1[idx] - 0.5, 1e30, 1e30)
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

    def member_of_x(self, i):
        """Member index of lattice column x = i (-1 in a gap)."""
        i = np.asarray(i)
        out = np.full(i.shape, -1, np.int64)
        for m, (a, b) in enumerate(zip(self.x0, self.x1)):
            out[(i >= a) & (i < b)] = m
        return out

    def macro(self):
        """rho, u per active node and the member of each node."""
        rho, u = self.solver.macro()
        fl = np.argwhere(self.mask > 0)
        return rho, u, self.member_of_x(fl[:, 2])

    def wss(self):
        w = self.solver.wss()
        nx = self.mask.shape[2]
        w["member"] = self.member_of_x(w["pt"] % nx)
        return w
