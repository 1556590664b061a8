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


def voxelize_members(members):
    """Each member voxelized alone with the reference's bbox rule:
    (triangles as tri12 rows, mask [z][y][x], lattice origin x, y, z)."""
    parts = []
    for m in members:
        tri = m["surface"].tri12()
        mask, vd = capi.voxelize(tri, 1.0)
        bb = np.array(vd.bbox[:])
        parts.append((tri, mask, np.array([bb[0], bb[2], bb[4]])))
    return parts


def split_balanced(sizes, groups):
    """Cut the list of member sizes into at most `groups` contiguous runs of
    about equal total size: run k ends at the member whose cumulative size
    lies nearest to (k + 1) / groups of the total.  Returns (first, end)
    pairs covering every member once, none empty."""
    sizes = [max(0, int(s)) for s in sizes]
    n = len(sizes)
    groups = max(1, min(int(groups), n))
    cum = np.cumsum(sizes, dtype=np.float64)
    total = cum[-1] if n else 0.0
    cuts, start = [], 0
    for k in range(groups - 1):
        target = total * (k + 1) / groups
        # leave at least one member for each later run
        hi = n - (groups - 1 - k)
        end = int(np.searchsorted(cum, target, side="left")) + 1
        if end > start + 1 and abs(cum[end - 2] - target) <= abs(cum[end - 1] - target):
            end -= 1
        end = min(max(end, start + 1), hi)
        cuts.append((start, end))
        start = end
    cuts.append((start, n))
    return cuts


class Ensemble:
    def __init__(self, members, Q=19, precision="f16", tau=0.55, gap=1, tawss_div=1.0, device=0, periods=None,
                 steady=False, collision=0, parts=None):
        """members: dicts with "surface" (geometry.Surface), "center" (tube axis
        x, y in surface coordinates), "radius", "inlet_mean", "period".
        collision: capi.LBM_COLLISION_BGK or LBM_COLLISION_REGULARIZED.
        steady: a constant inlet at each member's mean instead of its waveform.
        parts: the members' voxelizations (voxelize_members), if already made."""
        self.members = members
        parts = voxelize_members(members) if parts is None else parts
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

    def close(self):
        self.solver.close()


class GroupedEnsemble:
    """The members packed into `groups` lattices instead of one: contiguous
    runs of the member list of about equal fluid-node counts, each an
    Ensemble (one handle, its own stream and captured graph), all advanced
    concurrently.

    One packed lattice advances step by step: every launch waits for the
    whole previous step, so each step ends in a drain where the last blocks
    run alone.  Independent lattices on their own streams fill each other's
    drains (64 seeded stenosed tubes, FP16: 4 or 8 groups ran 1.04-1.05x
    one packed lattice).  Advancing the groups one after another instead, so
    that a group's populations could stay in L2 across its steps, gained
    nothing (groups of 2 to 16 members: 0.91-1.01x one packed lattice).

    Member k of the ensemble is member k - first[g] of group g; macro() and
    wss() return the members in order, as one packed Ensemble would."""

    def __init__(self, members, groups=4, Q=19, precision="f16", tau=0.55, **kw):
        parts = voxelize_members(members)
        cuts = split_balanced([int(np.count_nonzero(p[1])) for p in parts], groups)
        self.members = members
        self.first = [a for a, _ in cuts]
        self.groups = [Ensemble(members[a:b], Q, precision, tau, parts=parts[a:b], **kw) for a, b in cuts]

    @property
    def active(self) -> int:
        return sum(e.active for e in self.groups)

    def solvers(self):
        return [e.solver for e in self.groups]

    def autotune(self, trial_steps=5):
        return [e.solver.autotune(trial_steps)[0] for e in self.groups]

    def set_graph_steps(self, n):
        for e in self.groups:
            e.solver.set_graph_steps(n)

    def step_async(self, n=1):
        """Issue n steps of every group, each on its own stream."""
        for e in self.groups:
            e.step_async(n)

    def sync(self):
        for e in self.groups:
            e.solver.sync()

    def step(self, n=1):
        self.step_async(n)
        self.sync()
        self.check_status()

    def check_status(self):
        for e in self.groups:
            e.solver.check_status()

    def launches(self) -> int:
        return sum(e.solver.launches() for e in self.groups)

    def macro(self):
        """rho, u per active node (groups in member order) and the member of each node."""
        out = [e.macro() for e in self.groups]
        return (np.concatenate([o[0] for o in out]), np.concatenate([o[1] for o in out]),
                np.concatenate([o[2] + f for o, f in zip(out, self.first)]))

    def wss(self):
        ws = [e.wss() for e in self.groups]
        out = {k: np.concatenate([w[k] for w in ws]) for k in ws[0] if k not in ("pt", "member")}
        out["member"] = np.concatenate([w["member"] + f for w, f in zip(ws, self.first)])
        return out

    def conservation(self):
        """Mass, momentum and per-rule flux, rules in member order (inlet, outlet per member)."""
        cs = [e.solver.conservation() for e in self.groups]
        return sum(c[0] for c in cs), sum(c[1] for c in cs), np.concatenate([c[2] for c in cs])

    def close(self):
        for e in self.groups:
            e.close()


def main(argv=None):
    """python -m pv_dec_original_gb300.ensemble [--members N] [--steps K]
    [--precision f16] [--groups G] [--variant V]: build the seeded C4
    ensemble (geometry.config_c4_ensemble, seed 0), advance it K steps (one
    launch per step, no graph) and print its active nodes and the host-clock
    MLUPS of those steps.  --variant fixes the launch shape (lbm_set_variant)
    instead of the default one."""
    import argparse
    import time

    from . import geometry as G
    ap = argparse.ArgumentParser(prog="python -m pv_dec_original_gb300.ensemble")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--precision", default="f16", choices=["f32", "f16", "bf16"])
    ap.add_argument("--groups", type=int, default=1)
    ap.add_argument("--variant", type=int, default=None)
    ap.add_argument("--tau", type=float, default=0.55)
    a = ap.parse_args(argv)
    members = G.config_c4_ensemble(a.members, seed=0)
    ens = GroupedEnsemble(members, a.groups, 19, a.precision, a.tau)
    if a.variant is not None:
        for s in ens.solvers():
            s.set_variant(a.variant)
    ens.sync()
    t0 = time.perf_counter()
    ens.step(a.steps)
    dt = time.perf_counter() - t0
    print(f"members {a.members} groups {len(ens.groups)} active {ens.active} steps {a.steps} "
          f"host-clock MLUPS {ens.active * a.steps / dt / 1e6:.0f} launches {ens.launches()}")
    ens.close()


if __name__ == "__main__":
    main()
