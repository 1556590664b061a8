"""Generate the golden fixtures from the reference's own C++ (compiled unchanged).

Run in a checkout that has the reference sources (the directory given by
--ref, else $LBM_REFERENCE_DIR, else the REF default of oracle/Makefile):

    python tests/golden/make_golden.py [--ref DIR]

It builds ``oracle/_ref/ref_harness`` (see oracle/Makefile), generates the
input geometries with the package's generators, runs the reference's
voxelizer / solver / waveform through the harness, and stores inputs and
outputs as ``tests/golden/*.npz``.  Triangles are stored verbatim, so the
fixtures do not depend on the platform's libm.  Large arrays are stored as
SHA-256 digests of their little-endian bytes plus a strided sample.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from pv_dec_original_gb300 import geometry as G  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def geometries():
    """name -> (tri12, spacing)"""
    g = {}
    g["c1_cylinder"] = (G.config_c1_cylinder().tri12(), 1.0)
    g["c1x_cylinder"] = (G.config_c1_cylinder_x().tri12(), 1.0)
    g["elbow_z"] = (G.elbow(radius=5.0, leg=22.0, h=1.6, seed=1, exit="z-").tri12(), 1.0)
    g["elbow_y"] = (G.elbow(radius=5.0, leg=22.0, h=1.6, seed=2, exit="y+").tri12(), 1.0)
    bif = G.y_bifurcation(6.0, 4.25, 30.0, z_in=1.3, z_out=60.6, z_split=38.0, center=(16.2, 10.1), seed=0, h=1.5)
    g["bifurcation_small"] = (bif.tri12(), 1.0)
    return g


def write_stl_rows(path, tri12):
    s = G.Surface(tri12[:, :9].reshape(-1, 3, 3).copy(), tri12[:, 9:].copy())
    G.write_stl_ascii(path, s)


def classify(mask, rules, Q=19):
    """Plane rules as the harness applies them: first match wins, rest wall."""
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


def vox_fixture(name, tri, spacing, tmp):
    stl = os.path.join(tmp, name + ".stl")
    write_stl_rows(stl, tri)
    ref = O.run_reference_vox(stl, spacing, os.path.join(tmp, name + ".vox"))
    # the harness reads the STL text: its triangles must be the stored ones
    assert np.array_equal(G.read_stl_ascii(stl), tri)
    np.savez_compressed(
        os.path.join(OUT, f"vox_{name}.npz"), tri12=tri, spacing=spacing, dims=np.array(ref["dims"]),
        bbox=ref["bbox"], mask_bits=np.packbits(ref["mask"].reshape(-1)), nfluid=int(ref["mask"].sum()),
        boundary_ijk_sha=sha(ref["boundary_ijk"].astype(np.int32)), nboundary=len(ref["boundary_ijk"]),
        ref_seconds=ref["seconds"])
    print(f"vox_{name}: dims={ref['dims']} fluid={int(ref['mask'].sum())} boundary={len(ref['boundary_ijk'])}")
    return ref


# (rules as (harness key, axis, plane)), profile (c1, c2, R) or None
SIMS = {
    # x-min inlet (uniform, ramped amplitude) and z-min outlet (outlet 2)
    "elbow_z": dict(rules=[("inlet", 0, None, "min"), ("outlet2", 2, None, "min")], profile=None,
                    tau=0.8, dt=1e-4, nsteps=60, amp=lambda s: 0.02 + 0.0005 * s),
    # x-min inlet with a parabolic profile and y-max outlet (outlet 1)
    "elbow_y": dict(rules=[("inlet", 0, None, "min"), ("outlet1", 1, None, "max")], profile="auto",
                    tau=0.7, dt=8e-6, nsteps=80, amp=lambda s: 0.04),
    # the C1 cylinder along x: parabolic x-min inlet (u_max 0.05), tau 0.8;
    # the reference has no x-max outlet formula, so the far end is wall
    # (the run covers the inflow transient: 200 steps, before the pressure
    # wave returns from the closed end)
    "c1x_cylinder": dict(rules=[("inlet", 0, None, "min")], profile="auto", tau=0.8, dt=1e-4, nsteps=200,
                         amp=lambda s: 0.05),
}


def sim_fixture(name, tri, spacing, tmp):
    cfg = SIMS[name]
    mask, bb, dims = O.voxelize(tri, spacing)
    nz, ny, nx = mask.shape
    fl = np.argwhere(mask.transpose(2, 1, 0) > 0)  # (i, j, k)
    rules, rule_txt = [], []
    for key, axis, plane, side in cfg["rules"]:
        if plane is None:
            plane = int(fl[:, axis].min() if side == "min" else fl[:, axis].max())
        rules.append((axis, plane))
        rule_txt.append(f"{key} {'xyz'[axis]} {plane}")
    prof = None
    if cfg["profile"] == "auto":
        # inlet on x-min: centre and radius from the inlet plane's fluid points
        pts = fl[fl[:, 0] == rules[0][1]]
        y = bb[2] + pts[:, 1] * spacing
        z = bb[4] + pts[:, 2] * spacing
        prof = (float(0.5 * (y.min() + y.max())), float(0.5 * (z.min() + z.max())),
                float(0.5 * max(y.max() - y.min(), z.max() - z.min()) + 0.5))
    amps = np.array([cfg["amp"](s) for s in range(cfg["nsteps"])], np.float64)
    stl = os.path.join(tmp, name + "_sim.stl")
    write_stl_rows(stl, tri)
    bc_txt = os.path.join(tmp, name + ".bc")
    with open(bc_txt, "w") as f:
        f.write("\n".join(rule_txt) + "\n")
        if prof:
            f.write(f"profile 1 {prof[0]!r} {prof[1]!r} {prof[2]!r}\n")
    inlet_txt = os.path.join(tmp, name + ".inlet")
    with open(inlet_txt, "w") as f:
        f.write("\n".join(repr(float(a)) for a in amps) + "\n")
    ref = O.run_reference_sim(stl, spacing, bc_txt, cfg["tau"], cfg["dt"], cfg["nsteps"], inlet_txt,
                              os.path.join(tmp, name + ".sim"))
    act = ref["active"]
    lin = act["ijk"][:, 2].astype(np.int64) * nx * ny + act["ijk"][:, 1] * nx + act["ijk"][:, 0]
    act = act[np.argsort(lin)]
    lin = np.sort(lin)
    nw = ref["nw"]
    nlin = nw["ijk"][:, 2].astype(np.int64) * nx * ny + nw["ijk"][:, 1] * nx + nw["ijk"][:, 0]
    nw = nw[np.argsort(nlin)]
    nlin = np.sort(nlin)
    tmap = {0: 1, 1: 3, 2: 3, 3: 3, 4: 3, 5: 2}
    # class per active node in this library's numbering: 1 fluid, 2 wall, 3+b bc b
    kinds = {"inlet": 1, "outlet1": 2, "outlet2": 3, "outlet3": 4}
    order = [kinds[k] for k, *_ in cfg["rules"]]
    cls = np.array([1 if t == 0 else 2 if t == 5 else 3 + order.index(t) for t in act["type"]], np.uint8)
    sample = slice(0, None, 13)
    np.savez_compressed(
        os.path.join(OUT, f"sim_{name}.npz"), tri12=tri, spacing=spacing, dims=np.array([nx, ny, nz]), bbox=bb,
        rules=np.array(rules, np.int64), rule_keys=np.array([k for k, *_ in cfg["rules"]]),
        profile=np.array(prof if prof else (0.0, 0.0, 1.0)), has_profile=prof is not None, tau=cfg["tau"],
        dt=cfg["dt"], nsteps=cfg["nsteps"], amp=amps, active_pt=lin, active_cls=cls,
        f_sha=sha(act["f"]), fnew_sha=sha(act["fnew"]), feq_sha=sha(act["feq"]), rho_sha=sha(act["rho"]),
        u_sha=sha(act["u"]), f_sample=act["f"][sample], f_sample_idx=np.arange(len(act))[sample],
        rho=act["rho"], u=act["u"], nw_pt=nlin, nw_normal=nw["normal"], nw_wss=nw["wss"], nw_acc=nw["acc"],
        nw_acc_mag=nw["acc_mag"], nw_osi=nw["osi"], nw_tawss=nw["tawss"], ref_step_seconds=ref["step_s"])
    print(f"sim_{name}: active={len(act)} nw={len(nw)} rules={rule_txt} profile={prof} "
          f"{ref['step_s']:.2f}s for {cfg['nsteps']} steps")
    return ref


def pulse_fixture(tmp):
    out = os.path.join(tmp, "pulse.bin")
    import subprocess
    subprocess.run([O.REF_HARNESS, "pulse", repr(8e-6), "120000", out], check=True, stdout=subprocess.DEVNULL)
    tv = np.fromfile(out, np.float64).reshape(-1, 2)
    sel = np.concatenate([np.arange(0, len(tv), 997), [len(tv) - 1]])
    np.savez_compressed(os.path.join(OUT, "pulse.npz"), dt=8e-6, n=len(tv), idx=sel, t=tv[sel, 0], v=tv[sel, 1],
                        v_sha=sha(tv[:, 1]))
    print(f"pulse: {len(tv)} steps")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=O.reference_dir())
    ap.add_argument("--only", nargs="*", default=None,
                    help="fixture names to (re)generate, e.g. sim_c1x_cylinder vox_c1_cylinder pulse")
    a = ap.parse_args()
    if not O.build_reference(a.ref):
        sys.exit(f"reference sources not found at {a.ref}")
    want = (lambda name: True) if a.only is None else (lambda name: name in a.only)
    with tempfile.TemporaryDirectory() as tmp:
        geos = geometries()
        for name, (tri, sp) in geos.items():
            if want("vox_" + name) and name != "c1x_cylinder":
                vox_fixture(name, tri, sp, tmp)
        for name in SIMS:
            if want("sim_" + name):
                sim_fixture(name, geos[name][0], geos[name][1], tmp)
        if want("pulse"):
            pulse_fixture(tmp)


if __name__ == "__main__":
    main()
