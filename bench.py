"""Benchmark: lattice-Boltzmann step throughput (MLUPS) and HBM bandwidth.

Workload (default): the 256x192x512 Y-bifurcation (parent r=24 lu, daughters
r=17 lu at +/-30 deg, seed 0), D3Q19 BGK, FP32 storage, tau=0.55, parabolic
pulsatile velocity inlet u(t)=0.03(1+0.5 sin(2 pi t/4000)+0.2 sin(4 pi t/4000))
on the z-min face, density outlet rho=1 on the z-max face, half-way
bounce-back walls, wall shear stress on every next-to-wall node each step.

One bench "step" is one LBM time step over the whole lattice.  Each timed
step is bracketed by CUDA events on the solver's own stream, and the L2 is
flushed between timed steps, outside the events: a 512 MB device write, then
a 256 MB device read, so that the step starts with an L2 of clean unrelated
lines (the read evicts the write's dirty lines, whose write-back would
otherwise land inside the next timed step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --gpus N > 1 (launched by torchrun) every rank advances an independent
replica of the lattice (the single-domain solver has no inter-GPU exchange);
value = total lattice updates of all ranks / max rank time.
--impl reference times the CPU oracle (the reference's algorithm restated in
C, FP64, parity semantics) on this host's cores, each of its K steps a
bounded sample of full-lattice steps.

At N = 1 the line's "extra" object adds secondary measurements (skipped by
--quick or their --no-* flags): FP16 storage, D3Q27, the voxelizer's ray
tests per second, the reference's own PV.stl case (752x583x472, its
inlet / outlet windows and polynomial pulse), the 384x288x768 precision
comparison against an FP64 run, three inlet periods of the bifurcation
(with an FP64 run from a one-ulp-perturbed start as the yardstick), the
64-vessel packed ensemble, the learned warm start, and (with
--small-ensembles) launch-bound lattices stepped one launch per step vs
persistent launches.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_LU = {(19, "f32"): 152, (19, "f16"): 76, (19, "bf16"): 76, (19, "f64"): 304,
                (27, "f32"): 216, (27, "f16"): 108, (27, "bf16"): 108, (27, "f64"): 432}
L2_FLUSH_BYTES = 512 << 20
L2_READ_BYTES = 256 << 20
E2E_BATCHES = 20  # timed end-to-end batches of 100 steps (2000 LBM steps), whatever --steps is
TAU = 0.55
U_MEAN = 0.03
PERIOD = 4000.0


# --------------------------------------------------------------------------- cudart via ctypes

class Cudart:
    def __init__(self):
        self.L = C.CDLL("libcudart.so.13")
        for name in ("cudaEventCreate", "cudaEventRecord", "cudaEventSynchronize", "cudaEventElapsedTime",
                     "cudaEventDestroy", "cudaMalloc", "cudaFree", "cudaMemsetAsync", "cudaHostAlloc",
                     "cudaFreeHost", "cudaStreamSynchronize", "cudaSetDevice", "cudaGetDeviceProperties",
                     "cudaStreamWaitEvent"):
            getattr(self.L, name).restype = C.c_int

    def ck(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: cuda error {rc}")

    def event(self):
        e = C.c_void_p()
        self.ck(self.L.cudaEventCreate(C.byref(e)), "cudaEventCreate")
        return e

    def record(self, e, stream):
        self.ck(self.L.cudaEventRecord(e, C.c_void_p(stream)), "cudaEventRecord")

    def wait(self, stream, e):
        self.ck(self.L.cudaStreamWaitEvent(C.c_void_p(stream), e, 0), "cudaStreamWaitEvent")

    def elapsed_ms(self, a, b):
        self.ck(self.L.cudaEventSynchronize(b), "cudaEventSynchronize")
        ms = C.c_float()
        self.ck(self.L.cudaEventElapsedTime(C.byref(ms), a, b), "cudaEventElapsedTime")
        return ms.value

    def malloc(self, n):
        p = C.c_void_p()
        self.ck(self.L.cudaMalloc(C.byref(p), C.c_size_t(n)), "cudaMalloc")
        return p

    def memset_async(self, p, v, n, stream):
        self.ck(self.L.cudaMemsetAsync(p, C.c_int(v), C.c_size_t(n), C.c_void_p(stream)), "cudaMemsetAsync")

    def host_alloc(self, n):
        p = C.c_void_p()
        self.ck(self.L.cudaHostAlloc(C.byref(p), C.c_size_t(n), C.c_uint(0)), "cudaHostAlloc")
        return p


def pinned_array(cr, n, dtype):
    p = cr.host_alloc(max(1, n) * np.dtype(dtype).itemsize)
    buf = (C.c_char * (max(1, n) * np.dtype(dtype).itemsize)).from_address(p.value)
    return np.frombuffer(buf, dtype=dtype, count=n), p


# --------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- workload

def c2_workload():
    from pv_dec_original_gb300 import geometry as G
    surf = G.config_c2_bifurcation()
    return surf, surf.tri12()


def make_solver(capi, mask, surf, tri, Q, prec, origin, device, collision=0):
    from pv_dec_original_gb300 import workloads as W
    return W.bifurcation_solver(capi, mask, surf, tri, Q, prec, origin, device, collision)


class L2Flush:
    """Write L2_FLUSH_BYTES, then read L2_READ_BYTES, on a given stream."""

    def __init__(self, device):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.w = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=self.dev)
        self.r = torch.ones(L2_READ_BYTES // 4, dtype=torch.float32, device=self.dev)
        self.sink = None

    def __call__(self, stream):
        ext = self.torch.cuda.ExternalStream(stream, device=self.dev)
        with self.torch.cuda.stream(ext):
            self.w.zero_()
            self.sink = self.r.sum()


def time_steps(cr, s, steps, flush, stream):
    """Per-step event timing with an L2 flush between steps (outside events)."""
    evs = [(cr.event(), cr.event()) for _ in range(steps)]
    for a, b in evs:
        flush(stream)
        cr.record(a, stream)
        s.step_async(1)
        cr.record(b, stream)
    ms = [cr.elapsed_ms(a, b) for a, b in evs]
    s.check_status()
    for a, b in evs:
        cr.L.cudaEventDestroy(a)
        cr.L.cudaEventDestroy(b)
    return ms


def d3q27_extra(capi, cr, mask, surf, tri, origin, device, flush, steps):
    """D3Q27 on the same bifurcation: FP32 and FP16 storage, per-step CUDA
    events with the L2 flushed between steps (as the headline)."""
    out = {}
    for prec in ("f32", "f16"):
        s, _ = make_solver(capi, mask, surf, tri, 27, prec, origin, device)
        s.step(5)
        best, _ = s.autotune(5)
        ms = time_steps(cr, s, steps, flush, s.stream())
        m = sum(ms) / len(ms)
        act = s.counts()["active"]
        out[prec] = {"mlups": act / (m * 1e-3) / 1e6, "ms_per_step": m, "variant": best,
                     "hbm_gbs": act * BYTES_PER_LU[(27, prec)] / (m * 1e-3) / 1e9}
        s.close()
    return out


def precision_extra(capi, cr, device, steps=1200, timed=200):
    """The precision configuration: the bifurcation (parent r=24, daughters
    r=17) in a 384x288x768 lattice, D3Q19 BGK physics, pulsatile inlet;
    FP32, FP16-scaled and BF16 offset storage against an FP64 run of the same
    case on the GPU after `steps` steps (BGK at tau=0.55 stays stable for
    about 2000 steps on this lattice, FP64 included): velocity L2 relative
    error, relative error of the pressure drop (mean density on the inlet
    plane minus the outlet plane, over 3), TAWSS L2 relative error; MLUPS of
    each format (events around `timed` graph-replayed steps; the populations
    exceed L2)."""
    from pv_dec_original_gb300 import geometry as G
    surf = G.config_c2_bifurcation(lattice=(384, 288, 768))
    tri = surf.tri12()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    origin = (bb[0], bb[2], bb[4])
    fl = np.argwhere(mask > 0)
    res = {}
    ref = None
    for prec in ("f64", "f32", "f16", "bf16"):
        s, (kin, kout) = make_solver(capi, mask, surf, tri, 19, prec, origin, device)
        if prec != "f64":
            s.autotune(3)
        s.set_graph_steps(100)
        s.step(steps)
        rho, u = s.macro()
        tawss = s.wss()["tawss"]
        drop = (rho[fl[:, 0] == kin].mean() - rho[fl[:, 0] == kout].mean()) / 3.0
        st = s.stream()
        a, b = cr.event(), cr.event()
        cr.record(a, st)
        s.step_async(timed)
        cr.record(b, st)
        ms = cr.elapsed_ms(a, b) / timed
        s.check_status()
        act = s.counts()["active"]
        row = {"mlups": act / (ms * 1e-3) / 1e6, "ms_per_step": ms,
               "hbm_gbs": act * BYTES_PER_LU[(19, prec)] / (ms * 1e-3) / 1e9}
        if ref is None:
            ref = (u, drop, tawss)
        else:
            row["u_l2_rel"] = float(np.linalg.norm(u - ref[0]) / np.linalg.norm(ref[0]))
            row["pressure_drop_rel"] = float(abs(drop - ref[1]) / abs(ref[1]))
            row["tawss_l2_rel"] = float(np.linalg.norm(tawss - ref[2]) / np.linalg.norm(ref[2]))
        res[prec] = row
        s.close()
    for prec in ("f16", "bf16"):
        res[prec]["speedup_vs_f32"] = res[prec]["mlups"] / res["f32"]["mlups"]
    return {"lattice": [384, 288, 768], "active_nodes": int(len(fl)), "steps": steps, "tau": TAU,
            "reference": "FP64 run of the same case on the GPU (physics mode)", "formats": res}


def periods_extra(capi, mask, surf, tri, origin, device, periods=3):
    """C2 over three inlet periods (12,000 steps): FP32, FP16 and BF16
    storage against an FP64 run of the same case on the GPU, regularized
    collision (BGK diverges near step 2200 at tau = 0.55 on this lattice):
    velocity and pressure-drop errors at the end, and the TAWSS (time
    average over the three periods) error."""
    fl = np.argwhere(mask > 0)
    steps = int(periods * PERIOD)
    res, ref = {}, None
    # "f64_1ulp": FP64 from an initial state moved by one ulp per value
    # (random sign, seeded): the flow's own amplification of a rounding-size
    # difference, the yardstick of the other formats' errors
    for name in ("f64", "f64_1ulp", "f32", "f16", "bf16"):
        prec = "f64" if name.startswith("f64") else name
        t0 = time.perf_counter()
        s, (kin, kout) = make_solver(capi, mask, surf, tri, 19, prec, origin, device,
                                     collision=capi.LBM_COLLISION_REGULARIZED)
        if name == "f64_1ulp":
            f0 = s.distributions()
            rng = np.random.default_rng(7)
            s.set_distributions(np.where(rng.random(f0.shape) < 0.5, np.nextafter(f0, -np.inf),
                                         np.nextafter(f0, np.inf)))
        s.set_graph_steps(100)
        s.step(steps)
        rho, u = s.macro()
        tawss = s.wss()["tawss"]
        drop = (rho[fl[:, 0] == kin].mean() - rho[fl[:, 0] == kout].mean()) / 3.0
        row = {"seconds": time.perf_counter() - t0}
        if ref is None:
            ref = (u, drop, tawss)
        else:
            row["u_l2_rel"] = float(np.linalg.norm(u - ref[0]) / np.linalg.norm(ref[0]))
            row["pressure_drop_rel"] = float(abs(drop - ref[1]) / abs(ref[1]))
            row["tawss_l2_rel"] = float(np.linalg.norm(tawss - ref[2]) / np.linalg.norm(ref[2]))
        res[name] = row
        s.close()
    return {"lattice": [256, 192, 512], "steps": steps, "periods": periods, "tau": TAU,
            "collision": "regularized", "reference": "FP64 run of the same case on the GPU",
            "f64_1ulp": "FP64 started from the initial state moved by one ulp per value (random sign)",
            "formats": res}


def pv_extra(capi, cr, device, flush, steps=20):
    """The reference's own workload: PV.stl (11,670 triangles; the surface
    stored in tests/golden/pv_stl.npz) at spacing 0.05 -> a 752x583x472
    lattice, the reference's PV inlet / outlet windows (ComplexGeometry.cpp:
    1378-1408) with its formulas' faces, tau = 1.5 (LBM.cpp:62), the
    polynomial pulse of Pulsatile at dt = 8e-6 (pulsatile.h:14-28,
    Simulation.cpp:548-563), half-way bounce-back walls, D3Q19 physics mode.
    Voxelizer time, then per-step CUDA events with the L2 flushed between
    steps (as the headline) for FP32 and FP16 storage."""
    from pv_dec_original_gb300 import waveform
    d = np.load(os.path.join(ROOT, "tests", "golden", "pv_stl.npz"))
    tri = np.ascontiguousarray(np.concatenate([d["verts"][d["faces"]].reshape(-1, 9), d["normals"]], axis=1))
    sp = float(d["spacing"])
    t0 = time.perf_counter()
    mask, desc = capi.voxelize(tri, sp)
    vox_s = time.perf_counter() - t0
    bb = np.array(desc.bbox[:])
    org = (bb[0], bb[2], bb[4])
    windows = [(capi.LBM_BC_REF_INLET, "x-", -16.9538, (-191.0, -187.0), (-118.0, -114.0)),
               (capi.LBM_BC_REF_OUTLET_YMAX, "y+", -170.016, (2.0, 5.0), (-109.0, -106.0)),
               (capi.LBM_BC_REF_OUTLET_ZMIN, "z-", -110.0, (-27.0, -25.0), (-198.0, -195.0)),
               (capi.LBM_BC_REF_OUTLET_ZMIN, "z-", -123.0, (-33.0, -30.0), (-189.0, -186.0))]
    rules = [capi.bc_spec(k, f, -1, 1.0, region=(c, 1e-2, t1, t2)) for k, f, c, t1, t2 in windows]
    table = waveform.reference_table(8e-6, 20000)
    out = {"lattice": [int(v) for v in d["dims"]], "triangles": int(len(tri)), "voxelize_s": vox_s,
           "fluid_points": int(mask.sum())}
    for prec in ("f32", "f16"):
        t0 = time.perf_counter()
        s = capi.Solver(19, prec, capi.LBM_PHYSICS, 1.5, sp, org, 1.0, 0.9, device)
        s.set_geometry(mask, rules)
        s.set_normals(tri)
        s.set_inlet_table(table)
        setup_s = time.perf_counter() - t0
        s.step(5)
        best, _ = s.autotune(5)
        ms = time_steps(cr, s, steps, flush, s.stream())
        m = sum(ms) / len(ms)
        act = s.counts()["active"]
        gbs = act * BYTES_PER_LU[(19, prec)] / (m * 1e-3) / 1e9
        out[prec] = {"active_nodes": act, "mlups": act / (m * 1e-3) / 1e6, "ms_per_step": m, "hbm_gbs": gbs,
                     "frac_of_measured_hbm": gbs / read_peaks()[0], "variant": best, "setup_s": setup_s,
                     "bc_nodes": s.counts()["bc"]}
        s.close()
    out["f16"]["speedup_vs_f32"] = out["f16"]["mlups"] / out["f32"]["mlups"]
    return out


def concurrent_ms(cr, solvers, steps):
    """Device time of `steps` steps of every handle, each on its own stream,
    issued together: the first handle's stream forks to the others by an
    event and joins them back by one event each; CUDA events around the
    fork and the join."""
    s0 = solvers[0].stream()
    fork, end = cr.event(), cr.event()
    done = [cr.event() for _ in solvers]
    cr.record(fork, s0)
    for s in solvers[1:]:
        cr.wait(s.stream(), fork)
    for s, d in zip(solvers, done):
        s.step_async(steps)
        cr.record(d, s.stream())
    for d in done[1:]:
        cr.wait(s0, d)
    cr.record(end, s0)
    ms = cr.elapsed_ms(fork, end)
    for e in done + [fork, end]:
        cr.L.cudaEventDestroy(e)
    for s in solvers:
        s.check_status()
    return ms


def chained_ms(cr, solvers, steps):
    """Device time of `steps` steps of every handle one handle after another:
    each handle's steps wait on an event recorded after the previous
    handle's, so one runs at a time, with no host synchronisation between."""
    done = [cr.event() for _ in solvers]
    fork = cr.event()
    cr.record(fork, solvers[0].stream())
    for i, s in enumerate(solvers):
        if i:
            cr.wait(s.stream(), done[i - 1])
        s.step_async(steps)
        cr.record(done[i], s.stream())
    ms = cr.elapsed_ms(fork, done[-1])
    for e in done + [fork]:
        cr.L.cudaEventDestroy(e)
    for s in solvers:
        s.check_status()
    return ms


def ensemble_extra(capi, cr, device, Q, nmem=64, steps=64, groups=4):
    """Aggregate MLUPS of the C4 ensemble (64 seeded stenosed tubes, FP16
    storage): packed into one lattice (captured graph, one step-kernel
    launch per step); packed into `groups` lattices of about equal size
    advanced concurrently (GroupedEnsemble); and the members as 64 separate
    lattices, advanced concurrently (each its own stream and graph) and one
    after another (the plain solver in a loop).  Every arm: 32-step graphs,
    64 warm-up steps, CUDA events around `steps` steps.  The members'
    populations (about 1 GB) exceed the L2, so consecutive steps are timed
    without a flush."""
    from pv_dec_original_gb300 import geometry as G
    from pv_dec_original_gb300 import waveform
    from pv_dec_original_gb300.ensemble import Ensemble, GroupedEnsemble
    members = G.config_c4_ensemble(nmem, seed=0)
    t0 = time.perf_counter()
    ens = Ensemble(members, Q, "f16", TAU, device=device)
    setup_s = time.perf_counter() - t0
    ens.solver.autotune(5)
    ens.solver.set_graph_steps(32)
    st = ens.solver.stream()
    ens.step(64)
    a, b = cr.event(), cr.event()
    cr.record(a, st)
    ens.step_async(steps)
    cr.record(b, st)
    ms = cr.elapsed_ms(a, b)
    for e in (a, b):
        cr.L.cudaEventDestroy(e)
    ens.solver.check_status()
    active = ens.active
    packed = active * steps / (ms * 1e-3) / 1e6
    launches = ens.solver.launches()
    ens.solver.close()
    # packed into groups advanced concurrently
    grp = GroupedEnsemble(members, groups, Q, "f16", TAU, device=device)
    grp.autotune(5)
    grp.set_graph_steps(32)
    grp.step(64)
    g_ms = concurrent_ms(cr, grp.solvers(), steps)
    grouped = grp.active * steps / (g_ms * 1e-3) / 1e6
    g_sizes = [e.active for e in grp.groups]
    launches += grp.launches()
    grp.close()
    # the same members as separate lattices
    singles = []
    for m in members:
        tri = m["surface"].tri12()
        mask, vd = capi.voxelize(tri, 1.0)
        bb = np.array(vd.bbox[:])
        fl = np.argwhere(mask > 0)
        kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
        s = capi.Solver(Q, "f16", capi.LBM_PHYSICS, TAU, 1.0, (bb[0], bb[2], bb[4]), 1.0, 1.0, device)
        s.set_geometry(mask, [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, m["center"][0], m["center"][1],
                                           m["radius"]), capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)])
        s.set_normals(tri)
        s.set_inlet_table(waveform.sinusoid_table(m["inlet_mean"], m["period"]))
        s.set_graph_steps(32)
        s.step(64)
        singles.append(s)
    for s in singles:
        s.sync()
    assert sum(s.counts()["active"] for s in singles) == active
    looped = active * steps / (concurrent_ms(cr, singles, steps) * 1e-3) / 1e6
    serial = active * steps / (chained_ms(cr, singles, steps) * 1e-3) / 1e6
    launches += sum(s.launches() for s in singles)
    for s in singles:
        s.close()
    return {"members": nmem, "active_nodes": active, "storage": "f16", "steps": steps,
            "packed_mlups": packed, "packed_ms_per_step": ms / steps,
            "packed_hbm_gbs": active * BYTES_PER_LU[(Q, "f16")] / (ms / steps * 1e-3) / 1e9,
            "grouped_mlups": grouped, "groups": len(g_sizes), "group_active_nodes": g_sizes,
            "looped_mlups": looped, "looped_one_at_a_time_mlups": serial,
            "speedup_vs_looped": grouped / looped, "packed_vs_looped": packed / looped,
            "grouped_vs_packed": grouped / packed, "speedup_vs_one_at_a_time": grouped / serial,
            "setup_s": setup_s,
            "timing": "CUDA events; one lattice: around %d graph-replayed steps on its stream; %d groups and "
                      "looped: the lattices on their own streams, forked from and joined to one stream by "
                      "events; one at a time: the lattices chained by events" % (steps, len(g_sizes)),
            "l2": "not flushed (populations exceed L2)", "launches_total": launches}


def voxelizer_extra(capi, tri, spacing=1.0, repeats=3):
    """The +z ray-parity voxelizer on the bifurcation's STL: ray-triangle
    tests per second (each test: 13 FP64 adds / multiplies and one FP64
    division for the plane crossing; the in-triangle test runs only for
    crossings), host wall clock around lbm_voxelize (triangle upload, column
    binning, ray kernel, mask copy back), best of `repeats` after one
    warm-up call."""
    capi.voxelize(tri, spacing)
    best, desc = None, None
    for _ in range(repeats):
        t0 = time.perf_counter()
        _, desc = capi.voxelize(tri, spacing)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    tests = int(desc.ray_tests)
    fp64_nominal = 1.25e12  # GB300 FP64 FLOP/s, nominal (no measured FP64 peak is recorded)
    return {"lattice": list(desc.dims), "triangles": int(len(tri)), "points": int(np.prod(list(desc.dims))),
            "fluid_points": int(desc.fluid_count), "ray_tests": tests, "seconds": best,
            "tests_per_s": tests / best, "fp64_flop_per_test": 14,
            "fp64_frac_of_nominal": tests * 14 / best / fp64_nominal,
            "timing": "host wall clock around lbm_voxelize, best of %d after a warm-up call" % repeats}


def small_ensembles_extra(cr, device, sizes=(1, 4, 16, 64), steps=3000):
    """Launch-bound lattices: 1-64 seeded vessels (32x32x64 boxes, about 6k
    active nodes each) packed into one lattice, graph-replayed (96 steps a
    graph) with one step-kernel launch per step against persistent launches
    (lbm_set_persistent, 32 steps a launch, grid barrier between steps).
    CUDA events around `steps` steps after 200 warm-up steps; the lattices
    fit in L2 (no flush: this measures launch and barrier cost)."""
    from pv_dec_original_gb300 import warmstart as WS
    from pv_dec_original_gb300.ensemble import Ensemble
    rows = []
    for n in sizes:
        members = WS.vessel_members(n, seed=5)
        for prec in ("f32", "f16"):
            us = {}
            for persist in (0, 32):
                e = Ensemble(members, 19, prec, 0.6, device=device, steady=True, collision=1)
                e.solver.set_persistent(persist)
                e.solver.set_graph_steps(96)
                st = e.solver.stream()
                e.step(200)
                a, b = cr.event(), cr.event()
                cr.record(a, st)
                e.step_async(steps)
                cr.record(b, st)
                us[persist] = cr.elapsed_ms(a, b) * 1e3 / steps
                e.solver.check_status()
                nact = e.active
                e.solver.close()
            rows.append({"members": n, "storage": prec, "active_nodes": nact, "flat_us_per_step": us[0],
                         "persistent_us_per_step": us[32], "flat_mlups": nact / us[0],
                         "persistent_mlups": nact / us[32]})
    return {"rows": rows, "timing": f"CUDA events around {steps} steps; L2 not flushed (lattices fit in L2)"}


def warmstart_extra(device, box=(64, 64, 128), n_train=32, n_test=6, tau=0.55, radius=(2.0, 5.0),
                    train_iters=2000, conv=True):
    """Learned warm start under pulsatile inlets: seeded stenosed tubes and
    bifurcations in a D x H x W box (defaults: 128 x 64 x 64, tube radii
    4-10 lattice units, 32 training and 6 held-out vessels; the full C5 case
    is --warmstart-c5: 256 x 128 x 128, radii 8-20, 200 and 32), each with
    its own waveform u(s) = mean (1 + 0.5 sin(2 pi s/T) + 0.2 sin(4 pi s/T)),
    mean 0.01-0.04, T 2000-6000 steps.  Training targets: each training
    vessel's converged periodic state at phase 0 (its own lattice run from
    rest, period by period, until the cycle-to-cycle WSS change is below
    1e-3).  On every held-out vessel, three FP32 lattices (regularized
    collision: BGK diverges at tau = 0.55 here) start from rest (cold, as
    the reference does), from the Poiseuille prior alone and from the
    network's prediction, each run to its converged periodic state; the
    figure is the first step from which the WSS stays within 1% of the cold
    run's converged cycle at the same phase, and wall time = prediction time
    (all on the device) + steps x the lattice's measured time per step."""
    import torch
    from pv_dec_original_gb300 import capi
    from pv_dec_original_gb300 import warmstart as WS
    rlb = capi.LBM_COLLISION_REGULARIZED
    t0 = time.perf_counter()
    train_m = WS.vessel_members(n_train, seed=1, box=box, radius=radius)
    test_m = WS.vessel_members(n_test, seed=99, box=box, radius=radius)
    sols = WS.periodic_solutions(train_m, tau=tau, device=device, collision=rlb)
    samples = [WS.make_sample(mask, dict(m, period=T), rho, u, tau=tau, device=device)
               for (mask, rho, u, T, _, _), m in zip(sols, train_m)]
    periods = [k for (_, _, _, _, k, _) in sols]
    data_s = time.perf_counter() - t0
    net = WS.WarmStartNet(sols[0][0].shape, device=device, seed=0)
    t0 = time.perf_counter()
    hist = WS.train(net, samples, iters=train_iters, lr=2e-3, batch=4)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    # the network's forward pass is captured once for the grid size and
    # replayed for every vessel (capture outside the timed regions)
    net.forward_graphed(samples[0][0])
    torch.cuda.synchronize()
    del samples
    rows = [WS.periodic_arms(net, m, tau=tau, device=device, collision=rlb) for m in test_m]
    ok = [r for r in rows if all(r[k]["steps_1pct_wss"] is not None for k in ("cold", "prior", "net"))]
    tot = lambda arm, k: sum(r[arm][k] for r in ok)
    ratio = lambda a, b, k: (tot(a, k) / tot(b, k)) if ok and tot(b, k) > 0 else None
    out = {"grid": list(sols[0][0].shape), "train_vessels": n_train, "test_vessels": n_test, "tau": tau,
           "tube_radius_lu": [radius[0] * box[0] / 32.0, radius[1] * box[0] / 32.0],
           "inlet": "per vessel u(s) = mean (1 + 0.5 sin(2 pi s/T) + 0.2 sin(4 pi s/T)), mean 0.01-0.04, "
                    "T 2000-6000 steps",
           "training_targets": "converged periodic state at phase 0 (cycle-to-cycle WSS change < 1e-3)",
           "training_periods_run": [min(periods), max(periods)],
           "data_s": data_s, "train_s": train_s, "train_iters": train_iters, "loss_first_last": [hist[0], hist[-1]],
           "criterion": "FP32 lattice WSS within 1% of the cold run's converged periodic WSS at the same phase "
                        "(checked every 100 steps) from that step on; time = prediction (features, network "
                        "forward replayed from a CUDA graph captured once for the grid size, prior, smoothing, "
                        "state build) + steps x measured FP32 time per step",
           "vessels_reaching_1pct": {k: sum(r[k]["steps_1pct_wss"] is not None for r in rows)
                                     for k in ("cold", "prior", "net")},
           "net_over_cold_time": ratio("net", "cold", "s_1pct_wss"),
           "prior_over_cold_time": ratio("prior", "cold", "s_1pct_wss"),
           "net_over_cold_steps": ratio("net", "cold", "steps_1pct_wss"),
           "prior_over_cold_steps": ratio("prior", "cold", "steps_1pct_wss"),
           "per_vessel": rows}
    if conv:
        out["conv_forward_c5_grid"] = conv_forward_c5(device)
    return out


def conv_forward_c5(device, dims=(256, 128, 128), reps=5):
    """One forward pass of the warm-start network at the C5 grid (128 x 128
    x 256 voxels, random BF16 input), CUDA events around `reps` passes after
    a warm-up pass, on each convolution engine: tcgen05 (3x3x3 layers on the
    fifth-generation tensor cores, the 1x1 layer on mma.sync) and mma.sync
    everywhere; per layer, the tcgen05 engine's time of one convolution
    launch (10 launches timed); and one training step of one sample
    (forward, masked MSE, backward with the weight gradients, Adam) on each
    engine."""
    import ctypes as C
    import torch
    from pv_dec_original_gb300 import capi
    from pv_dec_original_gb300 import warmstart as WS
    L = capi.load()
    dev = torch.device("cuda", device)
    big = WS.WarmStartNet(dims, device=device, seed=0)
    nvox = dims[0] * dims[1] * dims[2]
    g = torch.Generator(device=dev).manual_seed(0)
    xb = (torch.rand(nvox * WS.C_IN, device=dev, generator=g) - 0.5).to(torch.bfloat16)
    flops = sum(2.0 * big.nvox(mm["lvl_out"]) * mm["co"] * mm["taps"] * mm["ci"] for mm in big.meta.values())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = {"grid": list(dims), "gflop": flops / 1e9}
    outputs = {}
    try:
        for name, engine in (("mma_sync", capi.LBM_NN_ENGINE_MMA_SYNC), ("tcgen05", capi.LBM_NN_ENGINE_AUTO)):
            capi._check(L.lbm_nn_set_conv_engine(engine))
            big.forward(xb)
            torch.cuda.synchronize(dev)
            outputs[name] = big.y32.clone()
            ev[0].record(big.stream)
            for _ in range(reps):
                big.forward(xb)
            ev[1].record(big.stream)
            torch.cuda.synchronize(dev)
            ms = ev[0].elapsed_time(ev[1]) / reps
            out[name] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12}
        layers = {}
        y = torch.empty(nvox * 64, dtype=torch.bfloat16, device=dev)
        for name, m in big.meta.items():
            src = m["src"]
            xin = big.up[name] if src.startswith("up:") else (xb if src == "x" else big.act[src])
            w = big.wb[m["w_off"]:m["w_off"] + m["w_n"]]
            b = big.b[m["b_off"]:m["b_off"] + m["co"]]
            gi = big.grid(m["lvl_in"])
            args = (C.c_void_p(xin.data_ptr()), (C.c_int * 3)(*gi), m["ci"], C.c_void_p(w.data_ptr()),
                    C.c_void_p(b.data_ptr()), m["co"], m["ks"], m["stride"], m["relu"], C.c_void_p(y.data_ptr()),
                    None, big.st)
            capi._check(L.lbm_nn_conv3d_fwd(*args))
            ev[0].record(big.stream)
            for _ in range(10):
                L.lbm_nn_conv3d_fwd(*args)
            ev[1].record(big.stream)
            torch.cuda.synchronize(dev)
            ms = ev[0].elapsed_time(ev[1]) / 10
            fl = 2.0 * big.nvox(m["lvl_out"]) * m["co"] * m["taps"] * m["ci"]
            go = [v // m["stride"] for v in gi]
            tc = m["ks"] == 3 and all(v % d == 0 for v, d in zip(go, (4 if m["stride"] == 1 else 1, 16, 8)))
            layers[name] = {"grid": list(gi), "ci": m["ci"], "co": m["co"], "k": m["ks"], "stride": m["stride"],
                            "engine": "tcgen05" if tc else "mma.sync", "us": ms * 1e3,
                            "tflops": fl / (ms * 1e-3) / 1e12}
        out["layers_tcgen05_engine"] = layers
        # one training step (forward, masked MSE, backward, Adam) of one
        # sample on each engine
        tgt = torch.rand(nvox * 4, device=dev, generator=g)
        msk = torch.ones(nvox, dtype=torch.uint8, device=dev)
        for name, engine in (("mma_sync", capi.LBM_NN_ENGINE_MMA_SYNC), ("tcgen05", capi.LBM_NN_ENGINE_AUTO)):
            capi._check(L.lbm_nn_set_conv_engine(engine))

            def train_step():
                big.zero_grad()
                y32 = big.forward(xb)
                big.backward(big.loss_and_grad(y32, tgt, msk, 1.0 / (4 * nvox)))
                big.adam(1e-4)

            train_step()
            torch.cuda.synchronize(dev)
            ev[0].record(big.stream)
            for _ in range(reps):
                train_step()
            ev[1].record(big.stream)
            torch.cuda.synchronize(dev)
            out[name]["train_step_ms"] = ev[0].elapsed_time(ev[1]) / reps
    finally:
        L.lbm_nn_set_conv_engine(capi.LBM_NN_ENGINE_AUTO)
    capi._check(L.lbm_nn_conv_status())
    a, b = outputs["tcgen05"], outputs["mma_sync"]
    out["engines_output_max_rel_diff"] = float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))
    out["ms"] = out["tcgen05"]["ms"]
    out["tflops"] = out["tcgen05"]["tflops"]
    out["speedup_vs_mma_sync"] = out["mma_sync"]["ms"] / out["tcgen05"]["ms"]
    out["kernel"] = ("3x3x3 layers (stride 1 and 2): tcgen05.mma kind::f16 (BF16 x BF16 -> FP32 in tensor "
                     "memory); the 1x1 output layer: mma.sync m16n8k16 BF16 implicit GEMM, FP32 accumulate")
    return out


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_traffic(name, variant):
    """DRAM bytes per launch (read + write, one ncu capture) of the step
    kernel the launch variant runs -- the compact kernel for variants 6 and
    7, the flat kernel otherwise -- from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    key = "traffic_bytes_per_launch[%s]" % ("compact" if variant in (6, 7) else "flat")
    for line in open(p):
        if line.startswith(key):
            try:
                return float(line.split("=", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def cpu_sim(mask, bb, planes, mode=None):
    """The CPU oracle (FP64, the reference's algorithm) on the C2 lattice
    with the GPU arm's boundary rules; mode None: physics semantics (the GPU
    arm's: half-way bounce-back, stress of the same time level), else the
    oracle's PARITY / PHYSICS constant."""
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import classify
    from pv_dec_original_gb300 import waveform
    kin, kout = planes
    cls = classify(mask, [(2, kin), (2, kout)])
    surf_c = (0.5 * 255 + 0.213, 0.5 * 191 + 0.087)
    bcs = [dict(kind=O.BC_VELOCITY, face=4, plane=kin, value=1.0, profile=1, c1=surf_c[0], c2=surf_c[1], R=24.0),
           dict(kind=O.BC_PRESSURE, face=5, plane=kout, value=1.0)]
    sim = O.Sim(19, O.PHYSICS if mode is None else mode, cls, (bb[0], bb[2], bb[4]), 1.0, TAU, bcs)
    sim.set_amplitude(waveform.sinusoid_table(U_MEAN, PERIOD))
    return sim


def cpu_sample(sim, cores, seconds, max_steps=200):
    """As many full-lattice steps as fit in ~seconds (at least one):
    (steps, seconds)."""
    n, t0 = 0, time.perf_counter()
    while True:
        sim.step(1, cores)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= max_steps:
            return n, el


def cpu_baseline(tri, mask, bb, planes, cores, seconds=12.0, mode=None):
    """The CPU oracle (FP64) on this host: as many C2 steps as fit in ~seconds."""
    sim = cpu_sim(mask, bb, planes, mode)
    sim.step(1, cores)  # warm-up (page-in)
    n, el = cpu_sample(sim, cores, seconds)
    return sim.nactive * n / el / 1e6, n, el, sim.nactive


# --------------------------------------------------------------------------- arms

def dist_setup(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group(backend=backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


def max_over_ranks(dist, x, backend_device=None):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=backend_device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mlups(ws, units_per_rank, steps, seconds_max):
    """Whole-job MLUPS: every rank advances its own replica (units_per_rank
    active nodes, `steps` steps); the slowest rank's time counts."""
    return ws * units_per_rank * steps / seconds_max / 1e6


def run_ours(args):
    ws, rank, local, dist = dist_setup("nccl")
    from pv_dec_original_gb300 import capi
    capi.load(build_if_missing=True)
    cr = Cudart()
    cr.ck(cr.L.cudaSetDevice(local), "cudaSetDevice")
    dev_t = None
    if dist is not None:
        import torch
        torch.cuda.set_device(local)
        dev_t = torch.device("cuda", local)

    surf, tri = c2_workload()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    origin = (bb[0], bb[2], bb[4])
    s, planes = make_solver(capi, mask, surf, tri, args.Q, args.precision, origin, local)
    cnt = s.counts()
    active = cnt["active"]
    stream = s.stream()
    flush = L2Flush(local)

    s.step(args.warmup)
    if args.variant is not None:
        s.set_variant(args.variant)
        tuned = (args.variant, [])
    else:
        tuned = s.autotune(10) if not args.no_tune else (0, [])
    if dist is not None:
        dist.barrier()
    cr.ck(cr.L.cudaStreamSynchronize(C.c_void_p(stream)), "sync")
    launches0 = s.launches()
    with ClockSampler(local) as clk:
        ms = time_steps(cr, s, args.steps, flush, stream)
    launches = s.launches() - launches0
    cr.ck(cr.L.cudaStreamSynchronize(C.c_void_p(stream)), "sync")
    total_ms = sum(ms)
    total_ms_max = max_over_ranks(dist, total_ms, dev_t)
    mean_ms = total_ms / len(ms)
    value = aggregate_mlups(ws, active, args.steps, total_ms_max * 1e-3)
    bpl = BYTES_PER_LU[(args.Q, args.precision)]
    peak, peak_kind = read_peaks()
    achieved = active * bpl / (mean_ms * 1e-3) / 1e9
    traffic = read_traffic(f"step_kernel_c2_q{args.Q}_{args.precision}.txt", tuned[0])

    # secondary: FP16-offset storage on the same lattice (the precision config's storage)
    extra = {}
    # the secondary measurements run at N = 1 only (a multi-GPU run reports
    # the replicated headline)
    extras = ws == 1 and not args.quick
    if args.precision == "f32" and extras:
        s16, _ = make_solver(capi, mask, surf, tri, args.Q, "f16", origin, local)
        s16.step(args.warmup)
        if args.variant is not None:
            s16.set_variant(args.variant)
        elif not args.no_tune:
            s16.autotune(10)
        ms16 = time_steps(cr, s16, args.steps, flush, s16.stream())
        m16 = sum(ms16) / len(ms16)
        extra["f16_store"] = {"mlups": active / (m16 * 1e-3) / 1e6,
                              "hbm_gbs": active * BYTES_PER_LU[(args.Q, "f16")] / (m16 * 1e-3) / 1e9,
                              "ms_per_step": m16, "speedup_vs_f32": mean_ms / m16}
        s16.close()

    # batched ensemble (64 seeded stenosed tubes, FP16 storage): one packed
    # lattice, one launch per step, vs the same members as 64 lattices
    if extras:
        try:
            extra["voxelizer"] = voxelizer_extra(capi, tri)
        except Exception as e:  # a measurement, not the benchmark: record why it is missing
            extra["voxelizer"] = {"error": str(e)}
    if extras and args.Q == 19:
        extra["d3q27"] = d3q27_extra(capi, cr, mask, surf, tri, origin, local, flush, args.steps)
    if extras:
        try:
            extra["pv_case"] = pv_extra(capi, cr, local, flush)
        except Exception as e:  # a measurement, not the benchmark: record why it is missing
            extra["pv_case"] = {"error": str(e)}
    if extras and not args.no_precision:
        extra["precision_c3"] = precision_extra(capi, cr, local)
        extra["c2_three_periods"] = periods_extra(capi, mask, surf, tri, origin, local)
    if extras and not args.no_ensemble:
        extra["ensemble_c4"] = ensemble_extra(capi, cr, local, args.Q)
    if extras and not args.no_warmstart:
        extra["warmstart_c5"] = dict(warmstart_extra(local),
                                     scale="C5 scaled down (128x64x64 grids, 32 + 6 vessels); the full C5 case: "
                                           "bench.py --warmstart-c5")
    if ws == 1 and args.small_ensembles:
        extra["small_ensembles"] = small_ensembles_extra(cr, local)

    # end to end through the C ABI: per e2e step, H2D of a 100-step inlet
    # table slice from pinned memory, 100 LBM steps (graph replay), D2H of
    # the wall shear stress arrays and the rho/u field (the reference's
    # output cadence, Simulation.cpp:589-591).  The read-outs are the
    # asynchronous calls: their copies run on the handle's copy stream while
    # the next batch steps; the timed region ends when the last copies land.
    from pv_dec_original_gb300 import waveform
    B = 100
    table = waveform.sinusoid_table(U_MEAN, PERIOD, 4000)
    amp_h, _ = pinned_array(cr, B, np.float64)
    nnw = cnt["next_to_wall"]
    wss_h = [pinned_array(cr, n, np.float64)[0] for n in (nnw, 3 * nnw, nnw, 3 * nnw, nnw, nnw, nnw)]
    pt_h, _ = pinned_array(cr, nnw, np.int64)
    rho_h, _ = pinned_array(cr, active, np.float64)
    u_h, _ = pinned_array(cr, 3 * active, np.float64)
    s.set_graph_steps(B)
    L = capi.load()
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    nb = E2E_BATCHES

    def e2e_batch(k):
        s0 = k * B + s_base
        idx = np.arange(s0, s0 + B)
        amp_h[idx % B] = table[idx % len(table)]  # step s reads amp[s % B]
        capi._check(L.lbm_set_inlet_table(s.h, amp_h, B), s.h)
        capi._check(L.lbm_step_async(s.h, B), s.h)
        capi._check(L.lbm_get_wss_async(s.h, P(pt_h), P(wss_h[1]), P(wss_h[0]), P(wss_h[3]), P(wss_h[2]),
                                        P(wss_h[4]), P(wss_h[5])), s.h)
        capi._check(L.lbm_get_macro_async(s.h, P(rho_h), P(u_h)), s.h)

    s_base = s.counts()["steps"]
    e2e_batch(0)  # captures the graph, allocates the staging buffers
    capi._check(L.lbm_wait_outputs(s.h), s.h)
    capi._check(L.lbm_check_status(s.h), s.h)
    t0 = time.perf_counter()
    for k in range(1, nb + 1):
        e2e_batch(k)
    capi._check(L.lbm_wait_outputs(s.h), s.h)
    e2e_times = [(time.perf_counter() - t0) / nb]
    capi._check(L.lbm_check_status(s.h), s.h)
    e2e_t = max_over_ranks(dist, sum(e2e_times) / len(e2e_times), dev_t)
    h2d = B * 8
    d2h = nnw * 8 * (1 + 3 + 1 + 3 + 1 + 1 + 1) + active * 8 * 4

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            try:
                cores = os.cpu_count() or 1
                v, n, el, na = cpu_baseline(tri, mask, bb, planes, cores, seconds=args.cpu_seconds)
                cpu = {"value": v, "unit": "MLUPS", "cores": cores, "kind": "port",
                       "sample": f"{n} FP64 steps of the full 256x192x512 lattice ({na} active nodes) in the "
                                 f"GPU arm's semantics (physics mode, same boundary rules), {el:.1f} s, OpenMP on "
                                 f"{cores} host threads, normals not computed"}
            except Exception as e:  # the baseline is reported, never required
                cpu = {"value": None, "unit": "MLUPS", "cores": 0, "kind": "port", "sample": f"failed: {e}"}
        out = {
            "metric": "MLUPS (D3Q19 BGK lattice updates per second, active nodes)",
            "value": value, "unit": "MLUPS", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "f32" else args.precision,
            "data": "synthetic (seeded Y-bifurcation STL generated in-process)",
            "config": {"workload": "Y-bifurcation 256x192x512, parent r=24, daughters r=17 at +/-30 deg, seed 0",
                       "lattice": f"D3Q{args.Q}", "storage": args.precision, "tau": TAU,
                       "inlet": "z-min Zou-He velocity, parabolic, u=0.03(1+0.5sin(2pi t/4000)+0.2sin(4pi t/4000))",
                       "outlet": "z-max Zou-He density 1", "walls": "half-way bounce-back",
                       "active_nodes": active, "lattice_points": cnt["points"],
                       "boundary_list_nodes": cnt["special"], "next_to_wall": nnw,
                       "l2": "flushed between timed steps, outside the events: 512 MB write then 256 MB read",
                       "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "bytes_per_lu": bpl, "peak_source": peak_kind,
                         "kernel": (f"lbm::step_compact_kernel<{args.Q}, {args.precision}>" if tuned[0] in (6, 7)
                                    else f"lbm::step_kernel<{args.Q}, {args.precision}, physics, step>"),
                         "launch_variant": tuned[0]},
            "cpu_baseline": cpu,
            "e2e": {"value": aggregate_mlups(ws, active, B, e2e_t), "unit": "MLUPS", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "step": f"{B} LBM steps per call batch + WSS/OSI/TAWSS and rho/u read-back (pinned host buffers; "
                            "the read-back copies of one batch overlap the next batch's steps)"},
            "gpu_launches": launches,
            "autotune": {"variant": tuned[0], "ms_per_step_by_variant": tuned[1],
                         "variants": "(block, min blocks/SM): (128,12) (128,10) (128,8) (256,3) (256,1); 5: tiled bulk-copy kernel"},
            "clocks": clk.summary(),
            "extra": extra,
        }
        print(json.dumps(out))
    s.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return out


def run_reference(args):
    ws, rank, local, dist = dist_setup("gloo")
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None
    from oracle import oracle as O
    O.build()
    from pv_dec_original_gb300 import geometry as G
    surf, tri = c2_workload()
    mask, bb, d = O.voxelize(tri, 1.0, culled=True)
    fl = np.argwhere(mask > 0)
    planes = (int(fl[:, 0].min()), int(fl[:, 0].max()))
    cores = os.cpu_count() or 1
    # one lattice; each of the W warm-up and K timed "steps" is a bounded
    # sample of full-lattice LBM steps, sized so that the K samples take
    # about --cpu-seconds together.  The timed semantics are the GPU arm's
    # (physics mode: half-way bounce-back, stress of the same time level,
    # the same Zou-He rules); the reference's own semantics (parity mode:
    # push streaming, its wall rule, time-lagged stress) are timed after it
    # as a second, labelled number.
    per_sample = max(0.05, args.cpu_seconds / args.steps)

    def timed(mode, samples):
        sim = cpu_sim(mask, bb, planes, mode)
        for _ in range(args.warmup):
            cpu_sample(sim, cores, per_sample, max_steps=1)
        tn, tt = 0, 0.0
        for _ in range(samples):
            n, el = cpu_sample(sim, cores, per_sample)
            tn += n
            tt += el
        return sim.nactive, tn, tt

    na, total_n, total_t = timed(O.PHYSICS, args.steps)
    value = na * total_n / total_t / 1e6
    _, pn, pt = timed(O.PARITY, max(1, args.steps // 4))
    out = {
        "impl": "reference", "metric": "MLUPS (D3Q19 BGK lattice updates per second, active nodes)",
        "value": value, "unit": "MLUPS", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Y-bifurcation STL generated in-process)",
        "config": {"workload": "Y-bifurcation 256x192x512, parent r=24, daughters r=17 at +/-30 deg, seed 0",
                   "lattice": "D3Q19", "storage": "f64", "tau": TAU,
                   "inlet": "z-min Zou-He velocity, parabolic, u=0.03(1+0.5sin(2pi t/4000)+0.2sin(4pi t/4000))",
                   "outlet": "z-max Zou-He density 1", "walls": "half-way bounce-back",
                   "active_nodes": na,
                   "implementation": "reference algorithm restated in C (oracle/lbm_oracle.c), physics semantics "
                                     "(the GPU arm's)",
                   "step": f"one bounded sample of full-lattice LBM steps (~{per_sample:.2f} s)",
                   "lbm_steps_timed": total_n, "ms_per_lbm_step": 1e3 * total_t / total_n},
        "parity_semantics": {"value": na * pn / pt / 1e6, "unit": "MLUPS", "lbm_steps_timed": pn,
                             "seconds": pt,
                             "what": "the same lattice in the reference's own semantics (push streaming, its "
                                     "in-place wall rule, time-lagged stress), FP64, same threads"},
        "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"{total_n} full-lattice FP64 steps in {total_t:.1f} s on {cores} threads, "
                                   f"{args.steps} samples"},
        "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "f16", "bf16", "f64"])
    ap.add_argument("--Q", type=int, default=19, choices=[19, 27])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the secondary FP16 and ensemble measurements")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble measurement")
    ap.add_argument("--no-precision", action="store_true", help="skip the 384x288x768 precision measurement")
    ap.add_argument("--no-warmstart", action="store_true", help="skip the learned warm-start measurement")
    ap.add_argument("--small-ensembles", action="store_true",
                    help="add the launch-bound small-ensemble measurement (flat vs persistent launches)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--variant", type=int, default=None, help="force a launch shape (skips the autotuner)")
    ap.add_argument("--conv-only", nargs=3, type=int, default=None, metavar=("D", "H", "W"),
                    help="only the warm-start network's forward pass on a D x H x W grid (both convolution "
                         "engines, per-layer times); prints its JSON")
    ap.add_argument("--warmstart-c5", action="store_true",
                    help="only the learned warm start at the full C5 case (256x128x128 grids, 200 training and 32 "
                         "held-out vessels, pulsatile inlets); prints its JSON (about 10-20 minutes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.conv_only:
        from pv_dec_original_gb300 import capi
        capi.load(build_if_missing=True)
        print(json.dumps(conv_forward_c5(0, tuple(args.conv_only))))
    elif args.warmstart_c5:
        from pv_dec_original_gb300 import capi
        capi.load(build_if_missing=True)
        print(json.dumps(warmstart_extra(0, box=(128, 128, 256), n_train=200, n_test=32, radius=(2.0, 5.0))))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
