"""GPU solver parity: FP64 parity mode vs the reference (bit-exact
distributions), every precision / lattice / mode vs the FP64 oracle."""
import numpy as np
import pytest

from helpers import classify, fixtures, load, sha, sim_bcs, wss_C

pytestmark = pytest.mark.gpu


def _gpu_parity_run(capi, d, precision, graph=0, split=None):
    mask, desc = capi.voxelize(d["tri12"], float(d["spacing"]))
    bb = np.array(desc.bbox[:])
    s = capi.Solver(19, precision, capi.LBM_PARITY, float(d["tau"]), float(d["spacing"]), (bb[0], bb[2], bb[4]),
                    wss_C(float(d["dt"]), float(d["spacing"])), 0.9)
    s.set_geometry(mask, [capi.bc_spec(**spec) for _, spec in sim_bcs(d)])
    s.set_normals(d["tri12"])
    s.set_inlet_table(d["amp"])
    if graph:
        s.set_graph_steps(graph)
    n = int(d["nsteps"])
    if split:
        s.step(split)
        s.step(n - split)
    else:
        s.step(n)
    return s, mask


@pytest.mark.parametrize("path", fixtures("sim"), ids=lambda p: p.split("/")[-1])
def test_gpu_fp64_parity_bit_exact_vs_reference(gpu_lib, path):
    d = load(path)
    s, mask = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    cls = s.classes().reshape(-1)
    act = np.flatnonzero(cls)
    assert np.array_equal(act, d["active_pt"])
    assert np.array_equal(cls[act] & 0x7F, d["active_cls"])
    f = s.distributions()
    ref_sample = d["f_sample"]
    got_sample = f[d["f_sample_idx"]]
    assert np.max(np.abs(got_sample - ref_sample)) <= 1e-13, "FP64 parity drifted from the reference"
    assert sha(f) == str(d["f_sha"]), "distributions are close but not bit-identical to the reference"
    # rho / u of the post-boundary distributions (the reference's node->density
    # is from the collision before the last stream, so compare with f itself)
    rho, u = s.macro()
    np.testing.assert_allclose(rho, f.sum(axis=1), rtol=1e-14)
    w = s.wss()
    assert np.array_equal(w["pt"], d["nw_pt"])
    np.testing.assert_allclose(w["normal"], d["nw_normal"], rtol=1e-13, atol=1e-15)
    for k in ("wss", "acc", "acc_mag", "tawss"):
        np.testing.assert_allclose(w[k], d["nw_" + k], rtol=1e-11, atol=1e-13 * np.abs(d["nw_" + k]).max())
    np.testing.assert_allclose(w["osi"], d["nw_osi"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("path", fixtures("sim"), ids=lambda p: p.split("/")[-1])
def test_gpu_parity_graph_and_split_calls_identical(gpu_lib, path):
    d = load(path)
    a, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    b, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, graph=4, split=7)
    assert np.array_equal(a.distributions(), b.distributions())
    assert np.array_equal(a.wss()["acc"], b.wss()["acc"])


@pytest.mark.parametrize("path", fixtures("sim"), ids=lambda p: p.split("/")[-1])
@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f16", 5e-3), ("bf16", 3e-2)])
def test_gpu_low_precision_parity_vs_fp64(gpu_lib, path, prec, tol):
    """Parity semantics in each storage format against the FP64 run of the
    same golden case: velocity L2 relative error within the stated
    tolerance (1e-5 for FP32)."""
    d = load(path)
    ref, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    got, _ = _gpu_parity_run(gpu_lib, d, prec)
    r_rho, r_u = ref.macro()
    g_rho, g_u = got.macro()
    rel = np.linalg.norm(g_u - r_u) / np.linalg.norm(r_u)
    assert rel <= tol, rel
    assert np.max(np.abs(g_rho - r_rho)) <= 10 * tol


def _physics_case(capi, oracle, Q, precision, nsteps=40, tau=0.7, collision=0, walls=False):
    """A stenosed tube with velocity inlet (z-min) and pressure outlet (z-max);
    walls=True: interpolated bounce-back with the surface's wall distances."""
    from pv_dec_original_gb300 import geometry as G
    surf = G.stenosed_tube(5.0, 40.0, 0.5, 0.2, center=(7.3, 7.1), z0=1.6, h=1.4, seed=3)
    surf = G.add_bbox_anchors(surf, (0.0, 0.0, 0.0), (14.0, 14.0, 44.0))
    tri = surf.tri12()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    org = (bb[0], bb[2], bb[4])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    bcs = [dict(kind=capi.LBM_BC_VELOCITY, face=4, plane=kin, value=1.0, profile=1, c1=7.3, c2=7.1, R=5.0),
           dict(kind=capi.LBM_BC_PRESSURE, face=5, plane=kout, value=1.0)]
    amp = 0.03 * (1 + 0.5 * np.sin(2 * np.pi * np.arange(64) / 64))
    s = capi.Solver(Q, precision, capi.LBM_PHYSICS, tau, 1.0, org, 1.0, 1.0, collision=collision)
    s.set_geometry(mask, [capi.bc_spec(**b) for b in bcs])
    s.set_normals(tri)
    s.set_inlet_table(amp)
    if walls:
        s.set_wall_distances(tri)
    s.step(nsteps)
    cls = classify(mask, [(2, kin), (2, kout)], Q)
    o = oracle.Sim(Q, oracle.PHYSICS, cls, org, 1.0, tau, bcs)
    o.set_amplitude(amp)
    o.set_collision(collision)
    if walls:
        o.set_wall_distances(tri)
    o.set_wss(1.0, 1.0)
    o.compute_normals(tri)
    o.step(nsteps)
    return s, o


@pytest.mark.parametrize("Q", [19, 27])
def test_gpu_fp64_physics_matches_oracle(gpu_lib, oracle_lib, Q):
    s, o = _physics_case(gpu_lib, oracle_lib, Q, gpu_lib.LBM_F64)
    f = s.distributions()
    fo, _, _ = o.f()
    assert np.max(np.abs(f - fo)) <= 1e-13
    w, wo = s.wss(), o.nw()
    assert np.array_equal(w["pt"], wo["pt"])
    np.testing.assert_allclose(w["acc"], wo["acc"], rtol=1e-9, atol=1e-14)
    m, p, fl = s.conservation()
    mo, po, flo = o.conservation()
    assert abs(m - mo) <= 1e-10 * mo
    np.testing.assert_allclose(p, po, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(fl, flo, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("prec,tol,wtol", [("f32", 1e-5, 1e-4), ("f16", 4e-3, 1e-2), ("bf16", 3e-2, 1e-1)])
def test_gpu_physics_precision_vs_fp64_oracle(gpu_lib, oracle_lib, Q, prec, tol, wtol):
    """Velocity L2 relative error of each storage format vs the FP64 oracle,
    and of the time-averaged wall shear stress and the last step's |tau|
    (60 steps: three folds of the FP32 stress ring plus 12 pending steps)."""
    s, o = _physics_case(gpu_lib, oracle_lib, Q, prec, nsteps=60)
    _, u = s.macro()
    fo, _, _ = o.f()
    rho_o = fo.sum(axis=1)
    c, _, _ = oracle_lib.lattice(Q)
    u_o = (fo @ c) / rho_o[:, None]
    rel = np.linalg.norm(u - u_o) / np.linalg.norm(u_o)
    assert rel <= tol, rel
    w, wo = s.wss(), o.nw()
    assert np.array_equal(w["pt"], wo["pt"])
    for key in ("tawss", "wss", "acc"):
        err = np.linalg.norm(w[key] - wo[key]) / np.linalg.norm(wo[key])
        assert err <= wtol, (key, err)


@pytest.mark.parametrize("prec", ["f32", "f16"])
def test_gpu_stress_ring_split_graph_and_checkpoint(gpu_lib, oracle_lib, tmp_path, prec):
    """The FP32 stress ring folds every 16 steps inside the step launch: runs
    split into odd chunks, run through 16-step graphs, or restored from a
    checkpoint with steps pending in the ring accumulate the same stress."""
    a, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=0)
    a.step(53)
    wa = a.wss()
    b, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=0)
    for n in (7, 16, 1, 29):
        b.step(n)
    wb = b.wss()
    for key in ("acc", "acc_mag", "wss"):
        assert np.array_equal(wa[key], wb[key]), key
    g, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=0)
    g.set_graph_steps(16)
    g.step(5)
    g.step(48)
    assert np.array_equal(g.wss()["acc_mag"], wa["acc_mag"])
    c, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=0)
    c.step(21)  # five steps pending in the ring
    c.save(str(tmp_path / "r.bin"))
    d, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=0)
    d.load_checkpoint(str(tmp_path / "r.bin"))
    w_loaded = d.wss()
    np.testing.assert_allclose(w_loaded["acc_mag"], c.wss()["acc_mag"], rtol=1e-6)
    np.testing.assert_allclose(w_loaded["wss"], c.wss()["wss"], rtol=1e-6)
    # the restart re-stores the pre-collision state in the storage format
    # (boundary nodes' populations are quantized once more), so the restarted
    # run agrees to the format's precision; five pending steps counted twice
    # (or lost) would be ~10% off
    d.step(32)
    tol = 1e-3 if prec == "f32" else 2e-2
    for key in ("acc_mag", "acc"):
        err = np.linalg.norm(d.wss()[key] - wa[key]) / np.linalg.norm(wa[key])
        assert err <= tol, (key, err)


def test_gpu_checkpoint_round_trip(gpu_lib, tmp_path):
    d = load(fixtures("sim")[0])
    a, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    a.save(str(tmp_path / "c.bin"))
    a.step(10)
    fa = a.distributions()
    b, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    b.step(3)  # diverge, then restore
    b.load_checkpoint(str(tmp_path / "c.bin"))
    b.step(10)
    assert np.array_equal(b.distributions(), fa)
    assert np.array_equal(b.wss()["acc"], a.wss()["acc"])


def test_gpu_readout_before_first_step_is_initial_state(gpu_lib, oracle_lib):
    d = load(fixtures("sim")[0])
    mask, desc = gpu_lib.voxelize(d["tri12"], 1.0)
    s = gpu_lib.Solver(19, gpu_lib.LBM_F64, gpu_lib.LBM_PARITY, 0.8, 1.0)
    s.set_geometry(mask, [])
    f = s.distributions()
    _, w, _ = oracle_lib.lattice(19)
    assert np.array_equal(f, np.tile(w, (len(f), 1)))
    m, p, _ = s.conservation()
    assert abs(m - len(f)) < 1e-9 and np.all(np.abs(p) < 1e-12)


def test_gpu_divergence_reports_status(gpu_lib):
    """A run driven unstable (Mach > 1 inlet, tau near 0.5) must come back as
    LBM_ERR_NONFINITE, not as a fault."""
    from pv_dec_original_gb300 import geometry as G
    tri = G.config_c1_cylinder().tri12()
    mask, desc = gpu_lib.voxelize(tri, 1.0)
    fl = np.argwhere(mask > 0)
    s = gpu_lib.Solver(19, gpu_lib.LBM_F32, gpu_lib.LBM_PHYSICS, 0.5001, 1.0)
    s.set_geometry(mask, [gpu_lib.bc_spec(gpu_lib.LBM_BC_VELOCITY, 4, int(fl[:, 0].min()), 1.0)])
    s.set_inlet_table([3.0])
    with pytest.raises(gpu_lib.LbmError) as e:
        for _ in range(50):
            s.step(20)
    assert e.value.code == -4


def test_gpu_autotune_restores_state(gpu_lib):
    """Autotuning times every launch variant on a snapshot and restores the
    state: FP64 parity results are bit-identical with or without it, and every
    variant computes the same step."""
    d = load(fixtures("sim")[0])
    a, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64)
    b, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, split=10)  # 10 steps, then the rest
    fa = a.distributions()
    # rerun b from scratch with an autotune after 10 steps
    c, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, split=None)
    best, ms = c.autotune(3)
    assert 0 <= best < gpu_lib.NUM_VARIANTS and all(m > 0 for m in ms)
    assert np.array_equal(c.distributions(), fa)
    for v in range(gpu_lib.NUM_VARIANTS):
        e, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, split=5)
        e.set_variant(v)
        e.step(5)
        r, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, split=5)
        r.step(5)
        assert np.array_equal(e.distributions(), r.distributions()), v


@pytest.mark.parametrize("Q", [19, 27])
def test_gpu_regularized_fp64_matches_oracle(gpu_lib, oracle_lib, Q):
    """Regularized collision: FP64 device run vs the oracle, which evaluates
    Pi = sum (f - feq) c c by direct summation (the kernel uses the analytic
    second moment of the equilibrium)."""
    s, o = _physics_case(gpu_lib, oracle_lib, Q, gpu_lib.LBM_F64, tau=0.56,
                         collision=gpu_lib.LBM_COLLISION_REGULARIZED)
    f = s.distributions()
    fo, _, _ = o.f()
    assert np.max(np.abs(f - fo)) <= 1e-12
    np.testing.assert_allclose(s.wss()["acc"], o.nw()["acc"], rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f16", 4e-3)])
def test_gpu_regularized_precision_vs_fp64_oracle(gpu_lib, oracle_lib, prec, tol):
    s, o = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=60, tau=0.56,
                         collision=gpu_lib.LBM_COLLISION_REGULARIZED)
    _, u = s.macro()
    fo, _, _ = o.f()
    c, _, _ = oracle_lib.lattice(19)
    u_o = (fo @ c) / fo.sum(axis=1)[:, None]
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= tol


def test_gpu_regularized_stable_where_bgk_diverges(gpu_lib):
    """The 256x192x512 bifurcation at tau = 0.55 under the pulsatile inlet:
    BGK diverges near step 2200 (FP32 and FP64 alike); the regularized
    collision runs 4000 steps with bounded velocity and density."""
    from pv_dec_original_gb300 import geometry as G, waveform
    capi = gpu_lib
    surf = G.config_c2_bifurcation()
    tri = surf.tri12()
    mask, desc = capi.voxelize(tri, 1.0)
    bb = np.array(desc.bbox[:])
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    cx, cy = surf.meta["center"]
    bcs = [capi.bc_spec(capi.LBM_BC_VELOCITY, "z-", kin, 1.0, 1, cx, cy, 24.0),
           capi.bc_spec(capi.LBM_BC_PRESSURE, "z+", kout, 1.0)]
    out = {}
    for coll in (capi.LBM_COLLISION_BGK, capi.LBM_COLLISION_REGULARIZED):
        s = capi.Solver(19, "f32", capi.LBM_PHYSICS, 0.55, 1.0, (bb[0], bb[2], bb[4]), 1.0, 4000.0,
                        collision=coll)
        s.set_geometry(mask, bcs)
        s.set_inlet_table(waveform.sinusoid_table(0.03, 4000.0))
        s.set_graph_steps(100)
        try:
            s.step(4000)
            rho, u = s.macro()
            out[coll] = (np.abs(u).max(), rho.min(), rho.max())
        except capi.LbmError as e:
            assert e.code == -4  # LBM_ERR_NONFINITE
            out[coll] = None
        s.close()
    assert out[capi.LBM_COLLISION_BGK] is None
    umax, rmin, rmax = out[capi.LBM_COLLISION_REGULARIZED]
    assert umax < 0.15 and 0.95 < rmin and rmax < 1.05, out


@pytest.mark.parametrize("Q", [19, 27])
def test_gpu_interpolated_walls_match_oracle(gpu_lib, oracle_lib, Q):
    """Interpolated bounce-back: the wall distances (segment-triangle
    intersections in FP64, rounded to FP32) are bit-identical to the
    oracle's, and FP64 distributions after 40 steps agree to 1e-13."""
    s, o = _physics_case(gpu_lib, oracle_lib, Q, gpu_lib.LBM_F64, walls=True)
    pt, q = s.wall_distances()
    opt, _ = o.active()
    qo = o.wall_distances()
    row = {int(p): a for a, p in enumerate(opt)}
    ref = qo[[row[int(p)] for p in pt]]
    assert np.array_equal(q, ref)
    # a real share of the missing links found the surface (not all half-way)
    assert np.mean((q != 0.5) & (q >= 0.0)) > 0.05
    f = s.distributions()
    fo, _, _ = o.f()
    assert np.max(np.abs(f - fo)) <= 1e-13
    # and the walls change the flow (the rule is in effect)
    h, _ = _physics_case(gpu_lib, oracle_lib, Q, gpu_lib.LBM_F64, walls=False)
    assert np.max(np.abs(h.distributions() - f)) > 1e-6


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f16", 4e-3)])
def test_gpu_interpolated_walls_precision(gpu_lib, oracle_lib, prec, tol):
    s, o = _physics_case(gpu_lib, oracle_lib, 19, prec, walls=True)
    _, u = s.macro()
    fo, _, _ = o.f()
    c, _, _ = oracle_lib.lattice(19)
    u_o = (fo @ c) / fo.sum(axis=1)[:, None]  # moments of the same post-boundary state
    assert np.linalg.norm(u - u_o) / np.linalg.norm(u_o) <= tol


def test_gpu_wall_distances_need_physics_mode(gpu_lib):
    d = load(fixtures("sim")[0])
    s, _ = _gpu_parity_run(gpu_lib, d, gpu_lib.LBM_F64, split=0)
    with pytest.raises(gpu_lib.LbmError):
        s.set_wall_distances(d["tri12"])


@pytest.mark.parametrize("prec", ["f64", "f32", "f16"])
def test_gpu_async_outputs_match_sync(gpu_lib, oracle_lib, prec):
    """Asynchronous read-outs hold the state at the time they were queued,
    even with later steps queued before the wait, and equal the
    synchronous read-outs of the same state bit for bit."""
    s, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=20)
    r, _ = _physics_case(gpu_lib, oracle_lib, 19, prec, nsteps=20)
    n, nw = s.counts()["active"], s.counts()["next_to_wall"]
    rho, u = np.zeros(n), np.zeros(3 * n)
    wss, osi, tawss = np.zeros(nw), np.zeros(nw), np.zeros(nw)
    s.outputs_async(rho, u, wss, osi, tawss)
    s.step_async(10)  # queued before the wait: must not change what was read
    s.wait_outputs()
    rho_r, u_r = r.macro()
    w_r = r.wss()
    assert np.array_equal(rho, rho_r) and np.array_equal(u, u_r.reshape(-1))
    # (OSI is 0/0 = NaN, as in the reference, where no stress has accumulated)
    assert np.array_equal(wss, w_r["wss"]) and np.array_equal(osi, w_r["osi"], equal_nan=True)
    assert np.array_equal(tawss, w_r["tawss"])
    # a second read-out after the extra steps sees them
    s.outputs_async(rho, u, wss, osi, tawss)
    s.wait_outputs()
    r.step(10)
    assert np.array_equal(rho, r.macro()[0])
    assert np.array_equal(tawss, r.wss()["tawss"])
