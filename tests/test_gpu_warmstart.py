"""Learned warm start end to end: steady LBM solutions of seeded vessels
(one packed ensemble) train the encoder-decoder on the device; on held-out
vessels the network's field is closer to the converged one than the
Poiseuille prior it corrects (and than rest), and a lattice started from it
converges to the same flow and wall shear stress as one started from rest
and settles within 1% of the converged WSS (the plain LBM decides).
Steps are reported, not asserted: on these small steady cases a start from
rest already converges within about one viscous time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

TAU = 0.55


def test_gpu_warm_start_checked_by_lbm(gpu_lib):
    from pv_dec_original_gb300 import warmstart as WS
    train_m = WS.vessel_members(32, seed=1)
    test_m = WS.vessel_members(3, seed=99)
    sols = WS.steady_ensemble(train_m, tau=TAU, steps=60000)
    samples = [WS.make_sample(mask, m, rho, u, tau=TAU) for (mask, rho, u), m in zip(sols, train_m)]
    net = WS.WarmStartNet(sols[0][0].shape, seed=0)
    hist = WS.train(net, samples, iters=1500, lr=2e-3, batch=4)
    assert hist[-1] < 0.05 * hist[0], hist
    diag = []
    for m in test_m:
        sc, mask = WS.single_lattice(m, tau=TAU)
        sc.set_graph_steps(100)
        nc, _, hc = WS.converge_with_history(sc, tol=1e-6, max_steps=60000)
        rc, uc = sc.macro()
        wc = sc.wss()["wss"]
        c1 = WS.first_within(hc, wc, 0.01)
        x, prior = WS.features(mask, m["inlet_mean"], m["period"], tau=TAU)
        _, u_prior = WS.prediction_to_macro(mask, WS.zero_output(prior), m["inlet_mean"], prior)
        rho, u = WS.prediction_to_macro(mask, net.forward(x), m["inlet_mean"], prior)
        err_net = np.linalg.norm(u - uc) / np.linalg.norm(uc)
        err_prior = np.linalg.norm(u_prior - uc) / np.linalg.norm(uc)
        sw, _ = WS.single_lattice(m, tau=TAU)
        sw.set_graph_steps(100)
        sw.init_from_macro(rho, u, True)
        nw, rw = WS.steps_to_converge(sw, tol=1e-6, max_steps=60000)
        sw1, _ = WS.single_lattice(m, tau=TAU)
        sw1.set_graph_steps(100)
        sw1.init_from_macro(rho, u, True)
        w1 = WS.steps_to_wss(sw1, wc, 0.01, max_steps=4 * c1 + 2000)
        diag.append(dict(cold=nc, warm=nw, warm_residual=rw, cold_1pct=c1, warm_1pct=w1, err_net=err_net,
                         err_prior=err_prior,
                         u_diff=np.linalg.norm(sw.macro()[1] - uc) / np.linalg.norm(uc),
                         wss_diff=np.linalg.norm(sw.wss()["wss"] - wc) / np.linalg.norm(wc)))
    print(diag)
    for d in diag:
        assert d["err_net"] < d["err_prior"] < 1.0, diag
        assert d["warm_residual"] < 1e-6, diag
        assert d["warm_1pct"] is not None and d["cold_1pct"] is not None, diag
        assert d["u_diff"] < 0.01 and d["wss_diff"] < 0.01, diag


def test_gpu_warm_start_periodic_beats_prior_and_cold(gpu_lib):
    """Pulsatile inlets (each vessel its own mean and period): trained on
    converged periodic states at phase 0, the network's start reaches the
    cold run's converged periodic WSS (within 1% at the same phase from
    then on) in less wall time than the Poiseuille prior alone, which beats
    a start from rest; every arm settles on the same periodic state.  Wall
    time counts the prediction (features, network, prior, smoothing, state
    build, all on the device) plus steps x the measured time per step;
    totals over 6 held-out vessels on 128 x 64 x 64 grids."""
    import bench
    r = bench.warmstart_extra(0, conv=False)
    print({k: v for k, v in r.items() if k != "per_vessel"})
    for row in r["per_vessel"]:
        for arm in ("cold", "prior", "net"):
            assert row[arm]["steps_1pct_wss"] is not None, (arm, row)
            assert row[arm]["last_cycle_change"] < 1e-3 or row[arm]["periods_run"] > row["cold"]["periods_run"], row
    assert r["net_over_cold_time"] < r["prior_over_cold_time"] < 1.0, r
    assert r["net_over_cold_steps"] < r["prior_over_cold_steps"] < 1.0, r
    # the network's phase-0 field is closer to the converged one than the prior's
    err = lambda arm: sum(row[arm]["err_u_phase0"] for row in r["per_vessel"])
    assert err("net") < err("prior"), r["per_vessel"]
