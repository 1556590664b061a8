"""Edge cases of the C ABI on the GPU: rejected arguments, an empty lattice,
a single fluid node, ragged lattice sizes against the oracle, and calls made
in the wrong state.  Every failure is a status code, never a fault."""
import numpy as np
import pytest

from helpers import classify

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kw", [dict(Q=20), dict(tau=0.5), dict(tau=0.3), dict(spacing=0.0), dict(collision=5),
                                dict(precision=7), dict(mode=9), dict(device=64)])
def test_gpu_create_rejects_bad_arguments(gpu_lib, kw):
    with pytest.raises(gpu_lib.LbmError) as e:
        gpu_lib.Solver(**kw)
    assert e.value.code < 0


def test_gpu_calls_in_the_wrong_state(gpu_lib):
    s = gpu_lib.Solver(19, "f32", gpu_lib.LBM_PHYSICS, 0.8)
    with pytest.raises(gpu_lib.LbmError):
        s.step(1)  # no geometry
    with pytest.raises(gpu_lib.LbmError):
        s.init_from_macro(np.ones(1, np.float32), np.zeros(3, np.float32))
    mask = np.ones((6, 5, 4), np.uint8)
    s.set_geometry(mask)
    with pytest.raises(gpu_lib.LbmError):
        s.step(-1)
    with pytest.raises(gpu_lib.LbmError):
        s.set_variant(gpu_lib.NUM_VARIANTS)
    with pytest.raises(gpu_lib.LbmError):
        s.set_waveform(gpu_lib.MAX_WAVES, [0.01])
    with pytest.raises(gpu_lib.LbmError):
        s.set_graph_steps(3)  # odd
    with pytest.raises(gpu_lib.LbmError):
        s.set_geometry(mask, [gpu_lib.bc_spec(gpu_lib.LBM_BC_PRESSURE, "z+", -1, 0.0)])  # density 0
    s.step(0)
    s.step(3)


@pytest.mark.parametrize("prec", ["f64", "f32", "f16"])
def test_gpu_empty_lattice(gpu_lib, prec):
    s = gpu_lib.Solver(19, prec, gpu_lib.LBM_PHYSICS, 0.8)
    s.set_geometry(np.zeros((5, 4, 3), np.uint8))
    c = s.counts()
    assert c["active"] == 0 and c["next_to_wall"] == 0
    s.step(7)
    rho, u = s.macro()
    assert rho.shape == (0,) and u.shape == (0, 3)
    assert len(s.wss()["wss"]) == 0
    m, p, _ = s.conservation()
    assert m == 0.0 and np.all(p == 0.0)


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "bf16"])
def test_gpu_single_fluid_node_stays_at_rest(gpu_lib, Q, prec):
    mask = np.zeros((3, 3, 3), np.uint8)
    mask[1, 1, 1] = 1
    s = gpu_lib.Solver(Q, prec, gpu_lib.LBM_PHYSICS, 0.7)
    s.set_geometry(mask)
    s.step(25)
    rho, u = s.macro()
    assert rho.shape == (1,)
    assert abs(rho[0] - 1.0) < 1e-6 and np.all(np.abs(u) < 1e-7)


@pytest.mark.parametrize("Q", [19, 27])
def test_gpu_ragged_lattice_matches_oracle(gpu_lib, oracle_lib, Q):
    """An odd-sized lattice (13 x 7 x 5) with a random fluid blob and a
    random initial state: FP64 physics steps agree with the oracle."""
    rng = np.random.default_rng(11)
    mask = (rng.random((5, 7, 13)) < 0.8).astype(np.uint8)
    s = gpu_lib.Solver(Q, "f64", gpu_lib.LBM_PHYSICS, 0.65)
    s.set_geometry(mask)
    n = s.counts()["active"]
    c, w, _ = oracle_lib.lattice(Q)
    f0 = w[None, :] * (1.0 + 0.02 * rng.standard_normal((n, Q)))
    s.set_distributions(f0)
    cls = classify(mask, [], Q)
    o = oracle_lib.Sim(Q, oracle_lib.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, 0.65, [])
    o.set_amplitude([0.0])
    o.set_wss(1.0, 1.0)
    o.set_f(f0)
    s.step(9)
    o.step(9)
    fo, _, _ = o.f()
    assert np.max(np.abs(s.distributions() - fo)) <= 1e-13
