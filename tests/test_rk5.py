"""GPU parity of the RK5 family (RK5DPStep, solver.c:217-421, and the adaptive
Dormand-Prince loop, solver.c:134-154) against the CPU oracle through the C
ABI: the fixed-step RK5CN in FP64 (1e-12 relative L2) and FP32 (1e-5), with
hyperviscosity, forcing and the CFL step; DP5CN with rejected attempts (same
accept/reject sequence, step sizes and state); RK5CN ensemble members equal
to single runs bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("N", [16, 32, 48])
def test_rk5cn_fp64_vs_oracle(ns3d, oracle, N):
    nu, dt = 0.01, 2e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, integrator="rk5cn")
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK5CN)
    s.InitialConditions("SPECTRUM", seed=21, k0=3.0)
    o.ic("SPECTRUM", seed=21, k0=3.0)
    s.RK4Step(12)
    o.step(12)
    assert rel_l2(s.get_state(), o.get_state()) < 1e-12
    t, _, it = s.get_time()
    assert it == 12 and abs(t - o.get_time()[0]) < 1e-15


def test_rk5cn_fp32_vs_oracle(ns3d, oracle):
    N, nu, dt = 64, 5e-3, 2e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, integrator="rk5cn", precision="fp32")
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK5CN)
    s.InitialConditions("SPECTRUM", seed=3, k0=4.0)
    o.ic("SPECTRUM", seed=3, k0=4.0)
    s.RK4Step(10)
    o.step(10)
    assert rel_l2(s.get_state(), o.get_state()) < 1e-5


def test_rk5cn_hyperviscosity_forcing_cfl(ns3d, oracle):
    N = 32
    kw = dict(nu=2e-5, dt=1e-3, visc_pow=2, cfl=0.4, force_k=2)
    s = ns3d.Solver(N, integrator="rk5cn", forcing="SHELL", **kw)
    o = oracle.Oracle(N, integrator=oracle.RK5CN, forcing=oracle.FORCE_SHELL, **kw)
    s.InitialConditions("SPECTRUM", seed=8, k0=4.0)
    o.ic("SPECTRUM", seed=8, k0=4.0)
    s.RK4Step(8)
    o.step(8)
    assert rel_l2(s.get_state(), o.get_state()) < 1e-11
    t, dt, it = s.get_time()
    rt, rdt, rit = o.get_time()
    assert it == rit == 8 and abs(dt / rdt - 1) < 1e-12 and abs(t / rt - 1) < 1e-12


def test_dp5cn_vs_oracle_with_rejections(ns3d, oracle):
    # a first step far too long: the controller rejects it and shrinks dt;
    # the GPU must take the same accept/reject decisions as the oracle
    N, nu = 32, 0.01
    s = ns3d.Solver(N, nu=nu, dt=0.05, integrator="dp5cn")
    o = oracle.Oracle(N, nu=nu, dt=0.05, integrator=oracle.DP5CN)
    s.InitialConditions("SPECTRUM", seed=5, k0=4.0, energy=4.0)
    o.ic("SPECTRUM", seed=5, k0=4.0, energy=4.0)
    for _ in range(3):
        s.RK4Step(2)
        o.step(2)
        err, rej = s.dp_stats()
        rerr, rrej = o.dp_stats()
        assert rej == rrej
        assert abs(err / rerr - 1) < 1e-7
        t, dt, it = s.get_time()
        rt, rdt, rit = o.get_time()
        assert it == rit and abs(t / rt - 1) < 1e-9 and abs(dt / rdt - 1) < 1e-9
    assert rrej >= 1
    assert rel_l2(s.get_state(), o.get_state()) < 1e-10


def test_dp5cn_tolerances_and_fp32(ns3d, oracle):
    # FP32 sums of the error estimate are accurate to ~1e-7 |k| h, so the
    # comparison uses tolerances at which the estimate is far above that
    N, nu = 48, 4e-3
    s = ns3d.Solver(N, nu=nu, dt=0.05, integrator="dp5cn", precision="fp32")
    s.set_dp_tolerances(1e-3, 1e-3)
    o = oracle.Oracle(N, nu=nu, dt=0.05, integrator=oracle.DP5CN, dp_atol=1e-3, dp_rtol=1e-3)
    s.InitialConditions("SPECTRUM", seed=2, k0=3.0)
    o.ic("SPECTRUM", seed=2, k0=3.0)
    s.RK4Step(4)
    o.step(4)
    assert s.dp_stats()[1] == o.dp_stats()[1]
    assert rel_l2(s.get_state(), o.get_state()) < 1e-5


def test_dp5cn_rejects_cfl(ns3d):
    with pytest.raises(ns3d.NS3DError):
        ns3d.Solver(16, nu=0.01, dt=1e-3, integrator="dp5cn", cfl=0.5)


def test_rk5cn_ensemble_equals_single_runs(ns3d):
    members = [dict(N=32, nu=0.01, dt=2e-3, precision="fp32", integrator="rk5cn"),
               dict(N=32, nu=0.003, dt=1e-3, precision="fp32", integrator="rk5cn")]
    ens = ns3d.Ensemble(members)
    for m in range(2):
        ens.InitialConditions(m, "SPECTRUM", seed=m + 1, k0=3.0)
    ens.step(5)
    for m, kw in enumerate(members):
        s = ns3d.Solver(**kw)
        s.InitialConditions("SPECTRUM", seed=m + 1, k0=3.0)
        s.RK4Step(5)
        assert np.array_equal(ens.get_state(m), s.get_state())
