"""Failure detection, exercised without faulting the GPU: the reference
defines limits (MIN_STEP_SIZE, MAX_ITERS, MAX_VORT_LIM, data_types.h:130-136)
but never checks them; this library reports failures as status codes.

* A bounded wait that runs out: the wait budget of the copy-fed passes (the
  z pass, and the tensor-tile x-inverse pass of variant 3) is cut to a few
  clock cycles, so the first wait on an asynchronous copy gives up; the pass
  lets its copies land, records the timeout and returns, ns3d_step reports
  NS3D_ERR_TIMEOUT, and after the budget is restored the same context steps
  correctly again.
* A NaN inside the dealiased sphere of a small host field: ns3d_step reports
  NS3D_ERR_NUMERIC; the context recovers once a clean state is loaded.
* A learned closure that injects energy (its output layer negated) fails the
  per-step energy-budget check, and that step is the plain coarse solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def dealiased_random(N, seed):
    rng = np.random.default_rng(seed)
    uh = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    k = np.fft.fftfreq(N, 1.0 / N)
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
    uh[np.sqrt(K2) > N // 3] = 0
    return uh


@pytest.mark.parametrize("N,variant", [(64, None), (256, None), (64, 3)])
def test_wait_timeout_is_reported_and_recovered(ns3d, oracle, N, variant):
    """variant 3: the tensor-tile x-inverse pass, the first pass of the step, gives up first."""
    saved = ns3d.tuning(N, "fp32")
    v = variant if variant is not None else (saved["variant"] if saved else 0)
    ns3d.tuning_set(N, v, zform=0, precision="fp32")   # the bulk-copy z pass
    try:
        nu, dt = 0.01, 1e-3
        s = ns3d.Solver(N, nu=nu, dt=dt, precision="fp32")
        s.InitialConditions("SPECTRUM", seed=4, k0=3.0)
        u0 = s.get_state()
        s.set_wait_budget(2)
        with pytest.raises(ns3d.NS3DError) as e:
            s.RK4Step(1)
        assert e.value.status == ns3d.ERR_TIMEOUT
        s.set_wait_budget(0)
        s.set_state(u0)
        s.set_time(0.0, dt, 0)
        s.RK4Step(2)
        if N == 64:
            o = oracle.Oracle(N, nu=nu, dt=dt)
            o.set_state(u0)
            o.step(2)
            assert rel(s.get_state(), o.get_state()) < 1e-5
        else:
            assert np.isfinite(s.ComputeSystemMeasurables()[0]["energy"])
        s.close()
    finally:
        if saved:
            ns3d.tuning_set(N, saved["variant"], zform=saved["zform"], precision="fp32")
        else:
            ns3d.tuning_clear()


@pytest.mark.parametrize("N,prec,tol", [(16, "fp64", 1e-12), (32, "fp32", 1e-5)])
def test_nan_in_field_is_reported_and_recovered(ns3d, oracle, N, prec, tol):
    nu, dt = 0.01, 1e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, precision=prec)
    u = dealiased_random(N, 11)
    bad = u.copy()
    bad[2, 1, 1, 0] = complex(np.nan, 0.0)   # inside the sphere |k| <= N/3
    s.set_state(bad)
    with pytest.raises(ns3d.NS3DError) as e:
        s.RK4Step(1)
    assert e.value.status == ns3d.ERR_NUMERIC
    s.set_state(u)
    s.set_time(0.0, dt, 0)
    s.RK4Step(1)
    o = oracle.Oracle(N, nu=nu, dt=dt)
    o.set_state(u)
    o.step(1)
    assert rel(s.get_state(), o.get_state()) < tol
    s.close()


def test_energy_injecting_closure_falls_back(ns3d):
    """T_sgs = sum m Re(u_hat . conj(F_hat)) is linear in the network's output
    layer, so negating that layer flips its sign: of the two runs from the same
    state exactly one keeps the closure, and the other is the plain step."""
    Nc, nu, dt = 16, 5e-3, 2e-3
    les = ns3d.LES(Nc, capacity=0, seed=3)
    les.set_scales(1.0, 1.0)
    w = les.weights()
    n_out = 6 * 32 * 27 + 6   # the 32 -> 6 output layer: weights, then biases, last in the vector
    states, counters = {}, {}
    for sign in (1.0, -1.0):
        w2 = w.copy()
        w2[-n_out:] *= sign
        les.set_weights(w2)
        c = ns3d.Solver(Nc, nu=nu, dt=dt, precision="fp32")
        c.InitialConditions("SPECTRUM", seed=1, k0=3.0)
        c.attach_closure(les)
        c.RK4Step(1)
        counters[sign] = c.closure_counters()
        states[sign] = c.get_state()
        c.close()
    p = ns3d.Solver(Nc, nu=nu, dt=dt, precision="fp32")
    p.InitialConditions("SPECTRUM", seed=1, k0=3.0)
    p.RK4Step(1)
    plain = p.get_state()
    p.close()
    assert sorted(counters.values()) == [(0, 1), (1, 0)], counters
    fell_back = 1.0 if counters[1.0] == (0, 1) else -1.0
    kept = -fell_back
    assert rel(states[fell_back], plain) < 1e-6
    assert rel(states[kept], plain) > 1e-6
    les.close()
