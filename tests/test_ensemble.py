"""Ensembles (ns3d_ensemble_*): independent runs of mixed grid sizes,
viscosities and initial conditions stepped by one graph launch per step must
give exactly the result of the same runs stepped one by one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_ensemble_matches_single_runs(ns3d, oracle):
    members = [
        dict(N=16, nu=0.02, dt=2e-3, precision="fp64"),
        dict(N=24, nu=0.01, dt=2e-3, precision="fp64"),
        dict(N=16, nu=0.005, dt=1e-3, precision="fp64"),
        dict(N=32, nu=0.004, dt=1e-3, precision="fp32", cfl=0.5),
        dict(N=32, nu=0.002, dt=1e-3, precision="fp32", cfl=0.5),
        dict(N=48, nu=0.003, dt=1e-3, precision="fp32"),
    ]
    seeds = [11, 12, 13, 14, 15, 16]
    k0s = [2.0, 3.0, 4.0, 5.0, 6.0, 3.5]
    ens = ns3d.Ensemble(members)
    groups, kps = ens.info()
    assert groups == 4 and kps == 3 * 21 + 22
    for i, (s, k) in enumerate(zip(seeds, k0s)):
        ens.InitialConditions(i, "SPECTRUM", seed=s, k0=k)
    ens.step(7)
    for i, m in enumerate(members):
        single = ns3d.Solver(**m)
        single.InitialConditions("SPECTRUM", seed=seeds[i], k0=k0s[i])
        single.RK4Step(7)
        assert np.array_equal(ens.get_state(i), single.get_state()), i
        assert ens.get_time(i) == single.get_time()
        single.close()
    # one FP64 member against the CPU oracle
    o = oracle.Oracle(24, nu=0.01, dt=2e-3)
    o.ic("SPECTRUM", seed=12, k0=3.0)
    o.step(7)
    ref = o.get_state()
    got = ens.get_state(1)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12
    tot, Ek, _ = ens.measurables(1)
    rt, rE, _ = o.measurables()
    assert abs(tot["energy"] - rt[0]) < 1e-12 * rt[0]
    ens.close()


def test_ensemble_run_is_one_launch_of_the_same_steps(ns3d):
    """ns3d_ensemble_run: the captured step in a device-side while loop (one graph
    launch for the whole run) gives the ensemble's per-step result bit for bit,
    over two runs in a row (the loop counter is reset by every call)."""
    members = [dict(N=16, nu=0.02, dt=2e-3, precision="fp64"),
               dict(N=32, nu=0.004, dt=1e-3, precision="fp32", cfl=0.5),
               dict(N=48, nu=0.003, dt=1e-3, precision="fp32", forcing="SHELL", force_k=2)]
    a, b = ns3d.Ensemble(members), ns3d.Ensemble(members)
    for e in (a, b):
        for i in range(len(members)):
            e.InitialConditions(i, "SPECTRUM", seed=30 + i, k0=3.0)
    a.step(9)
    a.step(4)
    b.run(9)
    b.run(4)
    for i in range(len(members)):
        assert np.array_equal(a.get_state(i), b.get_state(i)), i
        assert a.get_time(i) == b.get_time(i)
    a.close()
    b.close()


def test_group_profile(ns3d):
    """ns3d_ensemble_profile: per launch group, the device time of each kernel
    class of one step of all the group's members."""
    members = [dict(N=32, nu=0.01, dt=1e-3, precision="fp32") for _ in range(3)] + \
              [dict(N=48, nu=0.01, dt=1e-3, precision="fp32") for _ in range(2)]
    ens = ns3d.Ensemble(members)
    for m in range(len(members)):
        ens.InitialConditions(m, "SPECTRUM", seed=m, k0=3.0)
    groups, _ = ens.info()
    assert groups == 2
    seen = set()
    for g in range(groups):
        n, prof = ens.profile_group(g, reps=2)
        seen.add(n)
        names = [p[0] for p in prof]
        assert "k_xinv" in names and "k_xfwd" in names and len(prof) == 6
        assert all(t >= 0.0 for _, t, _ in prof) and sum(t for _, t, _ in prof) > 0.0
    assert seen == {32, 48}
    with pytest.raises(ns3d.NS3DError):
        ens.profile_group(groups)
    ens.close()


def test_ensemble_96_fp32_matches_single_runs(ns3d):
    """The C4 ensemble's 96^3 FP32 group (the inverse y pass on its 12 x 8 plan of 24
    elements per thread): two members stepped together equal the same runs stepped alone."""
    members = [dict(N=96, nu=nu, dt=1e-3, precision="fp32", cfl=0.5) for nu in (0.004, 0.002)]
    ens = ns3d.Ensemble(members)
    for i in range(2):
        ens.InitialConditions(i, "SPECTRUM", seed=21 + i, k0=3.0 + i)
    ens.step(3)
    for i, m in enumerate(members):
        single = ns3d.Solver(**m)
        single.InitialConditions("SPECTRUM", seed=21 + i, k0=3.0 + i)
        single.RK4Step(3)
        assert np.array_equal(ens.get_state(i), single.get_state()), i
        single.close()
    ens.close()
