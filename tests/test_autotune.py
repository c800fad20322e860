"""Autotuner (ns3d_autotune / ns3d_tuning_*): every compiled shape of a grid
size (tile / radix variant x z-pass form) is timed and the fastest kept;
engines built afterwards use it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(ns3d, N, steps=5):
    s = ns3d.Solver(N, nu=0.005, dt=1e-3, precision="fp32")
    s.InitialConditions("SPECTRUM", seed=2, k0=4.0)
    s.RK4Step(steps)
    return s.get_state()


@pytest.mark.parametrize("N", [48, 64, 128])
def test_tile_variants_are_bit_identical(ns3d, N):
    """Variants 1, 2, 4 and 6 change only the pencils per CTA: bit-identical. Variant 3
    (another x-pass radix plan, where compiled), variant 5 (the per-mode x-forward
    epilogue at two CTAs per SM) and the z-pass forms change the order of
    operations: FP32 rounding."""
    states = {}
    for v in range(7):
        for z in (0, 1):
            ns3d.tuning_set(N, v, z)
            states[(v, z)] = run(ns3d, N)
    ns3d.tuning_clear()
    for v in (1, 2, 4, 6):
        assert np.array_equal(states[(v, 0)], states[(0, 0)])
        assert np.array_equal(states[(v, 1)], states[(0, 1)])
    ref = states[(0, 0)]
    for key in ((0, 1), (3, 0), (3, 1), (5, 0), (5, 1)):
        assert np.linalg.norm(states[key] - ref) < 1e-6 * np.linalg.norm(ref), key


def test_autotune_picks_fastest_and_persists(ns3d, tmp_path):
    ns3d.tuning_clear()
    best, tried = ns3d.autotune(64, steps=10, precision="fp32", nu=0.005, dt=1e-3)
    assert len(tried) == 21   # 7 variants x 3 z-pass forms at 64^3 (form 2: the tensor-core z pass)
    assert {t["zform"] for t in tried} == {0, 1, 2}
    assert best["ms_per_step"] == min(t["ms_per_step"] for t in tried)
    assert ns3d.tuning(64) == best
    f = tmp_path / "tune.txt"
    ns3d.tuning_save(f)
    ns3d.tuning_clear()
    assert ns3d.tuning(64) is None
    ns3d.tuning_load(f)
    got = ns3d.tuning(64)
    assert (got["variant"], got["zform"]) == (best["variant"], best["zform"])
    # an ensemble built now uses the tuned shape and still equals single runs
    members = [dict(N=64, nu=0.005, dt=1e-3, precision="fp32"), dict(N=64, nu=0.002, dt=1e-3, precision="fp32")]
    ens = ns3d.Ensemble(members)
    for m in range(2):
        ens.InitialConditions(m, "SPECTRUM", seed=m + 4, k0=3.0)
    ens.step(3)
    for m, kw in enumerate(members):
        s = ns3d.Solver(**kw)
        s.InitialConditions("SPECTRUM", seed=m + 4, k0=3.0)
        s.RK4Step(3)
        assert np.array_equal(ens.get_state(m), s.get_state())
    ns3d.tuning_clear()


def test_fp64_has_one_shape(ns3d):
    best, tried = ns3d.autotune(32, steps=3, precision="fp64", nu=0.01, dt=1e-3)
    assert len(tried) == 1 and best["zform"] == 1   # no line kernel and no tensor-core z pass in FP64
    ns3d.tuning_clear()


def test_line_kernel_1024_matches_cta_pass(ns3d):
    """1024-point z lines span two warps (named-barrier exchanges): the persistent
    line kernel and the CTA-synchronous pass give the same step to FP32 rounding
    (compared through the spectra; the state itself is 26 GB on the host)."""
    N = 1024
    res = []
    for z in (0, 1):
        ns3d.tuning_set(N, 0, z)
        s = ns3d.Solver(N, nu=4e-4, dt=5e-4, precision="fp32", forcing="SHELL", force_k=2)
        s.InitialConditions("SPECTRUM", seed=1, k0=4.0)
        s.RK4Step(2)
        tot, Ek, Ok = s.ComputeSystemMeasurables()
        res.append((tot, Ek, Ok))
        s.close()
    ns3d.tuning_clear()
    (t0, E0, O0), (t1, E1, O1) = res
    for key in ("energy", "enstrophy", "dissipation"):
        assert abs(t0[key] / t1[key] - 1) < 1e-6, key
    # FP32 round-off is relative to the spectrum's peak (its tail sits ~20 decades down)
    assert np.max(np.abs(E0 - E1)) < 1e-6 * E1.max()
    assert np.max(np.abs(O0 - O1)) < 1e-6 * O1.max()
