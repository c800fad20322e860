"""GPU longitudinal velocity-increment statistics (ns3d_increment_stats, the
post-processing of PostProcessing/src/stats.c) against the CPU oracle: FP64
moments to 1e-9, bin edges to 1e-12, counts exactly; FP32 to its rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [16, 32])
def test_increment_stats_fp64_vs_oracle(ns3d, oracle, N):
    s = ns3d.Solver(N, nu=0.01, dt=1e-3)
    o = oracle.Oracle(N, nu=0.01, dt=1e-3)
    s.InitialConditions("SPECTRUM", seed=4, k0=3.0)
    o.ic("SPECTRUM", seed=4, k0=3.0)
    s.RK4Step(3)
    o.step(3)
    got = s.increment_stats(n_bins=200)
    ref = o.increment_stats(n_bins=200)
    assert np.allclose(got["stats"], ref["stats"], rtol=1e-9, atol=1e-12)
    assert np.allclose(got["ranges"], ref["ranges"], rtol=1e-12, atol=1e-14)
    assert np.array_equal(got["counts"], ref["counts"])


def test_increment_stats_fp32_and_custom_increments(ns3d, oracle):
    N = 64
    s = ns3d.Solver(N, nu=0.01, dt=1e-3, precision="fp32")
    o = oracle.Oracle(N, nu=0.01, dt=1e-3)
    s.InitialConditions("SPECTRUM", seed=8, k0=4.0)
    o.ic("SPECTRUM", seed=8, k0=4.0)
    inc = [1, 5, 17, 63, 64]
    got = s.increment_stats(inc, n_bins=1000)
    ref = o.increment_stats(inc, n_bins=1000)
    assert np.allclose(got["stats"][:, [0, 1, 3]], ref["stats"][:, [0, 1, 3]], rtol=1e-5, atol=1e-6)
    assert np.allclose(got["stats"][:, 4:], ref["stats"][:, 4:], atol=1e-4)
    assert np.all(got["stats"][-1] == 0) and got["counts"][-1].sum() == 0       # r = N: no pairs
    n_pairs = [3 * N * N * (N - r) for r in inc[:-1]]
    assert np.array_equal(got["counts"].sum(axis=1)[:-1], n_pairs)
    # FP32 samples move across a bin edge only rarely
    assert np.abs(got["counts"] - ref["counts"]).sum() <= 5e-4 * sum(n_pairs)
