"""The x-inverse pass fed by tensor-tile copies (k_xinv_tma, the FP32 engines of
tile variant 3): persistent CTAs load each velocity component of a 16-pencil
tile with cp.async.bulk.tensor boxes of the kx rows inside the sphere. Checked
against the oracle's nonlinear term (FP32 bar 1e-5), against tile variant 0 over
a few steps (FP32 rounding), through an ensemble, whose members sit at
different offsets of the tensor maps, against single runs (bit-identical), and
at 512^3, the size the autotuner picks this variant for, against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def dealiased_random(N, seed):
    rng = np.random.default_rng(seed)
    uh = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    k = np.fft.fftfreq(N, 1.0 / N)
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
    uh[np.sqrt(K2) > N // 3] = 0
    return uh


@pytest.fixture
def variant3(ns3d):
    saved = {}

    def use(N):
        saved[N] = ns3d.tuning(N, "fp32")
        ns3d.tuning_set(N, 3, zform=0, precision="fp32")

    yield use
    ns3d.tuning_clear()
    for N, t in saved.items():
        if t:
            ns3d.tuning_set(N, t["variant"], zform=t["zform"], precision="fp32")


@pytest.mark.parametrize("N", [48, 64, 128, 256])
def test_rhs_vs_oracle(ns3d, oracle, variant3, N):
    variant3(N)
    u = dealiased_random(N, N + 5)
    s = ns3d.Solver(N, precision="fp32")
    got = s.NonlinearRHSBatch(u)
    s.close()
    ref = oracle.Oracle(N).rhs(u)
    assert rel_l2(got, ref) < 1e-5


@pytest.mark.parametrize("N", [64, 128])
def test_steps_vs_variant0(ns3d, N):
    """IF-RK4 evaluates the RHS of U (stage 1) and of UT (stages 2-4): both maps."""
    states = {}
    for v in (0, 3):
        ns3d.tuning_set(N, v, zform=0, precision="fp32")
        s = ns3d.Solver(N, nu=0.005, dt=1e-3, precision="fp32", forcing="SHELL", force_k=2)
        s.InitialConditions("SPECTRUM", seed=3, k0=4.0)
        s.RK4Step(5)
        states[v] = s.get_state()
        s.close()
    ns3d.tuning_clear()
    assert rel_l2(states[3], states[0]) < 1e-6


def test_ensemble_members_match_single_runs(ns3d, variant3):
    N = 64
    variant3(N)
    members = [dict(N=N, nu=nu, dt=1e-3, precision="fp32") for nu in (0.005, 0.002, 0.01)]
    ens = ns3d.Ensemble(members)
    for m in range(len(members)):
        ens.InitialConditions(m, "SPECTRUM", seed=m + 11, k0=3.0)
    ens.step(4)
    for m, kw in enumerate(members):
        s = ns3d.Solver(**kw)
        s.InitialConditions("SPECTRUM", seed=m + 11, k0=3.0)
        s.RK4Step(4)
        assert np.array_equal(ens.get_state(m), s.get_state())
        s.close()


def test_512_matches_variant0_spectra(ns3d):
    """512^3 forced turbulence, two steps: the energy and every shell of E(k)
    agree with tile variant 0 to FP32 rounding (relative to the spectrum's peak)."""
    N = 512
    res = {}
    for v in (0, 3):
        ns3d.tuning_set(N, v, zform=0, precision="fp32")
        s = ns3d.Solver(N, nu=1e-3, dt=5e-4, precision="fp32", forcing="SHELL", force_k=2)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s.RK4Step(2)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        res[v] = (tot["energy"], Ek)
        s.close()
    ns3d.tuning_clear()
    (e0, E0), (e3, E3) = res[0], res[3]
    assert abs(e3 / e0 - 1) < 1e-6
    assert np.max(np.abs(E3 - E0)) < 1e-6 * E0.max()


def test_rhs_512_tuned_shape_vs_oracle(ns3d, oracle, variant3):
    """The tuned 512^3 shape (tile variant 3, line-kernel z pass): the tensor-tile
    x-inverse pass at its largest size and the half-length Nz transform, which
    only the 512-point z lines use; the nonlinear term of a dealiased spectrum
    against the oracle (FP64, all host cores) at the FP32 bar."""
    N = 512
    variant3(N)
    s = ns3d.Solver(N, nu=1e-3, dt=1e-3, precision="fp32")
    s.InitialConditions("SPECTRUM", seed=3, k0=4.0)
    u = s.get_state()
    got = s.NonlinearRHSBatch(u)
    s.close()
    ref = oracle.Oracle(N).rhs(u)
    assert rel_l2(got, ref) < 1e-5
