"""z-pass form 2: the z transforms of the FP32 engines as DFT matrix products on
the tensor cores (tcgen05, split-BF16 operands, three terms hi*hi + hi*lo +
lo*hi accumulated in FP32), for N in {16, 32, 48, 64, 96, 128}; it replaces the
z-axis FFTs of NonlinearRHSBatch (solver.c:656, 658, 683).

Bars, relative L2 against the FP64 oracle: 1e-4 for one nonlinear evaluation
and after 10 IF-RK4 steps (the split-BF16 products carry ~1e-5 relative error
per transform, against ~1e-7 for the FP32 FFT form); the CFL speed bound, the
energy and E(k) agree with the FFT form of the same engine to 1e-4."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def dealiased_random(N, seed):
    rng = np.random.default_rng(seed)
    uh = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    k = np.fft.fftfreq(N, 1.0 / N)
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
    uh[np.sqrt(K2) > N // 3] = 0
    return uh


@pytest.fixture
def zform2(ns3d):
    saved = {}

    def use(N, z=2):
        if N not in saved:
            saved[N] = ns3d.tuning(N, "fp32")
        ns3d.tuning_set(N, 0, zform=z, precision="fp32")

    yield use
    for N, t in saved.items():
        if t:
            ns3d.tuning_set(N, t["variant"], zform=t["zform"], precision="fp32")
    if not any(saved.values()):
        ns3d.tuning_clear()


@pytest.mark.parametrize("N", [16, 32, 48, 64, 96, 128])
def test_zgemm_rhs_vs_oracle(ns3d, oracle, zform2, N):
    zform2(N)
    s = ns3d.Solver(N, nu=0.01, precision="fp32")
    assert s.kernels_per_step == 4 * 6 + 1   # two z kernels per evaluation
    u = dealiased_random(N, 40 + N)
    got = s.NonlinearRHSBatch(u)
    ref = oracle.Oracle(N, nu=0.01).rhs(u)
    err = rel(got, ref)
    print(f"N={N} zgemm rhs rel-L2 {err:.3e}")
    assert err < TOL
    s.close()


@pytest.mark.parametrize("N", [32, 64, 128])
def test_zgemm_steps_vs_oracle(ns3d, oracle, zform2, N):
    zform2(N)
    nu, dt = 0.01, 2e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, precision="fp32", cfl=0.5, forcing="SHELL", force_k=2)
    s.InitialConditions("SPECTRUM", seed=9, k0=4.0)
    o = oracle.Oracle(N, nu=nu, dt=dt, cfl=0.5, forcing=oracle.FORCE_SHELL, force_k=2)
    o.ic("SPECTRUM", seed=9, k0=4.0)
    s.RK4Step(10)
    o.step(10)
    err = rel(s.get_state(), o.get_state())
    print(f"N={N} zgemm 10 forced CFL steps rel-L2 {err:.3e}")
    assert err < TOL
    assert abs(s.get_time()[0] - o.get_time()[0]) < TOL * o.get_time()[0]
    s.close()


@pytest.mark.parametrize("N", [48, 96])
def test_zgemm_matches_fft_form(ns3d, zform2, N):
    """Same engine shape, z pass as FFTs (form 0) and as GEMMs (form 2): the CFL
    speed bound and the diagnostics after 5 steps."""
    out = {}
    for z in (0, 2):
        zform2(N, z)
        s = ns3d.Solver(N, nu=0.005, dt=1e-3, precision="fp32", cfl=0.5)
        s.InitialConditions("SPECTRUM", seed=2, k0=3.0)
        umax = s.max_speed_sum()
        s.RK4Step(5)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        out[z] = (umax, tot["energy"], Ek)
        s.close()
    assert abs(out[2][0] - out[0][0]) <= TOL * out[0][0]
    assert abs(out[2][1] - out[0][1]) <= TOL * out[0][1]
    assert rel(out[2][2], out[0][2]) < TOL
