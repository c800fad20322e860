"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle
on the same inputs, plus size-independent properties at larger grids.

Tolerances: FP64 relative L2 <= 1e-12 (the bar for the 64^3 Taylor–Green
run after 100 steps); FP32-bulk results are checked at 1e-5 relative."""
import numpy as np
import pytest
from helpers import shapiro_exact

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def kgrid(N):
    k = np.array([i if i <= N // 2 else i - N for i in range(N)], dtype=np.float64)
    return np.meshgrid(k, k, np.arange(N // 2 + 1, dtype=np.float64), indexing="ij")


def dealiased_random(N, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((N, N, N, 3)) * scale
    uh = np.fft.rfftn(u, axes=(0, 1, 2))
    KX, KY, KZ = kgrid(N)
    uh[np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2) > N // 3] = 0
    return uh


@pytest.mark.parametrize("N", [8, 16, 24, 32, 48, 64, 96])
def test_rhs_fp64(ns3d, oracle, N):
    u = dealiased_random(N, N)
    s = ns3d.Solver(N, precision="fp64")
    got = s.NonlinearRHSBatch(u)
    ref = oracle.Oracle(N).rhs(u)
    assert rel_l2(got, ref) < FP64_TOL


@pytest.mark.parametrize("N", [16, 32, 64, 96, 128])
def test_rhs_fp32(ns3d, oracle, N):
    u = dealiased_random(N, N + 1)
    s = ns3d.Solver(N, precision="fp32")
    got = s.NonlinearRHSBatch(u)
    ref = oracle.Oracle(N).rhs(u)
    assert rel_l2(got, ref) < FP32_TOL


@pytest.mark.parametrize("name", ["TAYLOR_GREEN", "SHAPIRO", "SPECTRUM", "RANDOM", "TESTING"])
@pytest.mark.parametrize("N", [16, 48])
def test_initial_conditions(ns3d, oracle, name, N):
    s = ns3d.Solver(N)
    s.InitialConditions(name, seed=7, k0=3.0, energy=1.0)
    o = oracle.Oracle(N)
    o.ic(name, seed=7, k0=3.0, energy=1.0)
    ref = o.get_state()
    got = s.get_state()
    if name == "TESTING":
        assert np.all(got == 0) and np.all(ref == 0)
    else:
        assert rel_l2(got, ref) < FP64_TOL


@pytest.mark.parametrize("N,prec,tol", [(32, "fp64", FP64_TOL), (48, "fp64", FP64_TOL), (64, "fp32", FP32_TOL)])
def test_measurables(ns3d, oracle, N, prec, tol):
    o = oracle.Oracle(N, nu=0.01)
    o.ic("SPECTRUM", seed=3, k0=4.0, energy=1.0)
    u = o.get_state()
    s = ns3d.Solver(N, nu=0.01, precision=prec)
    s.set_state(u)
    tot, Ek, Ok = s.ComputeSystemMeasurables()
    rt, rE, rO = o.measurables()
    got = np.array([tot["energy"], tot["enstrophy"], tot["palinstrophy"], tot["helicity"], tot["dissipation"]])
    scale = np.array([rt[0], rt[1], rt[2], np.sqrt(rt[0] * rt[1]), rt[4]])
    assert np.all(np.abs(got - rt) <= tol * scale)
    assert rel_l2(Ek, rE) < tol and rel_l2(Ok, rO) < tol


def test_taylor_green_64_100_steps_fp64(ns3d, oracle):
    """Config 1: TG 64^3, nu = 1/400, dt = 1e-3, IF-RK4, 2/3 dealias, 100 steps;
    per-step energy, enstrophy and E(k) compared every 10 steps."""
    N, nu, dt = 64, 1.0 / 400.0, 1e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, precision="fp64")
    o = oracle.Oracle(N, nu=nu, dt=dt)
    s.InitialConditions("TAYLOR_GREEN")
    o.ic("TAYLOR_GREEN")
    for _ in range(10):
        s.RK4Step(10)
        o.step(10)
        tot, Ek, Ok = s.ComputeSystemMeasurables()
        rt, rE, rO = o.measurables()
        assert abs(tot["energy"] - rt[0]) <= FP64_TOL * rt[0]
        assert abs(tot["enstrophy"] - rt[1]) <= FP64_TOL * rt[1]
        assert rel_l2(Ek, rE) < FP64_TOL
    assert rel_l2(s.get_state(), o.get_state()) < FP64_TOL
    t, dt_, it = s.get_time()
    assert it == 100 and abs(t - 0.1) < 1e-15


def test_rk4cn_matches_reference_integrator(ns3d, oracle):
    N, nu, dt = 32, 0.01, 2e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, integrator="rk4cn")
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK4CN)
    s.InitialConditions("SPECTRUM", seed=11, k0=3.0)
    o.ic("SPECTRUM", seed=11, k0=3.0)
    s.RK4Step(20)
    o.step(20)
    assert rel_l2(s.get_state(), o.get_state()) < FP64_TOL


@pytest.mark.parametrize("integrator", ["ifrk4", "rk4cn"])
def test_hyperviscosity(ns3d, oracle, integrator):
    N, nu, dt = 24, 1e-4, 2e-3
    s = ns3d.Solver(N, nu=nu, dt=dt, visc_pow=2, integrator=integrator)
    o = oracle.Oracle(N, nu=nu, dt=dt, visc_pow=2, integrator=oracle.IFRK4 if integrator == "ifrk4" else oracle.RK4CN)
    s.InitialConditions("SPECTRUM", seed=4, k0=3.0)
    o.ic("SPECTRUM", seed=4, k0=3.0)
    s.RK4Step(10)
    o.step(10)
    assert rel_l2(s.get_state(), o.get_state()) < FP64_TOL


def test_forcing_and_cfl(ns3d, oracle):
    N, nu = 32, 5e-3
    kw = dict(nu=nu, dt=1e-3, cfl=0.5, force_k=2)
    s = ns3d.Solver(N, forcing="SHELL", **kw)
    o = oracle.Oracle(N, forcing=oracle.FORCE_SHELL, **kw)
    s.InitialConditions("SPECTRUM", seed=9, k0=4.0)
    o.ic("SPECTRUM", seed=9, k0=4.0)
    assert abs(s.forcing_target - o.forcing_target) < FP64_TOL * o.forcing_target
    s.RK4Step(10)
    o.step(10)
    assert rel_l2(s.get_state(), o.get_state()) < 1e-11
    t, dt, it = s.get_time()
    rt, rdt, rit = o.get_time()
    assert it == rit == 10 and abs(dt - rdt) < 1e-12 * rdt and abs(t - rt) < 1e-12 * rt
    _, Ek, _ = s.ComputeSystemMeasurables()
    assert abs(Ek[1] + Ek[2] - o.forcing_target) < 1e-11 * o.forcing_target


def test_shapiro_exact_solution_gpu(ns3d):
    # the reference's known-answer test (ShapiroExactSolution, solver.c:1654-1702), D13 fixed
    N, nu, dt, n = 32, 0.05, 1e-3, 50
    s = ns3d.Solver(N, nu=nu, dt=dt)
    s.InitialConditions("SHAPIRO")
    s.RK4Step(n)
    u, _ = s.real_space()
    ex = shapiro_exact(N, n * dt, nu)
    assert np.abs(u[:, :, :N] - ex).max() < 1e-12 * np.abs(ex).max()


def test_real_space_and_dealias(ns3d, oracle):
    N = 32
    s = ns3d.Solver(N)
    o = oracle.Oracle(N)
    s.InitialConditions("SPECTRUM", seed=1)
    o.ic("SPECTRUM", seed=1)
    u, w = s.real_space()
    ru, rw = o.real_space()
    assert rel_l2(u, ru) < FP64_TOL and rel_l2(w, rw) < FP64_TOL
    a = np.random.default_rng(0).standard_normal((N, N, N // 2 + 1, 3)) * (1 + 1j)
    assert np.array_equal(ns3d.ApplyDealiasing(a), o.dealias(a))


def test_step_host_contract(ns3d):
    N = 32
    s = ns3d.Solver(N, nu=0.01, dt=2e-3)
    s.InitialConditions("SPECTRUM", seed=2)
    u0 = s.get_state()
    s.RK4Step(1)
    ref = s.get_state()
    out = np.empty_like(u0)
    s.step_host(u0, out)
    assert np.array_equal(out, ref)


def test_determinism(ns3d):
    N = 48
    res = []
    for _ in range(2):
        s = ns3d.Solver(N, nu=0.01, dt=2e-3, precision="fp32")
        s.InitialConditions("SPECTRUM", seed=21)
        s.RK4Step(5)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        res.append((s.get_state(), tot, Ek))
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1] and np.array_equal(res[0][2], res[1][2])


def test_fp32_vs_fp64_energy(ns3d):
    """Reduced config 2: decaying turbulence, FP32 bulk vs FP64, energy error <= 1e-5."""
    N, nu = 64, 2e-3
    res = {}
    for prec in ("fp64", "fp32"):
        s = ns3d.Solver(N, nu=nu, dt=1e-3, cfl=0.5, precision=prec)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s.RK4Step(200)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        res[prec] = (tot, Ek, s.get_time())
    e64, e32 = res["fp64"][0]["energy"], res["fp32"][0]["energy"]
    assert abs(e32 - e64) / e64 < 1e-5
    d64, d32 = res["fp64"][0]["dissipation"], res["fp32"][0]["dissipation"]
    assert abs(d32 - d64) / d64 < 1e-4


@pytest.mark.parametrize("N,prec,tol", [(192, "fp64", FP64_TOL), (192, "fp32", FP32_TOL), (384, "fp32", FP32_TOL)])
def test_rhs_radix3_sizes(ns3d, oracle, N, prec, tol):
    """Grids with a factor 3 (12 elements per thread, radix-3/6/12 stages): the
    reference accepts any even N (utils.c:88-104)."""
    u = dealiased_random(N, N + 2)
    s = ns3d.Solver(N, precision=prec)
    got = s.NonlinearRHSBatch(u)
    s.close()
    ref = oracle.Oracle(N).rhs(u)
    assert rel_l2(got, ref) < tol


def test_step_radix3_fp64(ns3d, oracle):
    N = 192
    s = ns3d.Solver(N, nu=2e-3, dt=1e-3, precision="fp64", forcing="SHELL", force_k=2)
    o = oracle.Oracle(N, nu=2e-3, dt=1e-3, forcing=oracle.FORCE_SHELL, force_k=2)
    s.InitialConditions("SPECTRUM", seed=3, k0=4.0)
    o.ic("SPECTRUM", seed=3, k0=4.0)
    s.RK4Step(1)
    o.step(1)
    assert rel_l2(s.get_state(), o.get_state()) < FP64_TOL


@pytest.mark.parametrize("N", [256, 512, 768])
def test_large_grid_properties(ns3d, N):
    """Size-independent properties at full sizes: the energy budget of one FP32
    step (dE/dt = -eps for unforced flow), divergence-free and dealiased state,
    Hermitian kz = 0 plane."""
    s = ns3d.Solver(N, nu=1e-3, dt=1e-3, precision="fp32")
    s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
    t0, _, _ = s.ComputeSystemMeasurables()
    s.RK4Step(2)
    t1, _, _ = s.ComputeSystemMeasurables()
    dE = (t1["energy"] - t0["energy"]) / 2e-3
    eps = 0.5 * (t0["dissipation"] + t1["dissipation"])
    assert abs(dE + eps) < 1e-2 * eps
    if N == 256:
        u = s.get_state()
        KX, KY, KZ = kgrid(N)
        div = KX * u[..., 0] + KY * u[..., 1] + KZ * u[..., 2]
        assert np.abs(div).max() < 1e-4 * np.abs(u).max() * N
        assert np.all(u[np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2) > N // 3] == 0)
        p0 = u[:, :, 0]
        pm = np.conj(p0[(-np.arange(N)) % N][:, (-np.arange(N)) % N])
        assert np.abs(p0 - pm).max() < 1e-5 * np.abs(u).max()


def test_fp32_512_tracks_fp64(ns3d):
    """The 512^3 FP32 step (one-warp z lines with FP32x2 butterfly additions, the
    tuned x-pass plan) against the FP64 engine over 3 forced steps from the same
    state: total energy to 1e-6 and every shell of E(k) to 1e-6 of its maximum."""
    N = 512
    res = {}
    for prec in ("fp64", "fp32"):
        s = ns3d.Solver(N, nu=1e-3, dt=1e-3, precision=prec, forcing="SHELL", force_k=2)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s.RK4Step(3)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        res[prec] = (tot["energy"], np.asarray(Ek))
        del s
    e64, k64 = res["fp64"]
    e32, k32 = res["fp32"]
    assert abs(e32 - e64) < 1e-6 * e64
    assert np.max(np.abs(k32 - k64)) < 1e-6 * k64.max()


def test_spectra_match_reference_fixture(ns3d):
    """E(k), Omega(k) and the energy and enstrophy of the FP64 GPU path against
    the reference's own ComputeSystemMeasurables output (tests/golden/ref_N16.npz;
    its spectra carry none of the reference's defects)."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_N16.npz"))
    s = ns3d.Solver(16, nu=0.01, precision="fp64")
    s.set_state(d["uh"])
    tot, Ek, Ok = s.ComputeSystemMeasurables()
    assert rel_l2(Ek, d["Ek"]) < FP64_TOL and rel_l2(Ok, d["Ok"]) < FP64_TOL
    assert abs(tot["energy"] - d["Ek"].sum()) <= FP64_TOL * tot["energy"]
    assert abs(tot["enstrophy"] - d["Ok"].sum()) <= FP64_TOL * tot["enstrophy"]
