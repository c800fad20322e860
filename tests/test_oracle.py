"""CPU tests of the oracle (the checker for the GPU path): its FFT against
numpy.fft and a direct DFT, its hot path against the independent numpy
restatement in tests/golden/, and the reference's known answers
(Shapiro exact solution, solver.c:1654-1702; Taylor–Green invariants)."""
import os

import numpy as np
import pytest
from helpers import shapiro_exact

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 8, 10, 12, 16, 24, 30, 48, 64, 96, 128, 512])
def test_fft1d_vs_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(oracle.fft1d(x), np.fft.fft(x)) < 1e-14
    assert rel(oracle.fft1d(x, inverse=True), np.fft.ifft(x) * n) < 1e-14


@pytest.mark.parametrize("n", [6, 12, 20])
def test_fft1d_vs_direct_dft(oracle, n):
    x = np.random.default_rng(7).standard_normal(n) + 0j
    k = np.arange(n)
    D = np.exp(-2j * np.pi * np.outer(k, k) / n)
    assert rel(oracle.fft1d(x), D @ x) < 1e-13


@pytest.mark.parametrize("N", [8, 12, 16])
def test_r2c_c2r_vs_numpy(oracle, N):
    o = oracle.Oracle(N)
    r = np.zeros((N, N, N + 2, 3))
    r[:, :, :N] = np.random.default_rng(N).standard_normal((N, N, N, 3))
    uh = o.r2c(r)
    ref = np.fft.rfftn(r[:, :, :N], axes=(0, 1, 2))
    assert rel(uh, ref) < 1e-14
    back = o.c2r(uh)
    assert rel(back[:, :, :N] / N ** 3, r[:, :, :N]) < 1e-14
    assert np.all(back[:, :, N:] == 0)


def test_c2r_ignores_antihermitian_dc(oracle):
    # c2r semantics of the kz = 0 plane: imaginary parts of the z-DC entry are ignored
    N = 8
    o = oracle.Oracle(N)
    uh = np.zeros((N, N, N // 2 + 1, 3), complex)
    uh[1, 2, 0, 0] = 1.0 + 0.5j     # no conjugate partner at (-1,-2,0)
    r = o.c2r(uh)[:, :, :N, 0]
    ref = np.fft.irfftn(uh[..., 0], s=(N, N, N), axes=(0, 1, 2)) * N ** 3
    assert rel(r, ref) < 1e-14


@pytest.mark.parametrize("N", [8, 12])
def test_oracle_vs_numpy_golden(oracle, N):
    d = np.load(os.path.join(GOLD, f"golden_N{N}.npz"))
    nu, dt = float(d["nu"]), float(d["dt"])
    o = oracle.Oracle(N, nu=nu, dt=dt)
    assert rel(o.rhs(d["u0"]), d["rhs"]) < 1e-13
    o.set_state(d["u0"]); o.step(1)
    assert rel(o.get_state(), d["ifrk4_1"]) < 1e-13
    o.set_state(d["u0"]); o.step(10)
    assert rel(o.get_state(), d["ifrk4_10"]) < 1e-13
    o2 = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK4CN)
    o2.set_state(d["u0"]); o2.step(1)
    assert rel(o2.get_state(), d["rk4cn_1"]) < 1e-13
    o3 = oracle.Oracle(N, nu=nu * 1e-2, dt=dt, visc_pow=2)
    o3.set_state(d["u0"]); o3.step(1)
    assert rel(o3.get_state(), d["ifrk4_hyper_1"]) < 1e-13
    o.set_state(d["u0"])
    tot, Ek, Ok = o.measurables()
    assert np.allclose(tot, d["tot"], rtol=1e-13, atol=1e-13 * abs(tot[0]))
    assert rel(Ek, d["Ek"]) < 1e-13 and rel(Ok, d["Ok"]) < 1e-13


@pytest.mark.parametrize("N", [16, 32, 64])
def test_taylor_green_invariants(oracle, N):
    # u = (sin x cos y cos z, -cos x sin y cos z, 0): E = pi^3, Omega = 3 pi^3 (reference normalisation)
    o = oracle.Oracle(N, nu=1 / 400, dt=1e-3)
    o.ic("TAYLOR_GREEN")
    tot, Ek, Ok = o.measurables()
    assert abs(tot[0] / np.pi ** 3 - 1) < 1e-13
    assert abs(tot[1] / np.pi ** 3 - 3) < 1e-13
    assert abs(Ek[2] / np.pi ** 3 - 1) < 1e-13    # all energy in shell round(sqrt 3) = 2
    assert abs(tot[4] - 2 * (1 / 400) * 3 * np.pi ** 3) / tot[4] < 1e-13   # eps = 2 nu Omega


def test_taylor_green_bugcompat_energy(oracle):
    # defect D4 reproduced: the reference's saved TotalEnergy of TG at t = 0 is 0.75 pi^3
    o = oracle.Oracle(16, bugcompat_measures=True)
    o.ic("TAYLOR_GREEN")
    tot, _, _ = o.measurables()
    assert abs(tot[0] / np.pi ** 3 - 0.75) < 1e-13


@pytest.mark.parametrize("integrator,tol", [("ifrk4", 1e-12), ("rk4cn", 1e-6)])
def test_shapiro_known_answer(oracle, integrator, tol):
    # the reference's own known-answer test: Beltrami flow, u x w = 0, exact decay
    N, nu, dt, n = 16, 0.05, 1e-3, 20
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.IFRK4 if integrator == "ifrk4" else oracle.RK4CN)
    o.ic("SHAPIRO")
    assert np.abs(o.rhs(o.get_state())).max() < 1e-9 * np.abs(o.get_state()).max()
    o.step(n)
    u, _ = o.real_space()
    ex = shapiro_exact(N, n * dt, nu)
    assert np.abs(u[:, :, :N] - ex).max() < tol * np.abs(ex).max()


def test_ifrk4_fourth_order(oracle):
    N, nu = 12, 0.02
    d = np.load(os.path.join(GOLD, "golden_N12.npz"))
    u0 = d["u0"] / np.abs(d["u0"]).max() * 50.0
    T = 0.08

    def run(h):
        o = oracle.Oracle(N, nu=nu, dt=h)
        o.set_state(u0)
        o.step(int(round(T / h)))
        return o.get_state()

    ref = run(T / 64)
    e1 = np.abs(run(T / 4) - ref).max()
    e2 = np.abs(run(T / 8) - ref).max()
    assert 12 < e1 / e2 < 20     # 2^4 = 16


def test_dealias_and_bugcompat(oracle):
    N = 12
    a = np.random.default_rng(3).standard_normal((N, N, N // 2 + 1, 3)) * (1 + 0j)
    o = oracle.Oracle(N)
    b = o.dealias(a)
    k = np.array([i if i <= N // 2 else i - N for i in range(N)])
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
    keep = np.sqrt(K2) <= N // 3
    assert np.all(b[~keep] == 0) and np.all(b[keep] == a[keep])
    ob = oracle.Oracle(N, bugcompat_dealias=True)
    assert not np.array_equal(ob.dealias(a), b)    # D2 reproduced


def test_spectrum_ic_properties(oracle):
    N = 24
    o = oracle.Oracle(N)
    o.ic("SPECTRUM", seed=5, k0=4.0, energy=1.0)
    u = o.get_state()
    tot, Ek, _ = o.measurables()
    assert abs(tot[0] / (8 * np.pi ** 3) - 1) < 1e-13           # unit energy: 0.5 <|u|^2> = 1
    k = np.array([i if i <= N // 2 else i - N for i in range(N)])
    KX, KY, KZ = np.meshgrid(k, k, np.arange(N // 2 + 1), indexing="ij")
    div = KX * u[..., 0] + KY * u[..., 1] + KZ * u[..., 2]
    assert np.abs(div).max() < 1e-12 * np.abs(u).max()           # solenoidal
    p0 = u[:, :, 0]                                                # Hermitian kz = 0 plane
    pm = p0[(-np.arange(N)) % N][:, (-np.arange(N)) % N]
    assert np.abs(p0 - np.conj(pm)).max() < 1e-12 * np.abs(u).max()
    r, _ = o.real_space()
    assert abs(0.5 * np.mean(np.sum(r[:, :, :N] ** 2, -1)) - 1) < 1e-12   # Parseval
    o2 = oracle.Oracle(N)
    o2.ic("SPECTRUM", seed=5, k0=4.0, energy=1.0)
    assert np.array_equal(o2.get_state(), u)                       # seeded, reproducible


def test_forcing_holds_low_shell_energy(oracle):
    N = 16
    o = oracle.Oracle(N, nu=0.02, dt=5e-3, forcing=oracle.FORCE_SHELL, force_k=2)
    o.ic("SPECTRUM", seed=1, k0=3.0, energy=1.0)
    e0 = o.forcing_target
    o.step(5)
    _, Ek, _ = o.measurables()
    assert abs(Ek[1] + Ek[2] - e0) < 1e-12 * e0


def test_cfl_step(oracle):
    N, cfl = 16, 0.5
    o = oracle.Oracle(N, nu=0.02, dt=1e-3, cfl=cfl)
    o.ic("SPECTRUM", seed=2, k0=3.0, energy=1.0)
    umax = o.max_speed_sum()
    r, _ = o.real_space()
    assert abs(umax - np.abs(r[:, :, :N]).sum(-1).max()) < 1e-12 * umax
    o.ic("SPECTRUM", seed=2, k0=3.0, energy=1.0)
    o.step(1)
    t, dt, it = o.get_time()
    assert it == 1 and abs(dt - cfl * (2 * np.pi / N) / umax) < 1e-12 * dt and abs(t - dt) < 1e-15


@pytest.mark.parametrize("N", [8, 12])
def test_oracle_rk5_vs_numpy_golden(oracle, N):
    d = np.load(os.path.join(GOLD, f"golden_N{N}.npz"))
    nu, dt = float(d["nu"]), float(d["dt"])
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK5CN)
    o.set_state(d["u0"]); o.step(1)
    assert rel(o.get_state(), d["rk5cn_1"]) < 1e-13
    dp = oracle.Oracle(N, nu=nu, dt=30 * dt, integrator=oracle.DP5CN)
    dp.set_state(d["u0"]); dp.step(1)
    assert rel(dp.get_state(), d["dp5_1"]) < 1e-13
    err, rejects = dp.dp_stats()
    t, h_next, iters = dp.get_time()
    assert rejects == int(d["dp5_rejects"]) and iters == 1
    # the error norm is a difference of two solutions: relative agreement ~1e-10
    assert abs(err - float(d["dp5_err"])) < 1e-9 * float(d["dp5_err"])
    # step sizes follow err^(-1/5)
    assert abs(t / float(d["dp5_h_used"]) - 1) < 1e-10 and abs(h_next / float(d["dp5_h_next"]) - 1) < 1e-10


def _order_runs(oracle, integrator, bugcompat=False):
    # nu = 0: the Crank–Nicolson factor is 1 and the stepper is the plain explicit scheme
    N = 12
    d = np.load(os.path.join(GOLD, "golden_N12.npz"))
    u0 = d["u0"] / np.abs(d["u0"]).max() * 200.0
    T = 0.08

    def run(h):
        o = oracle.Oracle(N, nu=0.0, dt=h, integrator=integrator, bugcompat_rk5=bugcompat)
        o.set_state(u0)
        o.step(int(round(T / h)))
        return o.get_state()

    ref = run(T / 64)
    return np.abs(run(T / 4) - ref).max() / np.abs(run(T / 8) - ref).max()


def test_rk5cn_fifth_order(oracle):
    # published tableau: 2^5 = 32; the reference's a32 = 1/2 (D19) loses consistency
    assert 25 < _order_runs(oracle, oracle.RK5CN) < 40
    assert _order_runs(oracle, oracle.RK5CN, bugcompat=True) < 5


def test_dp5_adaptive_control(oracle):
    # step-size control on a Taylor–Green run: the error of every accepted step
    # is <= 1, steps grow by at most 1.5x and a too-long first step is rejected
    o = oracle.Oracle(16, nu=0.01, dt=0.5, integrator=oracle.DP5CN, dp_atol=1e-9, dp_rtol=1e-9)
    o.ic("TAYLOR_GREEN")
    E0 = o.measurables()[0][0]
    hs = []
    for _ in range(6):
        t0 = o.get_time()[0]
        o.step(1)
        err, _ = o.dp_stats()
        assert err <= 1.0
        hs.append(o.get_time()[0] - t0)
    assert o.dp_stats()[1] >= 1
    assert all(b <= 1.5 * a * (1 + 1e-12) for a, b in zip(hs, hs[1:]))
    t = o.get_time()[0]
    # Taylor–Green at early times: E(t) ~ E0 exp(-6 nu t)
    assert abs(o.measurables()[0][0] / (E0 * np.exp(-6 * 0.01 * t)) - 1) < 5e-3


def test_increment_stats_vs_numpy(oracle):
    """The oracle's increment statistics (PostProcessing/src/stats.c) against an
    independent numpy computation on the same real-space field."""
    N, nb = 16, 50
    o = oracle.Oracle(N, nu=0.01)
    o.ic("SPECTRUM", seed=6, k0=3.0)
    got = o.increment_stats([1, 3, 8, 16], n_bins=nb)
    u, _ = o.real_space()
    u = u[:, :, :N, :]
    for r, dr in enumerate([1, 3, 8, 16]):
        d = np.concatenate([(u[dr:, :, :, 0] - u[:-dr, :, :, 0]).ravel() if dr < N else np.zeros(0),
                            (u[:, dr:, :, 1] - u[:, :-dr, :, 1]).ravel() if dr < N else np.zeros(0),
                            (u[:, :, dr:, 2] - u[:, :, :-dr, 2]).ravel() if dr < N else np.zeros(0)])
        st = got["stats"][r]
        if d.size == 0:
            assert np.all(st == 0) and np.all(got["counts"][r] == 0)
            continue
        n, m = d.size, d.mean()
        sd = d.std(ddof=1)
        ref = [d.min(), d.max(), m, sd, np.mean((d - m) ** 3) / sd ** 3, np.mean((d - m) ** 4) / sd ** 4 - 3]
        assert np.allclose(st, ref, rtol=1e-10, atol=1e-12)
        lo, hi = d.min() - 0.05, d.max() + 0.05
        b = np.arange(nb + 1)
        edges = ((nb - b) / nb) * lo + (b / nb) * hi
        assert np.array_equal(got["ranges"][r], edges)
        idx = np.searchsorted(edges, d, side="right") - 1
        assert np.array_equal(got["counts"][r], np.bincount(idx, minlength=nb)[:nb].astype(float))
