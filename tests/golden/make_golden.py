"""Generate the golden fixtures in tests/golden/ with an independent numpy
restatement of the reference solver's hot path (Solver/src/solver.c).

This is a second, independent restatement (numpy.fft / pocketfft instead of
the oracle's own FFT, vectorised array algebra instead of loops). The C oracle
is checked against these files in tests/test_oracle_golden.py, so two
independent readings of solver.c must agree before the oracle is trusted.

Run: python tests/golden/make_golden.py   (writes golden_N{8,12}.npz)
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def wavenumbers(N):
    # InitializeSpaceVariables, solver.c:1786-1823
    kx = np.array([i if i <= N // 2 else i - N for i in range(N)], dtype=np.float64)
    kz = np.arange(N // 2 + 1, dtype=np.float64)
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    return KX, KY, KZ


def dealias(a, N):
    # ApplyDealiasing, solver.c:1709-1756 (2/3 rule, D2 fixed)
    KX, KY, KZ = wavenumbers(N)
    mask = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2) > (N // 3)
    a = a.copy()
    a[mask] = 0
    return a


def c2r(uh, N):
    # unnormalised batched c2r (solver.c:656-658)
    return np.fft.irfftn(uh, s=(N, N, N), axes=(0, 1, 2)) * N ** 3


def r2c(u, N):
    return np.fft.rfftn(u, axes=(0, 1, 2))


def curl(uh, N):
    KX, KY, KZ = wavenumbers(N)
    w = np.empty_like(uh)
    w[..., 0] = 1j * (KY * uh[..., 2] - KZ * uh[..., 1])
    w[..., 1] = 1j * (KZ * uh[..., 0] - KX * uh[..., 2])
    w[..., 2] = 1j * (KX * uh[..., 1] - KY * uh[..., 0])
    return w


def rhs(uh, N):
    # NonlinearRHSBatch, solver.c:620-731
    KX, KY, KZ = wavenumbers(N)
    w = c2r(curl(uh, N), N)
    u = c2r(uh, N)
    nl = np.cross(u, w, axis=-1)
    nh = r2c(nl, N) / float(N ** 3) ** 2
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    kdn = KX * nh[..., 0] + KY * nh[..., 1] + KZ * nh[..., 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        kinv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    for d, K in enumerate((KX, KY, KZ)):
        nh[..., d] = np.where(k2 > 0, nh[..., d] - K * kinv * kdn, 0.0)
    return dealias(nh, N)


def visc(N, nu, vp):
    KX, KY, KZ = wavenumbers(N)
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    return (nu * (k2 ** 2 if vp == 2 else k2))[..., None]


def step_ifrk4(uh, N, nu, h, vp=1):
    # Lawson integrating-factor RK4
    L = visc(N, nu, vp)
    E = np.exp(-0.5 * h * L)
    k1 = rhs(uh, N)
    k2 = rhs(E * (uh + 0.5 * h * k1), N)
    k3 = rhs(E * uh + 0.5 * h * k2, N)
    k4 = rhs(E * E * uh + h * E * k3, N)
    return E * E * uh + h / 6.0 * (E * E * k1 + 2.0 * E * (k2 + k3) + k4)


def step_rk4cn(uh, N, nu, h, vp=1):
    # RK4Step with the Crank–Nicolson factor, solver.c:505-608
    D = h * visc(N, nu, vp)
    k1 = rhs(uh, N)
    k2 = rhs(uh + 0.5 * h * k1, N)
    k3 = rhs(uh + 0.5 * h * k2, N)
    k4 = rhs(uh + h * k3, N)
    return uh * ((2 - D) / (2 + D)) + (2 * h / (2 + D)) * (k1 / 6 + k2 / 3 + k3 / 3 + k4 / 6)


# Dormand & Prince (1980) RK5(4)7M; the reference's table (solver.c:34-42)
# has a32 = 1/2 where the published scheme has 9/40 (defect D19, fixed)
DP_A = [[], [1 / 5], [3 / 40, 9 / 40], [44 / 45, -56 / 15, 32 / 9],
        [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
        [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
        [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]]
DP_B = [35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84, 0]
DP_BS = [5179 / 57600, 0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40]


def rk5_attempt(uh, N, nu, h, dp, vp=1, atol=1e-7, rtol=1e-7):
    # RK5DPStep, solver.c:217-421: explicit stages on N(u), Crank–Nicolson
    # factor in the update; dp adds the 7th stage and the embedded error
    D = h * visc(N, nu, vp)
    ks = [rhs(uh, N)]
    for s in range(1, 7 if dp else 6):
        ks.append(rhs(uh + h * sum(a * k for a, k in zip(DP_A[s], ks)), N))
    a, b = (2 - D) / (2 + D), 2 * h / (2 + D)
    un = uh * a + b * sum(c * k for c, k in zip(DP_B, ks))
    if not dp:
        return un, None
    diff = b * sum((c - cs) * k for c, cs, k in zip(DP_B, DP_BS, ks))
    den = atol + np.maximum(np.abs(uh), np.abs(un)) * rtol
    err = np.sqrt(np.sum(np.abs(diff / den) ** 2, axis=(0, 1, 2)) / (N * N * (N // 2 + 1))).max()
    return un, err


def dp5_step(uh, N, nu, h):
    # adaptive loop (solver.c:134-154, D15/D18 fixed): retry from uh until err <= 1
    rejects = 0
    while True:
        un, err = rk5_attempt(uh, N, nu, h, True)
        hn = h * min(1.5, max(0.01, 0.8 * (1.0 / err) ** 0.2))
        if err <= 1.0:
            return un, h, hn, err, rejects
        rejects += 1
        h = hn


def measurables(uh, N, nu, vp=1):
    # ComputeSystemMeasurables, solver.c:1142-1276 (D4 fixed)
    KX, KY, KZ = wavenumbers(N)
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    w = curl(uh, N)
    c = curl(w, N)
    m = np.full(k2.shape, 2.0)
    m[:, :, 0] = 1.0
    m[:, :, -1] = 1.0
    nf = 0.5 / float(N ** 3) ** 2
    cf = 8.0 * np.pi ** 3
    eu = np.sum(np.abs(uh) ** 2, axis=-1)
    ew = np.sum(np.abs(w) ** 2, axis=-1)
    ec = np.sum(np.abs(c) ** 2, axis=-1)
    hel = np.real(np.sum(uh * np.conj(w), axis=-1))   # D12 fixed: Parseval form of u.w
    pre = nu * (k2 ** 2 if vp == 2 else k2)
    tot = np.array([np.sum(m * eu), np.sum(m * ew), np.sum(m * ec), np.sum(m * hel),
                    2.0 * np.sum(m * pre * eu)]) * cf * nf
    ns = int(np.sqrt(3.0 * (N / 2.0) ** 2)) + 1
    b = np.rint(np.sqrt(k2)).astype(int)
    Ek = np.bincount(b.ravel(), weights=(m * eu).ravel() * cf * nf, minlength=ns)[:ns]
    Ok = np.bincount(b.ravel(), weights=(m * ew).ravel() * cf * nf, minlength=ns)[:ns]
    return tot, Ek, Ok


def random_field(N, seed):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((N, N, N, 3))
    return dealias(r2c(u, N), N)


def make(N, nu=0.05, h=1e-2, seed=1234):
    u0 = random_field(N, seed)
    out = dict(N=N, nu=nu, dt=h, u0=u0, rhs=rhs(u0, N))
    out["ifrk4_1"] = step_ifrk4(u0, N, nu, h)
    u = u0
    for _ in range(10):
        u = step_ifrk4(u, N, nu, h)
    out["ifrk4_10"] = u
    out["rk4cn_1"] = step_rk4cn(u0, N, nu, h)
    out["ifrk4_hyper_1"] = step_ifrk4(u0, N, nu * 1e-2, h, vp=2)
    out["rk5cn_1"] = rk5_attempt(u0, N, nu, h, False)[0]
    # a first step 30x too long: rejected, then accepted with a shorter step
    un, h_used, h_next, err, rej = dp5_step(u0, N, nu, 30 * h)
    out.update(dp5_1=un, dp5_h_used=h_used, dp5_h_next=h_next, dp5_err=err, dp5_rejects=rej)
    tot, Ek, Ok = measurables(u0, N, nu)
    out.update(tot=tot, Ek=Ek, Ok=Ok)
    return out


if __name__ == "__main__":
    for N in (8, 12):
        d = make(N)
        np.savez_compressed(os.path.join(HERE, f"golden_N{N}.npz"), **d)
        print("wrote", N, {k: np.asarray(v).shape for k, v in d.items()})
