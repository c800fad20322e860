"""The oracle against the reference's own code.

``oracle/_ref`` is the reference's ``Solver/src/solver.c`` and ``utils.c``
compiled unchanged against single-rank MPI / FFTW-MPI stand-ins
(``oracle/ref_shim``); both of the reference's build variants are built
(``nu``: ``-D__NAVIER -D__TESTING -D__DEBUG``, nu k^2; ``hyper``:
``-D__NAVIER -D__HYPER``, nu k^4; Solver/Makefile:44-52). The oracle runs
with its bug-compatibility flags for the defects the reference's code carries
(D2 dealias aliasing, solver.c:1741; D4 precedence and D12 helicity,
solver.c:1227-1235; D13 Shapiro w, solver.c:1593), and must then agree with
the reference to 1e-12 relative L2 (integer work — wavenumbers, the dealias
mask, spectrum bins — bit for bit). The parts the defects do not touch are
also held to the fixed oracle: the dealias mask through ApplyDealiasing with
array_dim = 1 (where the D2 copy is the identity), the spectra E(k), Omega(k)
(no D4 in solver.c:1240-1262) and the real-space fields of the transposed
FFTW plans. These tests need the reference sources and are skipped without
them; tests/test_reference_golden.py holds the oracle to fixtures made from the
reference where the sources are absent.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref as R

TOL = 1e-12


def rel(a, b):
    n = np.linalg.norm(np.ravel(b))
    return float(np.linalg.norm(np.ravel(a - b)) / (n if n > 0 else 1.0))


@pytest.fixture(scope="module")
def built():
    if not R.build():
        pytest.skip("reference sources not present: oracle/_ref cannot be built here")
    return True


def field(N, seed, dealias=True):
    rng = np.random.default_rng(seed)
    uh = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    if dealias:
        k = np.fft.fftfreq(N, 1.0 / N)
        K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
        uh[np.sqrt(K2) > N // 3] = 0
    return uh


@pytest.mark.parametrize("N", [16, 32, 64])
def test_space_variables(built, N):
    r = R.Reference(N)
    (kx, ky, kz), (x, y, z) = r.space()
    r.close()
    k = np.array([i if i <= N // 2 else i - N for i in range(N)], np.int32)
    assert np.array_equal(kx, k) and np.array_equal(ky, k)
    assert np.array_equal(kz, np.arange(N // 2 + 1, dtype=np.int32))
    grid = np.arange(N) * (2.0 * np.pi / N)
    assert np.array_equal(x, grid) and np.array_equal(y, grid) and np.array_equal(z, grid)


def test_d1_substitution_on_the_hot_path_plans(built):
    before = R.d1_substitutions("nu")
    R.Reference(16).close()
    # the two transposed batch plans of solver.c:2067-2068 ask for {N, N, N/2+1}
    assert R.d1_substitutions("nu") - before == 2


@pytest.mark.parametrize("N", [16, 32, 64])
def test_dealias(built, N):
    r = R.Reference(N)
    raw = field(N, N, dealias=False)
    ob = O.Oracle(N, bugcompat_dealias=True)
    of = O.Oracle(N)
    # the reference's 3-component dealias carries D2: bit-equal to the oracle's bug-compatible form
    assert np.array_equal(r.dealias(raw), ob.dealias(raw))
    # per component (array_dim = 1, where the D2 copy is the identity): the mask itself, bit-equal
    per = np.stack([r.dealias(np.ascontiguousarray(raw[..., d])) for d in range(3)], -1)
    assert np.array_equal(per, of.dealias(raw))
    r.close()


@pytest.mark.parametrize("N", [16, 32, 64])
def test_nonlinear_rhs(built, N):
    r = R.Reference(N, nu=0.01)
    ob = O.Oracle(N, nu=0.01, bugcompat_dealias=True)
    of = O.Oracle(N, nu=0.01)
    uh = field(N, 100 + N)
    out, vel, vort = r.rhs(uh, real_fields=True)
    assert rel(out, ob.rhs(uh)) <= TOL
    # FFTW_MPI_TRANSPOSED_IN: the reference's real arrays hold u(x, y, z) at [y][x][z]
    u_nat = of.c2r(uh)[:, :, :N]
    assert rel(vel[:, :, :N].transpose(1, 0, 2, 3), u_nat) <= TOL
    k = np.fft.fftfreq(N, 1.0 / N)
    kk = np.stack(np.meshgrid(k, k, np.arange(N // 2 + 1), indexing="ij"), -1)
    w_hat = 1j * np.cross(kk, uh)
    assert rel(vort[:, :, :N].transpose(1, 0, 2, 3), of.c2r(w_hat)[:, :, :N]) <= TOL
    r.close()


@pytest.mark.parametrize("variant,visc_pow", [("nu", 1), ("hyper", 2)])
@pytest.mark.parametrize("N", [16, 32])
def test_rk4step(built, N, variant, visc_pow):
    nu, dt = 0.02, 2e-3
    r = R.Reference(N, nu=nu, dt=dt, variant=variant)
    ob = O.Oracle(N, nu=nu, dt=dt, integrator=O.RK4CN, visc_pow=visc_pow, bugcompat_dealias=True)
    uh = field(N, 200 + N)
    r.set_state(uh)
    ob.set_state(uh)
    r.rk4_step(dt, 3)
    ob.step(3)
    assert rel(r.get_state(), ob.get_state()) <= TOL
    r.close()


@pytest.mark.parametrize("variant,visc_pow", [("nu", 1), ("hyper", 2)])
@pytest.mark.parametrize("N", [16, 32, 64])
def test_measurables(built, N, variant, visc_pow):
    nu = 0.01
    r = R.Reference(N, nu=nu, variant=variant)
    ob = O.Oracle(N, nu=nu, visc_pow=visc_pow, bugcompat_measures=True)
    of = O.Oracle(N, nu=nu, visc_pow=visc_pow)
    uh = field(N, 300 + N)
    for x in (r, ob, of):
        x.set_state(uh)
    tr, Ekr, Okr = r.measurables()
    tb, _, _ = ob.measurables()
    tf, Ekf, Okf = of.measurables()
    assert len(Ekr) == O.n_spect(N) == R.n_spect(N)
    assert rel(tr, tb) <= TOL                      # totals carry D4 / D12
    assert rel(Ekr, Ekf) <= TOL and rel(Okr, Okf) <= TOL   # spectra do not
    assert abs(tf[0] - Ekr.sum()) <= TOL * tf[0]   # the fixed energy is the sum of the reference's E(k)
    assert abs(tf[1] - Okr.sum()) <= TOL * tf[1]
    r.close()


@pytest.mark.parametrize("N", [16, 32])
def test_initial_conditions(built, N):
    ob = O.Oracle(N, nu=0.01, bugcompat_dealias=True, bugcompat_measures=True)
    for name in ("SHAPIRO", "RANDOM", "TESTING"):
        r = R.Reference(N, nu=0.01, u0=name)
        r.initial_conditions()
        ob.ic(name)
        a, b = r.get_state(), ob.get_state()
        if name == "TESTING":
            assert not np.any(a) and not np.any(b)
        else:
            assert rel(a, b) <= TOL, name
        r.close()
    # D3: the reference's TAYLOR_GREEN branch is followed by the random fill
    r = R.Reference(N, nu=0.01, u0="TAYLOR_GREEN")
    r.initial_conditions()
    ob.ic("RANDOM")
    assert rel(r.get_state(), ob.get_state()) <= TOL
    r.close()


@pytest.mark.parametrize("variant,visc_pow", [("nu", 1), ("hyper", 2)])
def test_spectral_solve_end_to_end(built, variant, visc_pow):
    """The reference program's time loop (SpectralSolve, solver.c:50-208): its
    saved measurables every 5 iterations and its final state."""
    N, dt, nu, every = 16, 1.0 / 1024, 0.05, 5
    T = 20 * dt
    rows, final = R.spectral_solve(N, nu, dt, T, "RANDOM", every, variant=variant)
    assert rows.shape[0] == 5
    ob = O.Oracle(N, nu=nu, dt=dt, integrator=O.RK4CN, visc_pow=visc_pow, bugcompat_dealias=True,
                  bugcompat_measures=True)
    ob.ic("RANDOM")
    ns = O.n_spect(N)
    for i, row in enumerate(rows):
        if i:
            ob.step(every)
        assert row[0] == pytest.approx(i * every * dt, rel=1e-15)
        tot, Ek, Ok = ob.measurables()
        assert rel(row[1:6], tot) <= TOL
        assert rel(row[6:6 + ns], Ek) <= TOL and rel(row[6 + ns:], Ok) <= TOL
    assert rel(final, ob.get_state()) <= TOL
