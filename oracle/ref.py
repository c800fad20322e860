"""ORACLE: test infrastructure only, never product code.

ctypes wrapper over ``oracle/_ref/libns3d_ref_{nu,hyper}.so``: the reference's
own ``Solver/src/solver.c`` and ``utils.c``, compiled unchanged against the
single-rank MPI / FFTW-MPI stand-ins of ``oracle/ref_shim`` (recipe:
``make -C oracle ref``). The two libraries are the reference's two build
variants (Solver/Makefile:44-52): ``hyper`` = ``-D__NAVIER -D__HYPER``
(viscosity nu k^4, its default ``solver`` target) and ``nu`` =
``-D__NAVIER -D__TESTING -D__DEBUG`` (nu k^2, its ``solver_test`` target).

Only the CPU parity tests load it; it needs the reference sources to build,
so it exists only where they do.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.path.join(_HERE, "_ref")
_libs: dict = {}


def build() -> bool:
    """Build both variants; False when the reference sources are absent."""
    r = subprocess.run(["make", "-s", "-C", _HERE, "ref"], capture_output=True, text=True)
    return r.returncode == 0 and all(os.path.exists(path(v)) for v in ("nu", "hyper"))


def path(variant: str) -> str:
    return os.path.join(_REF_DIR, f"libns3d_ref_{variant}.so")


def _load(variant: str):
    if variant in _libs:
        return _libs[variant]
    L = ctypes.CDLL(path(variant), mode=ctypes.RTLD_LOCAL)
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    ARGV = ctypes.POINTER(ctypes.c_char_p)
    L.ref_create.argtypes = [ctypes.c_int, ARGV]
    L.ref_create.restype = ctypes.c_int
    L.ref_spectral_solve.argtypes = [ctypes.c_int, ARGV, D, ctypes.c_int, D]
    L.ref_spectral_solve.restype = ctypes.c_int
    L.ref_n_spect.restype = ctypes.c_int
    L.ref_local_nx.restype = ctypes.c_long
    L.ref_hyper.restype = ctypes.c_int
    L.ref_set_state.argtypes = [D]
    L.ref_get_state.argtypes = [D]
    L.ref_rhs.argtypes = [D, D, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_rk4_step.argtypes = [ctypes.c_double, ctypes.c_int]
    L.ref_dealias.argtypes = [D, ctypes.c_int]
    L.ref_measurables.argtypes = [D, D, D]
    L.ref_space.argtypes = [I, I, I, D, D, D]
    L.ns3d_ref_shim_d1_substitutions.restype = ctypes.c_int
    _libs[variant] = L
    return L


def _dp(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _argv(args):
    enc = [b"solver"] + [str(a).encode() for a in args]
    arr = (ctypes.c_char_p * len(enc))(*enc)
    return len(enc), arr


def flags(N, nu, dt, T, u0, save_every=100, t0=0.0):
    """The reference binary's command line (utils.c:74)."""
    return ["-n", N, "-n", N, "-n", N, "-s", repr(float(t0)), "-e", repr(float(T)), "-h", repr(float(dt)),
            "-v", repr(float(nu)), "-i", u0, "-p", save_every]


def n_spect(N: int) -> int:
    # InitializeSystemMeasurables, solver.c:1384 (cubic)
    return int(np.sqrt(3.0 * (N / 2.0) ** 2)) + 1


class Reference:
    """The reference's hot-path functions over its own global state (one
    instance at a time per variant: solver.c works on process globals)."""

    def __init__(self, N, nu=1.0, dt=1e-3, T=1.0, u0="TESTING", variant="nu", save_every=100):
        self.N = N
        self.L = _load(variant)
        self._argv = _argv(flags(N, nu, dt, T, u0, save_every))
        self.L.ref_create(*self._argv)

    @property
    def fshape(self):
        return (self.N, self.N, self.N // 2 + 1, 3)

    @property
    def rshape(self):
        return (self.N, self.N, self.N + 2, 3)

    def close(self):
        self.L.ref_destroy()

    def initial_conditions(self):
        self.L.ref_initial_conditions()

    def set_state(self, u_hat):
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        self.L.ref_set_state(_dp(u.view(np.float64)))

    def get_state(self):
        u = np.empty(self.fshape, np.complex128)
        self.L.ref_get_state(_dp(u.view(np.float64)))
        return u

    def rhs(self, u_hat, real_fields=False):
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        out = np.empty(self.fshape, np.complex128)
        vel = np.empty(self.rshape) if real_fields else None
        vort = np.empty(self.rshape) if real_fields else None
        self.L.ref_rhs(_dp(u.view(np.float64)), _dp(out.view(np.float64)),
                       vel.ctypes.data if real_fields else None, vort.ctypes.data if real_fields else None)
        return (out, vel, vort) if real_fields else out

    def rk4_step(self, dt, n=1):
        self.L.ref_rk4_step(dt, n)

    def dealias(self, arr):
        a = np.array(arr, dtype=np.complex128, order="C", copy=True)
        dim = a.shape[-1] if a.ndim == 4 else 1
        self.L.ref_dealias(_dp(a.view(np.float64)), dim)
        return a

    def measurables(self):
        ns = self.L.ref_n_spect()
        tot, Ek, Ok = np.zeros(5), np.zeros(ns), np.zeros(ns)
        self.L.ref_measurables(_dp(tot), _dp(Ek), _dp(Ok))
        return tot, Ek, Ok

    def space(self):
        N = self.N
        kx, ky, kz = (np.zeros(N, np.int32), np.zeros(N, np.int32), np.zeros(N // 2 + 1, np.int32))
        x, y, z = np.zeros(N), np.zeros(N), np.zeros(N)
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self.L.ref_space(ip(kx), ip(ky), ip(kz), _dp(x), _dp(y), _dp(z))
        return (kx, ky, kz), (x, y, z)


def spectral_solve(N, nu, dt, T, u0, save_every, variant="nu", max_rows=1000):
    """Run the reference program (SpectralSolve, solver.c:50-208) end to end.
    Returns (rows, u_hat_final); each row is
    [t, E, Omega, P, H, eps, Ek[n_spect], Ok[n_spect]]."""
    L = _load(variant)
    ns = n_spect(N)
    series = np.zeros((max_rows, 6 + 2 * ns))
    final = np.zeros((N, N, N // 2 + 1, 3), np.complex128)
    argv = _argv(flags(N, nu, dt, T, u0, save_every))
    rows = L.ref_spectral_solve(argv[0], argv[1], _dp(series), max_rows, _dp(final.view(np.float64)))
    return series[:rows], final


def d1_substitutions(variant="nu") -> int:
    return _load(variant).ns3d_ref_shim_d1_substitutions()
