"""ORACLE: test infrastructure only, never product code.

ctypes wrapper over the CPU FP64 restatement of the reference solver's
time-stepping hot path (oracle/ns3d_oracle.c, restating Solver/src/solver.c).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
it, and only as the checker or the timed CPU baseline.

Arrays use the reference layout: Fourier ``complex128[N, N, N//2+1, 3]``
(solver.c:644-647) and real ``float64[N, N, N+2, 3]`` (solver.c:667).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libns3d_oracle.so")
_lib = None

IFRK4, RK4CN, RK5CN, DP5CN = 0, 1, 2, 3
FORCE_NONE, FORCE_SHELL = 0, 1


class _Params(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("nu", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("t0", ctypes.c_double),
        ("visc_pow", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("forcing", ctypes.c_int),
        ("force_k", ctypes.c_int),
        ("bugcompat_dealias", ctypes.c_int),
        ("bugcompat_measures", ctypes.c_int),
        ("nthreads", ctypes.c_int),
        ("bugcompat_rk5", ctypes.c_int),
        ("dp_atol", ctypes.c_double),
        ("dp_rtol", ctypes.c_double),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP when available)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(_Params)]
        L.orc_destroy.argtypes = [P]
        L.orc_n_spect.restype = ctypes.c_int
        L.orc_n_spect.argtypes = [ctypes.c_int]
        L.orc_threads.restype = ctypes.c_int
        for name in ("orc_set_state", "orc_get_state"):
            getattr(L, name).argtypes = [P, D]
        L.orc_set_time.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_long]
        L.orc_get_time.argtypes = [P, D, D, ctypes.POINTER(ctypes.c_long)]
        L.orc_forcing_target.restype = ctypes.c_double
        L.orc_forcing_target.argtypes = [P]
        L.orc_set_forcing_target.argtypes = [P, ctypes.c_double]
        L.orc_fft_r2c.argtypes = [P, D, D]
        L.orc_fft_c2r.argtypes = [P, D, D]
        L.orc_fft1d.argtypes = [ctypes.c_int, D, D, ctypes.c_int]
        L.orc_dealias.argtypes = [P, D, ctypes.c_int]
        L.orc_rhs.argtypes = [P, D, D]
        L.orc_stage.argtypes = [P]
        L.orc_stage.restype = ctypes.c_int
        L.orc_step.argtypes = [P, ctypes.c_int]
        L.orc_step.restype = ctypes.c_int
        L.orc_dp_stats.argtypes = [P, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_increment_stats.argtypes = [P, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
        L.orc_measurables.argtypes = [P, D, D, D]
        L.orc_ic.restype = ctypes.c_int
        L.orc_ic.argtypes = [P, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
        L.orc_real_space.argtypes = [P, D, D]
        L.orc_max_speed_sum.restype = ctypes.c_double
        L.orc_max_speed_sum.argtypes = [P]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def n_spect(N: int) -> int:
    return lib().orc_n_spect(N)


def threads() -> int:
    return lib().orc_threads()


def fft1d(x: np.ndarray, inverse: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.empty_like(x)
    lib().orc_fft1d(x.size, _dp(x.view(np.float64)), _dp(out.view(np.float64)), int(inverse))
    return out


class Oracle:
    """CPU FP64 solver context mirroring the reference's hot-path functions."""

    def __init__(self, N, nu=1.0, dt=1e-3, t0=0.0, visc_pow=1, integrator=IFRK4, cfl=0.0,
                 forcing=FORCE_NONE, force_k=2, bugcompat_dealias=False,
                 bugcompat_measures=False, nthreads=0, bugcompat_rk5=False, dp_atol=0.0, dp_rtol=0.0):
        self.N = N
        p = _Params(N, nu, dt, t0, visc_pow, integrator, cfl, forcing, force_k,
                    int(bugcompat_dealias), int(bugcompat_measures), nthreads, int(bugcompat_rk5), dp_atol, dp_rtol)
        self._c = lib().orc_create(ctypes.byref(p))
        if not self._c:
            raise ValueError(f"oracle rejected N={N}")

    def close(self):
        if self._c:
            lib().orc_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def fshape(self):
        return (self.N, self.N, self.N // 2 + 1, 3)

    @property
    def rshape(self):
        return (self.N, self.N, self.N + 2, 3)

    def set_state(self, u_hat: np.ndarray):
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        lib().orc_set_state(self._c, _dp(u.view(np.float64)))

    def get_state(self) -> np.ndarray:
        u = np.empty(self.fshape, np.complex128)
        lib().orc_get_state(self._c, _dp(u.view(np.float64)))
        return u

    def set_time(self, t, dt, iters):
        lib().orc_set_time(self._c, t, dt, iters)

    def get_time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        lib().orc_get_time(self._c, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it))
        return t.value, dt.value, it.value

    @property
    def forcing_target(self):
        return lib().orc_forcing_target(self._c)

    def r2c(self, real: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(real, dtype=np.float64).reshape(self.rshape)
        out = np.empty(self.fshape, np.complex128)
        lib().orc_fft_r2c(self._c, _dp(r), _dp(out.view(np.float64)))
        return out

    def c2r(self, u_hat: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        out = np.empty(self.rshape, np.float64)
        lib().orc_fft_c2r(self._c, _dp(u.view(np.float64)), _dp(out))
        return out

    def dealias(self, arr: np.ndarray) -> np.ndarray:
        a = np.array(arr, dtype=np.complex128, order="C", copy=True)
        dim = a.shape[-1] if a.ndim == 4 else 1
        lib().orc_dealias(self._c, _dp(a.view(np.float64)), dim)
        return a

    def rhs(self, u_hat: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        out = np.empty(self.fshape, np.complex128)
        lib().orc_rhs(self._c, _dp(u.view(np.float64)), _dp(out.view(np.float64)))
        return out

    def step(self, n=1):
        if lib().orc_step(self._c, n) != 0:
            raise RuntimeError("DP5CN step rejected 50 times in a row")

    def stage(self) -> int:
        """One RK4 stage (IF-RK4 / RK4CN); returns the next stage, 0 after a completed step."""
        r = lib().orc_stage(self._c)
        if r < 0:
            raise RuntimeError("orc_stage: IF-RK4 and RK4CN only")
        return r

    def increment_stats(self, increments=None, n_bins=1000):
        """Longitudinal velocity-increment statistics, bin edges and counts
        (PostProcessing/src/stats.c); increments None: 1, 2, ..., 128, N/2."""
        inc = np.ascontiguousarray([1, 2, 4, 8, 16, 32, 64, 128, self.N // 2] if increments is None else increments,
                                   dtype=np.int32)
        nr = len(inc)
        stats, ranges, counts = np.zeros((nr, 6)), np.zeros((nr, n_bins + 1)), np.zeros((nr, n_bins))
        lib().orc_increment_stats(self._c, inc.ctypes.data, nr, n_bins, stats.ctypes.data, ranges.ctypes.data,
                                  counts.ctypes.data)
        return {"stats": stats, "ranges": ranges, "counts": counts}

    def dp_stats(self):
        """(error norm of the last DP5CN attempt, rejected attempts so far)"""
        e, r = ctypes.c_double(), ctypes.c_long()
        lib().orc_dp_stats(self._c, ctypes.byref(e), ctypes.byref(r))
        return e.value, r.value

    def measurables(self):
        ns = n_spect(self.N)
        tot = np.zeros(5)
        Ek = np.zeros(ns)
        Ok = np.zeros(ns)
        lib().orc_measurables(self._c, _dp(tot), _dp(Ek), _dp(Ok))
        return tot, Ek, Ok

    def ic(self, name: str, seed: int = 0, k0: float = 4.0, energy: float = 1.0):
        lib().orc_ic(self._c, name.encode(), seed, k0, energy)

    def real_space(self):
        u = np.empty(self.rshape, np.float64)
        w = np.empty(self.rshape, np.float64)
        lib().orc_real_space(self._c, _dp(u), _dp(w))
        return u, w

    def max_speed_sum(self) -> float:
        return lib().orc_max_speed_sum(self._c)
