"""GB300 (sm_103a) time-stepping hot path of a 3D periodic pseudospectral
Navier–Stokes solver, behind the C ABI of ``include/ns3d.h``.

This module is a thin ctypes layer over ``_build/libns3d.so``. Its method
names mirror the reference solver's hot-path functions (Solver/src/solver.c):
``InitialConditions``, ``RK4Step``, ``NonlinearRHSBatch``, ``ApplyDealiasing``,
``ComputeSystemMeasurables``. All compute runs in hand-written CUDA kernels;
there is no CPU path, and every entry point raises if the library is missing.

Host arrays use the reference layouts: Fourier ``complex128[N, N, N//2+1, 3]``
(solver.c:644-647) and real ``float64[N, N, N+2, 3]`` (solver.c:667).

The package directory starts with a digit, so import it with
``importlib.import_module("3d_navier_stokes_gb300")``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.environ.get("NS3D_BUILD_DIR") or os.path.join(_HERE, "_build"), "libns3d.so")
_lib = None

OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_NUMERIC, ERR_TIMEOUT = range(7)
FP64, FP32 = 0, 1
IFRK4, RK4CN = 0, 1
FORCE_NONE, FORCE_SHELL = 0, 1

# every symbol include/ns3d.h declares
EXPORTS = (
    "ns3d_status_string", "ns3d_supported_size", "ns3d_n_spect", "ns3d_create", "ns3d_destroy",
    "ns3d_last_error", "ns3d_initial_condition", "ns3d_set_state_host", "ns3d_get_state_host",
    "ns3d_step", "ns3d_step_host", "ns3d_rhs_host", "ns3d_dealias_host", "ns3d_measurables",
    "ns3d_real_space_host", "ns3d_get_time", "ns3d_set_time", "ns3d_get_forcing_target",
    "ns3d_set_forcing_target", "ns3d_max_speed_sum", "ns3d_stream", "ns3d_kernels_per_step",
    "ns3d_last_step_ms", "ns3d_profile_step", "ns3d_measurables_noalloc",
    "ns3d_ensemble_create", "ns3d_ensemble_destroy", "ns3d_ensemble_last_error",
    "ns3d_ensemble_initial_condition", "ns3d_ensemble_set_state_host", "ns3d_ensemble_get_state_host",
    "ns3d_ensemble_measurables", "ns3d_ensemble_get_time", "ns3d_ensemble_step", "ns3d_ensemble_info",
    "ns3d_ensemble_last_step_ms",
)


class NS3DError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ns3d status {status}: {msg}")
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("nu", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("t0", ctypes.c_double),
        ("visc_pow", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("forcing", ctypes.c_int),
        ("force_k", ctypes.c_int),
        ("device", ctypes.c_int),
        ("stream", ctypes.c_void_p),
    ]


class Measures(ctypes.Structure):
    _fields_ = [
        ("energy", ctypes.c_double),
        ("enstrophy", ctypes.c_double),
        ("palinstrophy", ctypes.c_double),
        ("helicity", ctypes.c_double),
        ("dissipation", ctypes.c_double),
    ]


def build(verbose: bool = False) -> str:
    from importlib import import_module
    b = import_module(__name__ + ".build")
    return b.build(verbose=verbose)


def lib():
    """Load libns3d.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                               "(the solver has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        P, D, I = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.ns3d_status_string.restype = ctypes.c_char_p
        L.ns3d_status_string.argtypes = [I]
        L.ns3d_supported_size.restype = I
        L.ns3d_supported_size.argtypes = [I]
        L.ns3d_n_spect.restype = I
        L.ns3d_n_spect.argtypes = [I]
        L.ns3d_create.restype = I
        L.ns3d_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.ns3d_destroy.restype = I
        L.ns3d_destroy.argtypes = [P]
        L.ns3d_last_error.restype = ctypes.c_char_p
        L.ns3d_last_error.argtypes = [P]
        L.ns3d_initial_condition.restype = I
        L.ns3d_initial_condition.argtypes = [P, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
        for n in ("ns3d_set_state_host", "ns3d_get_state_host"):
            getattr(L, n).restype = I
            getattr(L, n).argtypes = [P, D]
        L.ns3d_step.restype = I
        L.ns3d_step.argtypes = [P, I]
        L.ns3d_step_host.restype = I
        L.ns3d_step_host.argtypes = [P, D, D]
        L.ns3d_rhs_host.restype = I
        L.ns3d_rhs_host.argtypes = [P, D, D]
        L.ns3d_dealias_host.restype = I
        L.ns3d_dealias_host.argtypes = [I, D, I]
        L.ns3d_measurables.restype = I
        L.ns3d_measurables.argtypes = [P, ctypes.POINTER(Measures), D, D]
        L.ns3d_real_space_host.restype = I
        L.ns3d_real_space_host.argtypes = [P, D, D]
        L.ns3d_get_time.restype = I
        L.ns3d_get_time.argtypes = [P, D, D, ctypes.POINTER(ctypes.c_long)]
        L.ns3d_set_time.restype = I
        L.ns3d_set_time.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_long]
        L.ns3d_get_forcing_target.restype = I
        L.ns3d_get_forcing_target.argtypes = [P, D]
        L.ns3d_set_forcing_target.restype = I
        L.ns3d_set_forcing_target.argtypes = [P, ctypes.c_double]
        L.ns3d_max_speed_sum.restype = I
        L.ns3d_max_speed_sum.argtypes = [P, D]
        L.ns3d_stream.restype = P
        L.ns3d_stream.argtypes = [P]
        L.ns3d_kernels_per_step.restype = I
        L.ns3d_kernels_per_step.argtypes = [P]
        L.ns3d_last_step_ms.restype = I
        L.ns3d_last_step_ms.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
        L.ns3d_profile_step.restype = I
        L.ns3d_profile_step.argtypes = [P, I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_float),
                                        D, I, ctypes.POINTER(I)]
        L.ns3d_ensemble_create.restype = I
        L.ns3d_ensemble_create.argtypes = [ctypes.POINTER(Params), I, ctypes.POINTER(P)]
        L.ns3d_ensemble_destroy.restype = I
        L.ns3d_ensemble_destroy.argtypes = [P]
        L.ns3d_ensemble_last_error.restype = ctypes.c_char_p
        L.ns3d_ensemble_last_error.argtypes = [P]
        L.ns3d_ensemble_initial_condition.restype = I
        L.ns3d_ensemble_initial_condition.argtypes = [P, I, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_double,
                                                      ctypes.c_double]
        for n in ("ns3d_ensemble_set_state_host", "ns3d_ensemble_get_state_host"):
            getattr(L, n).restype = I
            getattr(L, n).argtypes = [P, I, D]
        L.ns3d_ensemble_measurables.restype = I
        L.ns3d_ensemble_measurables.argtypes = [P, I, ctypes.POINTER(Measures), D, D]
        L.ns3d_ensemble_get_time.restype = I
        L.ns3d_ensemble_get_time.argtypes = [P, I, D, D, ctypes.POINTER(ctypes.c_long)]
        L.ns3d_ensemble_step.restype = I
        L.ns3d_ensemble_step.argtypes = [P, I]
        L.ns3d_ensemble_info.restype = I
        L.ns3d_ensemble_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I)]
        L.ns3d_ensemble_last_step_ms.restype = I
        L.ns3d_ensemble_last_step_ms.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def n_spect(N: int) -> int:
    return lib().ns3d_n_spect(N)


def supported(N: int) -> bool:
    return bool(lib().ns3d_supported_size(N))


def ApplyDealiasing(array: np.ndarray) -> np.ndarray:
    """2/3-rule dealiasing of a reference-layout Fourier array (solver.c:1709-1756),
    computed on the GPU. Returns a new array."""
    a = np.array(array, dtype=np.complex128, order="C", copy=True)
    N = a.shape[0]
    dim = a.shape[3] if a.ndim == 4 else 1
    st = lib().ns3d_dealias_host(N, _dp(a.view(np.float64)), dim)
    if st != OK:
        raise NS3DError(st, lib().ns3d_status_string(st).decode())
    return a


class Solver:
    """One solver context on one GPU (AllocateMemory + InitializeFFTWPlans,
    solver.c:1832-2073). Not thread-safe; contexts are independent."""

    def __init__(self, N: int, nu: float = 1.0, dt: float = 1e-3, t0: float = 0.0, visc_pow: int = 1,
                 integrator: str = "ifrk4", precision: str = "fp64", cfl: float = 0.0,
                 forcing: str | None = None, force_k: int = 2, device: int = 0, stream: int | None = None):
        self.N = N
        self.precision = precision
        integ = {"ifrk4": IFRK4, "rk4cn": RK4CN}[integrator.lower()]
        prec = {"fp64": FP64, "fp32": FP32}[precision.lower()]
        force = FORCE_SHELL if (forcing or "").upper() in ("SHELL", "ENERGY_SHELL") else FORCE_NONE
        p = Params(N, nu, dt, t0, visc_pow, integ, prec, cfl, force, force_k, device, stream)
        h = ctypes.c_void_p()
        st = lib().ns3d_create(ctypes.byref(p), ctypes.byref(h))
        if st != OK:
            raise NS3DError(st, f"ns3d_create(N={N}): {lib().ns3d_status_string(st).decode()}")
        self._h = h

    # ------------------------------------------------------------ plumbing
    def _ck(self, st: int):
        if st != OK:
            raise NS3DError(st, lib().ns3d_last_error(self._h).decode() or lib().ns3d_status_string(st).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().ns3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def fshape(self):
        return (self.N, self.N, self.N // 2 + 1, 3)

    @property
    def rshape(self):
        return (self.N, self.N, self.N + 2, 3)

    # ---------------------------------------------- reference entry points
    def InitialConditions(self, name: str, seed: int = 0, k0: float = 4.0, energy: float = 1.0):
        self._ck(lib().ns3d_initial_condition(self._h, name.encode(), seed, k0, energy))

    def RK4Step(self, nsteps: int = 1):
        self._ck(lib().ns3d_step(self._h, nsteps))

    def NonlinearRHSBatch(self, u_hat: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        out = np.empty(self.fshape, np.complex128)
        self._ck(lib().ns3d_rhs_host(self._h, _dp(u.view(np.float64)), _dp(out.view(np.float64))))
        return out

    def ComputeSystemMeasurables(self):
        """Returns (totals dict, energy spectrum, enstrophy spectrum)."""
        m = Measures()
        ns = n_spect(self.N)
        Ek, Ok = np.zeros(ns), np.zeros(ns)
        self._ck(lib().ns3d_measurables(self._h, ctypes.byref(m), _dp(Ek), _dp(Ok)))
        tot = {k: getattr(m, k) for k, _ in Measures._fields_}
        return tot, Ek, Ok

    # ------------------------------------------------------------- state
    def set_state(self, u_hat: np.ndarray):
        u = np.ascontiguousarray(u_hat, dtype=np.complex128).reshape(self.fshape)
        self._ck(lib().ns3d_set_state_host(self._h, _dp(u.view(np.float64))))

    def get_state(self) -> np.ndarray:
        out = np.empty(self.fshape, np.complex128)
        self._ck(lib().ns3d_get_state_host(self._h, _dp(out.view(np.float64))))
        return out

    def step_host(self, u_in: np.ndarray | None, u_out: np.ndarray | None):
        ip = _dp(u_in.view(np.float64)) if u_in is not None else None
        op = _dp(u_out.view(np.float64)) if u_out is not None else None
        self._ck(lib().ns3d_step_host(self._h, ip, op))

    def real_space(self):
        u = np.empty(self.rshape, np.float64)
        w = np.empty(self.rshape, np.float64)
        self._ck(lib().ns3d_real_space_host(self._h, _dp(u), _dp(w)))
        return u, w

    def get_time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        self._ck(lib().ns3d_get_time(self._h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it)))
        return t.value, dt.value, it.value

    def set_time(self, t: float, dt: float, iters: int):
        self._ck(lib().ns3d_set_time(self._h, t, dt, iters))

    @property
    def forcing_target(self) -> float:
        e = ctypes.c_double()
        self._ck(lib().ns3d_get_forcing_target(self._h, ctypes.byref(e)))
        return e.value

    @forcing_target.setter
    def forcing_target(self, e: float):
        self._ck(lib().ns3d_set_forcing_target(self._h, e))

    def max_speed_sum(self) -> float:
        v = ctypes.c_double()
        self._ck(lib().ns3d_max_speed_sum(self._h, ctypes.byref(v)))
        return v.value

    # ---------------------------------------------------- instrumentation
    @property
    def stream(self) -> int:
        return lib().ns3d_stream(self._h) or 0

    @property
    def kernels_per_step(self) -> int:
        return lib().ns3d_kernels_per_step(self._h)

    def last_step_ms(self) -> float:
        v = ctypes.c_float()
        self._ck(lib().ns3d_last_step_ms(self._h, ctypes.byref(v)))
        return v.value

    def profile_step(self, reps: int = 3):
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_float * 16)()
        by = (ctypes.c_double * 16)()
        cnt = ctypes.c_int()
        self._ck(lib().ns3d_profile_step(self._h, reps, names, ms, by, 16, ctypes.byref(cnt)))
        return [(names[i].decode(), ms[i], by[i]) for i in range(cnt.value)]


def _params(N, nu=1.0, dt=1e-3, t0=0.0, visc_pow=1, integrator="ifrk4", precision="fp64", cfl=0.0,
            forcing=None, force_k=2, device=0, stream=None):
    integ = {"ifrk4": IFRK4, "rk4cn": RK4CN}[integrator.lower()]
    prec = {"fp64": FP64, "fp32": FP32}[precision.lower()]
    force = FORCE_SHELL if (forcing or "").upper() in ("SHELL", "ENERGY_SHELL") else FORCE_NONE
    return Params(N, nu, dt, t0, visc_pow, integ, prec, cfl, force, force_k, device, stream)


class Ensemble:
    """Independent runs stepped together (ns3d_ensemble_*): one graph launch per
    step advances every member; members of equal grid size share launches."""

    def __init__(self, members):
        """members: list of dicts with Solver keyword arguments (N, nu, dt, ...)."""
        self.members = [dict(m) for m in members]
        arr = (Params * len(members))(*[_params(**m) for m in members])
        h = ctypes.c_void_p()
        st = lib().ns3d_ensemble_create(arr, len(members), ctypes.byref(h))
        if st != OK:
            raise NS3DError(st, f"ns3d_ensemble_create: {lib().ns3d_status_string(st).decode()}")
        self._h = h

    def _ck(self, st):
        if st != OK:
            raise NS3DError(st, lib().ns3d_ensemble_last_error(self._h).decode() or
                            lib().ns3d_status_string(st).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().ns3d_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def InitialConditions(self, member, name, seed=0, k0=4.0, energy=1.0):
        self._ck(lib().ns3d_ensemble_initial_condition(self._h, member, name.encode(), seed, k0, energy))

    def step(self, nsteps=1):
        self._ck(lib().ns3d_ensemble_step(self._h, nsteps))

    def get_state(self, member):
        N = self.members[member]["N"]
        out = np.empty((N, N, N // 2 + 1, 3), np.complex128)
        self._ck(lib().ns3d_ensemble_get_state_host(self._h, member, _dp(out.view(np.float64))))
        return out

    def set_state(self, member, u_hat):
        u = np.ascontiguousarray(u_hat, dtype=np.complex128)
        self._ck(lib().ns3d_ensemble_set_state_host(self._h, member, _dp(u.view(np.float64))))

    def measurables(self, member):
        m = Measures()
        ns = n_spect(self.members[member]["N"])
        Ek, Ok = np.zeros(ns), np.zeros(ns)
        self._ck(lib().ns3d_ensemble_measurables(self._h, member, ctypes.byref(m), _dp(Ek), _dp(Ok)))
        return {k: getattr(m, k) for k, _ in Measures._fields_}, Ek, Ok

    def get_time(self, member):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        self._ck(lib().ns3d_ensemble_get_time(self._h, member, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it)))
        return t.value, dt.value, it.value

    def info(self):
        g, k = ctypes.c_int(), ctypes.c_int()
        self._ck(lib().ns3d_ensemble_info(self._h, ctypes.byref(g), ctypes.byref(k)))
        return g.value, k.value

    def last_step_ms(self):
        v = ctypes.c_float()
        self._ck(lib().ns3d_ensemble_last_step_ms(self._h, ctypes.byref(v)))
        return v.value
