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
IFRK4, RK4CN, RK5CN, DP5CN = 0, 1, 2, 3
FORCE_NONE, FORCE_SHELL = 0, 1
_INTEG = {"ifrk4": IFRK4, "rk4cn": RK4CN, "rk5cn": RK5CN, "dp5cn": DP5CN}

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
    "ns3d_ensemble_run", "ns3d_ensemble_profile",
    "ns3d_ensemble_last_step_ms", "ns3d_set_state_real_host",
    "ns3d_les_num_params", "ns3d_les_create", "ns3d_les_destroy", "ns3d_les_last_error", "ns3d_les_add_snapshot",
    "ns3d_les_dataset_size", "ns3d_les_filtered_velocity_host", "ns3d_les_set_scales", "ns3d_les_get_scales",
    "ns3d_les_train", "ns3d_les_dataset_loss", "ns3d_les_weights_host", "ns3d_les_gradients_host",
    "ns3d_les_forward_host", "ns3d_les_attach", "ns3d_les_counters", "ns3d_set_dp_tolerances", "ns3d_dp_stats",
    "ns3d_set_wait_budget", "ns3d_les_set_train_path", "ns3d_les_train_path",
    "ns3d_les_infer_host", "ns3d_les_profile_infer", "ns3d_io_bytes",
    "ns3d_autotune", "ns3d_autotune_ensemble", "ns3d_tuning_get", "ns3d_tuning_set", "ns3d_tuning_clear", "ns3d_tuning_save",
    "ns3d_tuning_load", "ns3d_increment_stats",
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


class Tuning(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("variant", ctypes.c_int),
        ("zform", ctypes.c_int),
        ("ms_per_step", ctypes.c_float),
    ]

    def as_dict(self):
        return {"N": self.N, "precision": "fp32" if self.precision == FP32 else "fp64", "variant": self.variant,
                "zform": self.zform, "ms_per_step": self.ms_per_step}


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
        L.ns3d_set_dp_tolerances.restype = I
        L.ns3d_set_dp_tolerances.argtypes = [P, ctypes.c_double, ctypes.c_double]
        L.ns3d_dp_stats.restype = I
        L.ns3d_les_set_train_path.restype = I
        L.ns3d_les_set_train_path.argtypes = [P, I]
        L.ns3d_les_train_path.restype = I
        L.ns3d_les_train_path.argtypes = [P]
        L.ns3d_set_wait_budget.restype = I
        L.ns3d_set_wait_budget.argtypes = [P, ctypes.c_longlong]
        L.ns3d_dp_stats.argtypes = [P, D, ctypes.POINTER(ctypes.c_long)]
        L.ns3d_autotune.restype = I
        L.ns3d_autotune.argtypes = [ctypes.POINTER(Params), I, ctypes.POINTER(Tuning), ctypes.POINTER(Tuning), I,
                                    ctypes.POINTER(ctypes.c_int)]
        L.ns3d_autotune_ensemble.restype = I
        L.ns3d_autotune_ensemble.argtypes = [ctypes.POINTER(Params), I, I, ctypes.POINTER(Tuning), I,
                                             ctypes.POINTER(ctypes.c_int)]
        L.ns3d_tuning_get.restype = I
        L.ns3d_tuning_get.argtypes = [I, I, ctypes.POINTER(Tuning)]
        L.ns3d_tuning_set.restype = I
        L.ns3d_tuning_set.argtypes = [ctypes.POINTER(Tuning)]
        L.ns3d_tuning_clear.restype = I
        L.ns3d_tuning_clear.argtypes = []
        L.ns3d_tuning_save.restype = I
        L.ns3d_tuning_save.argtypes = [ctypes.c_char_p]
        L.ns3d_tuning_load.restype = I
        L.ns3d_tuning_load.argtypes = [ctypes.c_char_p]
        L.ns3d_increment_stats.restype = I
        L.ns3d_increment_stats.argtypes = [P, ctypes.POINTER(ctypes.c_int), I, I, D, D, D]
        L.ns3d_io_bytes.restype = I
        L.ns3d_io_bytes.argtypes = [P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
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
        L.ns3d_ensemble_run.restype = I
        L.ns3d_ensemble_run.argtypes = [P, I]
        L.ns3d_ensemble_info.restype = I
        L.ns3d_ensemble_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I)]
        L.ns3d_ensemble_profile.restype = I
        L.ns3d_ensemble_profile.argtypes = [P, I, I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_float),
                                            ctypes.POINTER(ctypes.c_double), I, ctypes.POINTER(I), ctypes.POINTER(I)]
        L.ns3d_ensemble_last_step_ms.restype = I
        L.ns3d_ensemble_last_step_ms.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
        F = ctypes.POINTER(ctypes.c_float)
        L.ns3d_set_state_real_host.restype = I
        L.ns3d_set_state_real_host.argtypes = [P, D]
        L.ns3d_les_num_params.restype = I
        L.ns3d_les_num_params.argtypes = []
        L.ns3d_les_create.restype = I
        L.ns3d_les_create.argtypes = [I, I, ctypes.c_uint64, ctypes.POINTER(P)]
        L.ns3d_les_destroy.restype = I
        L.ns3d_les_destroy.argtypes = [P]
        L.ns3d_les_last_error.restype = ctypes.c_char_p
        L.ns3d_les_last_error.argtypes = [P]
        L.ns3d_les_add_snapshot.restype = I
        L.ns3d_les_add_snapshot.argtypes = [P, P]
        L.ns3d_les_dataset_size.restype = I
        L.ns3d_les_dataset_size.argtypes = [P, ctypes.POINTER(I)]
        L.ns3d_les_filtered_velocity_host.restype = I
        L.ns3d_les_filtered_velocity_host.argtypes = [P, P, D]
        L.ns3d_les_set_scales.restype = I
        L.ns3d_les_set_scales.argtypes = [P, ctypes.c_double, ctypes.c_double]
        L.ns3d_les_get_scales.restype = I
        L.ns3d_les_get_scales.argtypes = [P, D, D]
        L.ns3d_les_train.restype = I
        L.ns3d_les_train.argtypes = [P, I, ctypes.c_double, D]
        L.ns3d_les_dataset_loss.restype = I
        L.ns3d_les_dataset_loss.argtypes = [P, D]
        L.ns3d_les_weights_host.restype = I
        L.ns3d_les_weights_host.argtypes = [P, F, I]
        L.ns3d_les_gradients_host.restype = I
        L.ns3d_les_gradients_host.argtypes = [P, F, F, D, F]
        L.ns3d_les_forward_host.restype = I
        L.ns3d_les_forward_host.argtypes = [P, F, F]
        L.ns3d_les_infer_host.restype = I
        L.ns3d_les_infer_host.argtypes = [P, F, F]
        L.ns3d_les_profile_infer.restype = I
        L.ns3d_les_profile_infer.argtypes = [P, I, ctypes.POINTER(ctypes.c_float)]
        L.ns3d_les_attach.restype = I
        L.ns3d_les_attach.argtypes = [P, P]
        L.ns3d_les_counters.restype = I
        L.ns3d_les_counters.argtypes = [P, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long)]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def autotune(N: int, steps: int = 10, **kw):
    """Time every compiled shape (tile variant x z-pass form) of grid size N on the
    Solver configuration kw (precision, nu, dt, cfl, ...) and keep the fastest for
    the engines built afterwards. Returns (best, tried) as dicts."""
    p = _params(N, **kw)
    best = Tuning()
    cap = 64   # tile variants x z-pass forms
    tried = (Tuning * cap)()
    n = ctypes.c_int()
    st = lib().ns3d_autotune(ctypes.byref(p), steps, ctypes.byref(best), tried, cap, ctypes.byref(n))
    if st != OK:
        raise NS3DError(st, f"ns3d_autotune(N={N}): {lib().ns3d_status_string(st).decode()}")
    return best.as_dict(), [tried[i].as_dict() for i in range(min(n.value, cap))]


def autotune_ensemble(members, steps: int = 10):
    """Tune every (N, precision) group of an ensemble (list of Solver keyword dicts)
    with all of its members; returns the chosen shape per group."""
    arr = (Params * len(members))(*[_params(**m) for m in members])
    best = (Tuning * 16)()
    n = ctypes.c_int()
    st = lib().ns3d_autotune_ensemble(arr, len(members), steps, best, 16, ctypes.byref(n))
    if st != OK:
        raise NS3DError(st, f"ns3d_autotune_ensemble: {lib().ns3d_status_string(st).decode()}")
    return [best[i].as_dict() for i in range(n.value)]


def tuning(N: int, precision: str = "fp32"):
    """The tuning-table entry of (N, precision), or None."""
    t = Tuning()
    st = lib().ns3d_tuning_get(N, {"fp64": FP64, "fp32": FP32}[precision], ctypes.byref(t))
    return t.as_dict() if st == OK else None


def tuning_set(N: int, variant: int, zform: int = 0, precision: str = "fp32"):
    t = Tuning(N, {"fp64": FP64, "fp32": FP32}[precision], variant, zform, 0.0)
    st = lib().ns3d_tuning_set(ctypes.byref(t))
    if st != OK:
        raise NS3DError(st, "ns3d_tuning_set")


def tuning_clear():
    lib().ns3d_tuning_clear()


def tuning_save(path: str):
    if lib().ns3d_tuning_save(str(path).encode()) != OK:
        raise NS3DError(ERR_INVALID, f"ns3d_tuning_save({path})")


def tuning_load(path: str):
    if lib().ns3d_tuning_load(str(path).encode()) != OK:
        raise NS3DError(ERR_INVALID, f"ns3d_tuning_load({path})")


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
        integ = _INTEG[integrator.lower()]
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

    def set_state_real(self, u: np.ndarray):
        """r2c + dealiasing of a real-space velocity in the reference layout [N][N][N+2][3]."""
        a = np.ascontiguousarray(u, dtype=np.float64).reshape(self.rshape)
        self._ck(lib().ns3d_set_state_real_host(self._h, _dp(a)))

    def attach_closure(self, les: "LES | None"):
        self._ck(lib().ns3d_les_attach(self._h, les._h if les is not None else None))

    def closure_counters(self):
        a, b = ctypes.c_long(), ctypes.c_long()
        self._ck(lib().ns3d_les_counters(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

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

    def increment_stats(self, increments=None, n_bins: int = 1000):
        """Longitudinal velocity-increment statistics (min, max, mean, sd, skew, excess
        kurtosis per increment), bin edges and counts; increments None: 1, 2, ..., 128, N/2."""
        inc = None if increments is None else np.ascontiguousarray(increments, dtype=np.int32)
        nr = 9 if inc is None else len(inc)
        stats = np.zeros((nr, 6))
        ranges = np.zeros((nr, n_bins + 1))
        counts = np.zeros((nr, n_bins))
        ip = None if inc is None else inc.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self._ck(lib().ns3d_increment_stats(self._h, ip, nr, n_bins, _dp(stats), _dp(ranges), _dp(counts)))
        return {"stats": stats, "ranges": ranges, "counts": counts}

    def io_bytes(self):
        """(host->device, device->host) bytes moved over the host link by the last upload / download."""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._ck(lib().ns3d_io_bytes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_dp_tolerances(self, atol: float, rtol: float):
        """DP5CN error tolerances (DP_ABS_TOL, DP_REL_TOL; default 1e-7 each)."""
        self._ck(lib().ns3d_set_dp_tolerances(self._h, atol, rtol))

    def set_wait_budget(self, cycles: int):
        """Clock-cycle budget of the z pass's bounded waits (<= 0: the
        default); a step whose wait runs out raises with ERR_TIMEOUT."""
        self._ck(lib().ns3d_set_wait_budget(self._h, int(cycles)))

    def dp_stats(self):
        """(error norm of the last DP5CN attempt, rejected attempts so far)"""
        e, r = ctypes.c_double(), ctypes.c_long()
        self._ck(lib().ns3d_dp_stats(self._h, ctypes.byref(e), ctypes.byref(r)))
        return e.value, r.value

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
    integ = _INTEG[integrator.lower()]
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

    def run(self, nsteps):
        """nsteps steps in one graph launch (a device-side loop over the captured step)."""
        self._ck(lib().ns3d_ensemble_run(self._h, nsteps))

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

    def profile_group(self, group: int, reps: int = 3):
        """(N, [(kernel class, ms per launch, bytes)]) of launch group `group`;
        its members advance `reps` steps."""
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_float * 16)()
        by = (ctypes.c_double * 16)()
        cnt, n = ctypes.c_int(), ctypes.c_int()
        self._ck(lib().ns3d_ensemble_profile(self._h, group, reps, names, ms, by, 16, ctypes.byref(cnt),
                                             ctypes.byref(n)))
        return n.value, [(names[i].decode(), ms[i], by[i]) for i in range(cnt.value)]



def _fp(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class LES:
    """Learned subgrid closure (ns3d_les_*): dataset of box-filtered fine-run
    snapshots, a 3D CNN trained on the GPU, attachable to a coarse run."""

    def __init__(self, Nc: int, capacity: int = 0, seed: int = 0):
        self.Nc = Nc
        h = ctypes.c_void_p()
        st = lib().ns3d_les_create(Nc, capacity, seed, ctypes.byref(h))
        if st != OK:
            raise NS3DError(st, f"ns3d_les_create: {lib().ns3d_status_string(st).decode()}")
        self._h = h

    def _ck(self, st):
        if st != OK:
            raise NS3DError(st, lib().ns3d_les_last_error(self._h).decode() or lib().ns3d_status_string(st).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().ns3d_les_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def num_params() -> int:
        return lib().ns3d_les_num_params()

    def add_snapshot(self, fine: Solver):
        self._ck(lib().ns3d_les_add_snapshot(self._h, fine._h))

    @property
    def size(self) -> int:
        n = ctypes.c_int()
        self._ck(lib().ns3d_les_dataset_size(self._h, ctypes.byref(n)))
        return n.value

    def filtered_velocity(self, fine: Solver) -> np.ndarray:
        N = self.Nc
        out = np.empty((N, N, N + 2, 3), np.float64)
        self._ck(lib().ns3d_les_filtered_velocity_host(self._h, fine._h, _dp(out)))
        return out

    def set_scales(self, s_in: float, s_out: float):
        self._ck(lib().ns3d_les_set_scales(self._h, s_in, s_out))

    def scales(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._ck(lib().ns3d_les_get_scales(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def train(self, iterations: int, lr: float = 1e-3) -> float:
        v = ctypes.c_double()
        self._ck(lib().ns3d_les_train(self._h, iterations, lr, ctypes.byref(v)))
        return v.value

    def dataset_loss(self) -> float:
        v = ctypes.c_double()
        self._ck(lib().ns3d_les_dataset_loss(self._h, ctypes.byref(v)))
        return v.value

    def set_train_path(self, path: str):
        """"tc": tensor cores where compiled (Nc in 16, 32, 64; the default), "fp32": CUDA cores."""
        self._ck(lib().ns3d_les_set_train_path(self._h, {"tc": 0, "fp32": 1}[path]))

    @property
    def train_path(self) -> str:
        return "tc" if lib().ns3d_les_train_path(self._h) == 0 else "fp32"

    def weights(self) -> np.ndarray:
        w = np.empty(self.num_params(), np.float32)
        self._ck(lib().ns3d_les_weights_host(self._h, _fp(w), 0))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._ck(lib().ns3d_les_weights_host(self._h, _fp(w), 1))

    def gradients(self, u: np.ndarray, tau: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float32)
        tau = np.ascontiguousarray(tau, dtype=np.float32)
        g = np.empty(self.num_params(), np.float32)
        loss = ctypes.c_double()
        self._ck(lib().ns3d_les_gradients_host(self._h, _fp(u), _fp(tau), ctypes.byref(loss), _fp(g)))
        return loss.value, g

    def forward(self, u: np.ndarray) -> np.ndarray:
        """tau = network(u), FP32 training network."""
        u = np.ascontiguousarray(u, dtype=np.float32)
        out = np.empty((6,) + u.shape[1:], np.float32)
        self._ck(lib().ns3d_les_forward_host(self._h, _fp(u), _fp(out)))
        return out

    def profile_infer(self, reps: int = 10) -> float:
        """Mean device milliseconds of one inference (device-resident input)."""
        v = ctypes.c_float()
        self._ck(lib().ns3d_les_profile_infer(self._h, reps, ctypes.byref(v)))
        return v.value

    def infer(self, u: np.ndarray) -> np.ndarray:
        """tau = network(u) through the attached-run inference path (tensor cores for Nc in 16, 32, 64)."""
        u = np.ascontiguousarray(u, dtype=np.float32)
        out = np.empty((6,) + u.shape[1:], np.float32)
        self._ck(lib().ns3d_les_infer_host(self._h, _fp(u), _fp(out)))
        return out
