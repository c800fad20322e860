"""GPU tests of ns3d_measurables_noalloc, the diagnostics entry point for
callers that cannot allocate device memory (for example an analysis hook
running inside another simulation that has reserved the whole GPU).

It is called through the C ABI on caller-owned device arrays and must
reproduce
  * the context-based ns3d_measurables on two calls in a row (different grids,
    so leftovers from the first call in the shared static scratch cannot leak
    into the second), and at N = 512, the largest grid its scratch holds;
  * the oracle on arrays that were never dealiased (Nyquist and corner modes
    set, shells beyond n_spect), the part of its work that the context path
    never sees, for both viscosity powers;
  * itself after the device's primary context is reset by another module of
    the process (a child process drives the driver API directly).
This file sorts last so that a run that stops at the first failure has
already run every other test."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the FP64 tolerance of the other parity tests
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bind(L):
    f = L.ns3d_measurables_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _call(ns3d, torch, N, nu, vp, u):
    fn = _bind(ns3d.lib())
    d_u = torch.from_numpy(np.ascontiguousarray(u).view(np.float64)).cuda()
    ns = ns3d.n_spect(N)
    d_tot = torch.full((5,), np.nan, dtype=torch.float64, device="cuda")
    d_Ek = torch.full((ns,), np.nan, dtype=torch.float64, device="cuda")
    d_Ok = torch.full((ns,), np.nan, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = fn(N, nu, vp, d_u.data_ptr(), d_tot.data_ptr(), d_Ek.data_ptr(), d_Ok.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert st == ns3d.OK
    return d_tot.cpu().numpy(), d_Ek.cpu().numpy(), d_Ok.cpu().numpy()


def _check(tot, Ek, Ok, want, ref_Ek, ref_Ok):
    scale = np.array([want[0], want[1], want[2], np.sqrt(want[0] * want[1]), want[4]])
    assert np.all(np.abs(tot - want) <= TOL * scale), (tot, want)
    assert np.abs(Ek - ref_Ek).max() <= TOL * np.abs(ref_Ek).max()
    assert np.abs(Ok - ref_Ok).max() <= TOL * np.abs(ref_Ok).max()


@pytest.mark.parametrize("cases", [((64, 1, 0.01), (48, 2, 0.003)), ((512, 5, 0.001),)])
def test_measurables_noalloc_matches_context(ns3d, cases):
    torch = pytest.importorskip("torch")
    for N, seed, nu in cases:
        s = ns3d.Solver(N, nu=nu, precision="fp64")
        s.InitialConditions("SPECTRUM", seed=seed, k0=4.0, energy=1.0)
        ref_tot, ref_Ek, ref_Ok = s.ComputeSystemMeasurables()
        u = s.get_state()
        s.close()
        tot, Ek, Ok = _call(ns3d, torch, N, nu, 1, u)
        del u
        want = np.array([ref_tot[k] for k in ("energy", "enstrophy", "palinstrophy", "helicity", "dissipation")])
        _check(tot, Ek, Ok, want, ref_Ek, ref_Ok)


@pytest.mark.parametrize("N", [16, 48, 64])
@pytest.mark.parametrize("visc_pow", [1, 2])
def test_measurables_noalloc_every_mode_vs_oracle(ns3d, oracle, N, visc_pow):
    """A full half spectrum, never dealiased: Nyquist planes, the kz = N/2
    plane (weight 1) and the corner shells round(|k|) >= n_spect (N = 16, 48)
    all carry energy."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1000 + N + visc_pow)
    u = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    u[N // 2, N // 2, N // 2] = [3.0 + 1.0j, -2.0, 0.5j]   # the corner mode
    nu = 0.002
    o = oracle.Oracle(N, nu=nu, visc_pow=visc_pow)
    o.set_state(u)
    want, ref_Ek, ref_Ok = o.measurables()
    tot, Ek, Ok = _call(ns3d, torch, N, nu, visc_pow, u)
    _check(tot, Ek, Ok, want, ref_Ek, ref_Ok)


_CHILD = r'''
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
cu = ctypes.CDLL("libcuda.so.1")
P = ctypes.c_void_p
def ck(r, what):
    if r != 0:
        raise SystemExit(f"{what}: CUresult {r}")
ck(cu.cuInit(0), "cuInit")
dev = ctypes.c_int()
ck(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
import importlib
ns3d = importlib.import_module("3d_navier_stokes_gb300")
from oracle import oracle as O
fn = ns3d.lib().ns3d_measurables_noalloc
fn.restype = ctypes.c_int
fn.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 5
N, nu = 32, 0.004
rng = np.random.default_rng(7)
u = np.ascontiguousarray(np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2)))
o = O.Oracle(N, nu=nu)
o.set_state(u)
want, wEk, wOk = o.measurables()
ns = ns3d.n_spect(N)
def run():
    ctx = P()
    ck(cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "retain")
    ck(cu.cuCtxSetCurrent(ctx), "set current")
    bufs = []
    for n in (u.nbytes, 40, 8 * ns, 8 * ns):
        b = ctypes.c_uint64()
        ck(cu.cuMemAlloc_v2(ctypes.byref(b), ctypes.c_size_t(n)), "alloc")
        bufs.append(b.value)
    ck(cu.cuMemcpyHtoD_v2(ctypes.c_uint64(bufs[0]), u.ctypes.data_as(P), ctypes.c_size_t(u.nbytes)), "h2d")
    st = fn(N, nu, 1, bufs[0], bufs[1], bufs[2], bufs[3], None)
    ck(cu.cuCtxSynchronize(), "sync")
    out = [np.empty(5), np.empty(ns), np.empty(ns)]
    for a, b in zip(out, bufs[1:]):
        ck(cu.cuMemcpyDtoH_v2(a.ctypes.data_as(P), ctypes.c_uint64(b), ctypes.c_size_t(a.nbytes)), "d2h")
    for b in bufs:
        ck(cu.cuMemFree_v2(ctypes.c_uint64(b)), "free")
    return st, out
for rnd in range(2):
    st, (tot, Ek, Ok) = run()
    if st != 0:
        raise SystemExit(f"round {rnd}: status {st}")
    scale = np.array([want[0], want[1], want[2], np.sqrt(want[0] * want[1]), want[4]])
    assert np.all(np.abs(tot - want) <= 1e-12 * scale), (rnd, tot, want)
    assert np.abs(Ek - wEk).max() <= 1e-12 * np.abs(wEk).max(), rnd
    assert np.abs(Ok - wOk).max() <= 1e-12 * np.abs(wOk).max(), rnd
    if rnd == 0:
        # another module of the process resets the device: a new primary context
        ck(cu.cuDevicePrimaryCtxRelease_v2(dev), "release")
        ck(cu.cuDevicePrimaryCtxReset_v2(dev), "reset")
print("ok")
'''


def test_measurables_noalloc_after_context_reset(ns3d, tmp_path):
    """The scratch address is looked up in the current context on every call
    outside capture, so a device reset by another module (which gives the
    process a new primary context, and the static array a new address) cannot
    leave a stale address behind."""
    script = tmp_path / "child.py"
    script.write_text(_CHILD)
    r = subprocess.run([sys.executable, str(script), ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


def test_measurables_noalloc_rejects_oversize_and_misaligned(ns3d):
    fn = _bind(ns3d.lib())
    dummy = ctypes.c_void_p(16)   # never dereferenced: the argument checks come first
    assert fn(1024, 0.01, 1, dummy, dummy, None, None, None) == ns3d.ERR_INVALID
    assert fn(64, 0.01, 1, ctypes.c_void_p(24), dummy, None, None, None) == ns3d.ERR_INVALID
    assert fn(64, 0.01, 1, dummy, ctypes.c_void_p(20), None, None, None) == ns3d.ERR_INVALID
    assert fn(64, 0.01, 3, dummy, dummy, None, None, None) == ns3d.ERR_INVALID
