"""GPU test of ns3d_measurables_noalloc, the diagnostics entry point for
callers that cannot allocate device memory (for example an analysis hook
running inside another simulation that has reserved the whole GPU).

It is called through the C ABI on a caller-owned device copy of the state and
must reproduce the context-based ns3d_measurables on two calls in a row (the
second with a different grid, so leftovers from the first call in the shared
static scratch cannot leak into it). This file sorts last so that a run that
stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the FP64 tolerance of the other parity tests


def _bind(L):
    f = L.ns3d_measurables_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_measurables_noalloc_matches_context(ns3d):
    torch = pytest.importorskip("torch")
    fn = _bind(ns3d.lib())
    for N, seed, nu in ((64, 1, 0.01), (48, 2, 0.003)):
        s = ns3d.Solver(N, nu=nu, precision="fp64")
        s.InitialConditions("SPECTRUM", seed=seed, k0=4.0, energy=1.0)
        ref_tot, ref_Ek, ref_Ok = s.ComputeSystemMeasurables()
        u = s.get_state()
        s.close()
        d_u = torch.from_numpy(np.ascontiguousarray(u).view(np.float64)).cuda()
        ns = ns3d.n_spect(N)
        d_tot = torch.full((5,), np.nan, dtype=torch.float64, device="cuda")
        d_Ek = torch.full((ns,), np.nan, dtype=torch.float64, device="cuda")
        d_Ok = torch.full((ns,), np.nan, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st = fn(N, nu, 1, d_u.data_ptr(), d_tot.data_ptr(), d_Ek.data_ptr(), d_Ok.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert st == ns3d.OK
        tot, Ek, Ok = d_tot.cpu().numpy(), d_Ek.cpu().numpy(), d_Ok.cpu().numpy()
        want = np.array([ref_tot[k] for k in ("energy", "enstrophy", "palinstrophy", "helicity", "dissipation")])
        scale = np.array([want[0], want[1], want[2], np.sqrt(want[0] * want[1]), want[4]])
        assert np.all(np.abs(tot - want) <= TOL * scale), (tot, want)
        assert np.abs(Ek - ref_Ek).max() <= TOL * np.abs(ref_Ek).max()
        assert np.abs(Ok - ref_Ok).max() <= TOL * np.abs(ref_Ok).max()


def test_measurables_noalloc_rejects_oversize(ns3d):
    fn = _bind(ns3d.lib())
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    assert fn(1024, 0.01, 1, dummy, dummy, None, None, None) == ns3d.ERR_INVALID
