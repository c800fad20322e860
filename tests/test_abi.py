"""CPU tests of the C-ABI boundary: libns3d.so loads, exports every symbol
include/ns3d.h declares, and answers the no-GPU queries without computing."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ns3d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ns3d_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L(ns3d):
    if not os.path.exists(ns3d.LIB_PATH):
        ns3d.build()
    return ns3d.lib()


def test_exports_every_declared_symbol(L, ns3d):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), f"{s} declared in include/ns3d.h but not exported"
    assert set(syms) == set(ns3d.EXPORTS)


def test_static_queries(L):
    assert L.ns3d_n_spect(64) == 56 and L.ns3d_n_spect(512) == 444 and L.ns3d_n_spect(1024) == 887
    for n in (8, 16, 24, 32, 48, 64, 96, 128, 256, 512, 1024):
        assert L.ns3d_supported_size(n) == 1
    for n in (10, 40, 100, 2048):
        assert L.ns3d_supported_size(n) == 0
    assert L.ns3d_status_string(0) == b"ok"


def test_create_rejects_bad_params(L, ns3d):
    h = ctypes.c_void_p()
    for bad in (dict(N=7), dict(N=2), dict(N=64, nu=0.0), dict(N=64, dt=-1.0), dict(N=64, visc_pow=3),
                dict(N=64, integrator=5), dict(N=64, precision=9), dict(N=40)):
        kw = dict(N=64, nu=1.0, dt=1e-3, t0=0.0, visc_pow=1, integrator=0, precision=0, cfl=0.0,
                  forcing=0, force_k=2, device=0, stream=None)
        kw.update(bad)
        p = ns3d.Params(**kw)
        st = L.ns3d_create(ctypes.byref(p), ctypes.byref(h))
        assert st in (ns3d.ERR_INVALID, ns3d.ERR_UNSUPPORTED), (bad, st)


def test_no_gpu_is_an_error_not_a_fallback(L, ns3d):
    # without a GPU, creating a context must fail loudly (no CPU path exists)
    if os.path.exists("/dev/nvidia0") or os.environ.get("CUDA_VISIBLE_DEVICES", "") not in ("", "-1"):
        pytest.skip("a GPU may be present")
    with pytest.raises(ns3d.NS3DError):
        ns3d.Solver(16)
