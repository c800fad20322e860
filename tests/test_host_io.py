"""Host-array transfers through the C ABI: page-locked host arrays take the
direct path (the packing kernel reads the dealiased modes from host memory,
the unpacking kernel writes the 128-byte lines that hold them, host threads
zero the rest of the output), pageable arrays a full staged copy. Both must
fill every element of the output array identically, at every address
alignment, in place too."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pinned_complex(shape, offset_bytes=0):
    torch = pytest.importorskip("torch")
    n = int(np.prod(shape))
    raw = torch.empty(2 * n + 16, dtype=torch.float64, pin_memory=True).numpy()
    start = offset_bytes // 8
    return raw[start:start + 2 * n].view(np.complex128).reshape(shape), raw


@pytest.mark.parametrize("N,prec", [(32, "fp64"), (48, "fp32"), (64, "fp64")])
def test_pinned_and_pageable_outputs_are_identical(ns3d, N, prec):
    shape = (N, N, N // 2 + 1, 3)
    full = 48 * N * N * (N // 2 + 1)
    results = []
    for pinned_out in (False, True):
        s = ns3d.Solver(N, nu=0.01, dt=1e-3, precision=prec)
        s.InitialConditions("SPECTRUM", seed=5, k0=3.0)
        if pinned_out:
            out, keep = pinned_complex(shape)
        else:
            out = np.empty(shape, np.complex128)
        out[...] = np.nan
        s.step_host(None, out)
        h2d, d2h = s.io_bytes()
        assert np.isfinite(out).all()
        assert (d2h < full / 2) if pinned_out else (d2h == full)
        results.append(out.copy())
    assert np.array_equal(results[0], results[1])


@pytest.mark.parametrize("offset", [16, 48, 80, 112])
def test_pinned_alignments_and_in_place(ns3d, offset):
    N = 32
    shape = (N, N, N // 2 + 1, 3)
    a = ns3d.Solver(N, nu=0.01, dt=1e-3)
    a.InitialConditions("SPECTRUM", seed=9, k0=3.0)
    u0 = a.get_state()
    ref = np.empty(shape, np.complex128)
    a.step_host(u0, ref)
    b = ns3d.Solver(N, nu=0.01, dt=1e-3)
    buf, keep = pinned_complex(shape, offset)
    buf[...] = u0
    b.step_host(buf, buf)                 # in place, like RK4Step on run_data->u_hat
    h2d, d2h = b.io_bytes()
    assert h2d < 48 * N * N * (N // 2 + 1) / 2
    assert np.array_equal(buf, ref)
    buf[...] = np.nan
    b.step_host(None, buf)
    a.step_host(None, ref)
    assert np.array_equal(buf, ref)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_pinned_input_ignores_modes_outside_the_sphere(ns3d, prec):
    """The pinned upload reads whole 128-byte lines of the host array; values outside
    the dealiased sphere (NaN here) must not reach the state."""
    N = 48
    shape = (N, N, N // 2 + 1, 3)
    a = ns3d.Solver(N, nu=0.01, dt=1e-3, precision=prec)
    a.InitialConditions("SPECTRUM", seed=4, k0=3.0)
    u0 = a.get_state()
    ref = np.empty(shape, np.complex128)
    a.step_host(u0, ref)
    k = np.fft.fftfreq(N, 1.0 / N)
    kz = np.arange(N // 2 + 1)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    buf, keep = pinned_complex(shape)
    buf[...] = u0
    buf[k2 > (N // 3) ** 2] = np.nan
    b = ns3d.Solver(N, nu=0.01, dt=1e-3, precision=prec)
    b.step_host(buf, buf)
    assert np.array_equal(buf, ref)
