"""The reference-facing layers over the C ABI: the compat shim with the
reference's function names (include/ns3d_compat.h), the `solver` driver with
the reference's flags and output layout, and checkpoint/resume through -z."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def solver_bin(ns3d):
    return os.path.join(os.path.dirname(ns3d.LIB_PATH), "solver")


def read_container(path):
    idx = json.load(open(os.path.join(path, "index.json")))
    out = {}
    for d in idx["datasets"]:
        a = np.fromfile(os.path.join(path, d["file"]), dtype=np.dtype(d["dtype"])).reshape(d["shape"])
        out[d["path"]] = (a, d.get("attrs"))
    return out


def test_driver_rejects_bad_arguments(ns3d):
    # argument checks of GetCMLArgs (utils.c:87-160) happen before any GPU work
    exe = solver_bin(ns3d)
    if not os.path.exists(exe):
        pytest.skip("driver not built")
    for args in (["-n", "7"], ["-n", "2"], ["-h", "-1"], ["-v", "0"], ["-e", "-1"]):
        r = subprocess.run([exe] + args, capture_output=True, text=True)
        assert r.returncode == 1 and "ERROR" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("integrator,visc_pow", [(0, 0), (0, 1), (1, 1), (2, 1), (3, 1), (1, 2)])
def test_compat_shim_reference_shaped_driver(ns3d, oracle, tmp_path, integrator, visc_pow):
    """(0, 0) is a zero-filled sys_vars: the reference's default build, RK4 +
    Crank-Nicolson with nu k^4."""
    exe = tmp_path / "compat_driver"
    libdir = os.path.dirname(ns3d.LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "compat_driver.c"), "-o", str(exe), "-L", libdir, "-lns3d",
                    f"-Wl,-rpath,{libdir}"], check=True)
    N, nu, dt, n = 24, 0.01, 2e-3, 5
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(N), str(nu), str(dt), str(n), str(integrator), str(visc_pow), str(out)],
                   check=True)
    raw = np.fromfile(out, dtype=np.float64)
    nf = N * N * (N // 2 + 1) * 3
    u = raw[:2 * nf].view(np.complex128).reshape(N, N, N // 2 + 1, 3)
    E = raw[2 * nf:2 * nf + n + 1]
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=[oracle.RK4CN, oracle.IFRK4, oracle.RK5CN, oracle.DP5CN][integrator],
                      visc_pow=1 if visc_pow == 1 else 2)
    o.ic("TAYLOR_GREEN")
    ref_E = [o.measurables()[0][0]]
    for _ in range(n):
        o.step(1)
        ref_E.append(o.measurables()[0][0])
    ref = o.get_state()
    assert np.linalg.norm(u - ref) / np.linalg.norm(ref) < 1e-12
    assert np.max(np.abs(E - ref_E) / np.array(ref_E)) < 1e-12
    if integrator == 3:
        # the Dormand-Prince control hands back the new time and the next step size
        t_ref, dt_ref, _ = o.get_time()
        t_out, dt_out = raw[2 * nf + 2 * (n + 1):]
        assert abs(t_out - t_ref) <= 1e-12 * t_ref and abs(dt_out - dt_ref) <= 1e-10 * dt_ref
        assert dt_out != dt


@pytest.mark.gpu
def test_driver_outputs_match_oracle(ns3d, oracle, tmp_path):
    exe = solver_bin(ns3d)
    N, nu, dt = 32, 0.01, 2e-3
    args = [exe, "-o", str(tmp_path), "-n", str(N), "-n", str(N), "-n", str(N), "-s", "0.0", "-e", "0.02",
            "-h", str(dt), "-v", str(nu), "-i", "TAYLOR_GREEN", "-p", "5", "-t", "T1", "-I", "ifrk4", "-L"]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sub = [d for d in os.listdir(tmp_path) if d.startswith("SIM_DATA_NAVIER_IFRK4_FULL_N[32,32]")]
    assert len(sub) == 1 and sub[0].endswith("_TAG[T1]")
    main = read_container(os.path.join(tmp_path, sub[0], "Main_HDF_Data.ns3d"))
    spec = read_container(os.path.join(tmp_path, sub[0], "Spectra_HDF_Data.ns3d"))
    o = oracle.Oracle(N, nu=nu, dt=dt)
    o.ic("TAYLOR_GREEN")
    E = [o.measurables()[0][0]]
    for _ in range(2):
        o.step(5)
        E.append(o.measurables()[0][0])
    assert np.allclose(main["/TotalEnergy"][0], E, rtol=1e-12)
    assert np.allclose(main["/Time"][0], [0.0, 0.01, 0.02], rtol=0, atol=1e-15)
    u10, attrs = main["/Iter_00010/u_hat"]
    assert attrs["Iter"] == 10 and abs(attrs["TimeValue"] - 0.02) < 1e-15
    ref = o.get_state()
    assert np.linalg.norm(u10 - ref) / np.linalg.norm(ref) < 1e-12
    _, Ek, _ = o.measurables()
    assert np.allclose(spec["/Iter_00010/EnergySpectrum"][0], Ek, rtol=1e-12, atol=1e-14 * Ek.max())
    assert set(k for k in main if not k.startswith("/Iter")) >= {
        "/kx", "/ky", "/kz", "/x", "/y", "/z", "/Time", "/TotalEnergy", "/TotalEnstrophy",
        "/TotalPalinstrophy", "/TotalHelicity", "/EnergyDissipation"}


@pytest.mark.gpu
@pytest.mark.parametrize("integ", ["rk5cn", "dp5cn"])
def test_driver_rk5_integrators_match_oracle(ns3d, oracle, tmp_path, integ):
    """The solver binary with -I rk5cn (fixed step) and -I dp5cn (the
    Dormand-Prince loop of solver.c:125-194: step while t + dt <= T, record
    every step) against the oracle driven the same way."""
    exe = solver_bin(ns3d)
    N, nu, dt, T = 32, 0.01, 2e-3, 0.02
    args = [exe, "-o", str(tmp_path), "-n", str(N), "-n", str(N), "-n", str(N), "-s", "0.0", "-e", str(T),
            "-h", str(dt), "-v", str(nu), "-i", "TAYLOR_GREEN", "-p", "1", "-I", integ, "-t", "R5", "-L"]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tag = {"rk5cn": "RK5", "dp5cn": "DP5"}[integ]
    sub = [d for d in os.listdir(tmp_path) if d.startswith(f"SIM_DATA_NAVIER_{tag}_FULL_N[32,32]")]
    assert len(sub) == 1, os.listdir(tmp_path)
    main = read_container(os.path.join(tmp_path, sub[0], "Main_HDF_Data.ns3d"))
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK5CN if integ == "rk5cn" else oracle.DP5CN)
    o.ic("TAYLOR_GREEN")
    ts, E = [0.0], [o.measurables()[0][0]]
    while True:
        t, h, _ = o.get_time()
        if t + h > T + 1e-12 * T:
            break
        o.step(1)
        ts.append(o.get_time()[0])
        E.append(o.measurables()[0][0])
    Ts = main["/Time"][0]
    assert len(Ts) == len(ts)
    assert np.allclose(Ts, ts, rtol=1e-12, atol=1e-15)
    assert np.allclose(main["/TotalEnergy"][0], E, rtol=1e-12)
    steps = np.diff(Ts)
    if integ == "rk5cn":
        assert len(Ts) == 11 and np.allclose(steps, dt, rtol=1e-9)
    else:
        assert np.ptp(steps) > 1e-3 * dt   # the control changed the step size


@pytest.mark.gpu
def test_driver_defaults_are_the_reference_build(ns3d, oracle, tmp_path):
    """With no integrator or viscosity flag the binary runs what the
    reference's default build runs: RK4 + Crank-Nicolson (RK4Step,
    solver.c:505-608) with hyperviscosity nu k^4 (Makefile:44)."""
    exe = solver_bin(ns3d)
    N, nu, dt = 16, 1e-3, 2e-3
    args = [exe, "-o", str(tmp_path), "-n", str(N), "-n", str(N), "-n", str(N), "-s", "0.0", "-e", "0.01",
            "-h", str(dt), "-v", str(nu), "-i", "TAYLOR_GREEN", "-p", "5", "-t", "D"]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sub = [d for d in os.listdir(tmp_path) if d.startswith("SIM_DATA_NAVIER_RK4_FULL_N[16,16]")]
    assert len(sub) == 1, os.listdir(tmp_path)
    main = read_container(os.path.join(tmp_path, sub[0], "Main_HDF_Data.ns3d"))
    o = oracle.Oracle(N, nu=nu, dt=dt, integrator=oracle.RK4CN, visc_pow=2)
    o.ic("TAYLOR_GREEN")
    o.step(5)
    u5, _ = main["/Iter_00005/u_hat"]
    ref = o.get_state()
    assert np.linalg.norm(u5 - ref) / np.linalg.norm(ref) < 1e-12
    assert main["/EnergyDissipation"][0][-1] == pytest.approx(o.measurables()[0][4], rel=1e-12)


@pytest.mark.gpu
def test_checkpoint_resume_is_bitwise(ns3d, tmp_path):
    exe = solver_bin(ns3d)
    base = ["-n", "32", "-n", "32", "-n", "32", "-h", "2e-3", "-v", "0.005", "-i", "SPECTRUM", "-S", "3",
            "-f", "SHELL", "-p", "10", "-x"]
    a, b, c = tmp_path / "a", tmp_path / "b", tmp_path / "c"
    for d in (a, b, c):
        d.mkdir()
    subprocess.run([exe, "-o", str(a), "-o", str(a), "-s", "0", "-e", "0.02"] + base, check=True, capture_output=True)
    ck = [f for f in os.listdir(a) if f.startswith("Checkpoint")][0]
    subprocess.run([exe, "-o", str(b), "-o", str(b), "-s", "0", "-e", "0.04", "-z", str(a / ck)] + base, check=True,
                   capture_output=True)
    subprocess.run([exe, "-o", str(c), "-o", str(c), "-s", "0", "-e", "0.04"] + base, check=True, capture_output=True)

    def state(d):
        f = [x for x in os.listdir(d) if x.startswith("Checkpoint")][0]
        raw = open(d / f, "rb").read()
        return raw[-(32 * 32 * 17 * 3 * 16):]

    assert state(b) == state(c)
