"""Benchmark of the GB300 time-stepping hot path.

Workload (the configuration the headline metric is quoted on): forced
turbulence on a 512^3 periodic grid, FP32 bulk arithmetic with FP64
integrating factors, time accumulator and reductions; seeded random-phase
solenoidal initial field with E(k) ~ k^4 exp(-2 (k/4)^2) at unit energy;
nu = 1e-3; energy of shells k <= 2 held constant; CFL 0.5; integrating-factor
RK4; 2/3-rule dealiasing. A step is one full RK4 time step (four nonlinear
evaluations). Synthetic data: every input is generated from a seed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). value = grid points x steps / second summed
over ranks (each rank runs its own replica: the solver does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
SAVE_EVERY = 100   # diagnostics cadence inside the timed steps (SAVE_EVERY of the reference's runs)
sys.path.insert(0, ROOT)

UNIT = "grid-pt*steps/s"


def nu_for(N: int) -> float:
    """nu = 1e-3 at 512^3; the 1024^3 variant of the configuration runs nu = 4e-4."""
    return 4e-4 if N >= 1024 else 1e-3


def metric(N: int) -> str:
    return f"grid-pt*RK4-steps/s ({N}^3, FP32 bulk, forced turbulence)"


def workload(N: int) -> dict:
    nu = nu_for(N)
    nzp = (N // 3 + 1 + 7) // 8 * 8     # stored kz modes per (kx, ky) column
    field_mb = N * N * nzp * 8 / 1e6     # one FP32 complex component
    return dict(workload=f"forced turbulence {N}^3, FP32 bulk + FP64 integrating factors/reductions, IF-RK4, "
                         f"2/3 dealias, shell k<=2 energy forcing, CFL 0.5, SPECTRUM IC k0=4 seed 0, nu={nu:g}",
                N=N, nu=nu, cfl=0.5, k0=4.0, seed=0, forcing="shell k<=2", integrator="IF-RK4",
                precision="fp32 bulk",
                l2=f"inputs larger than L2: each state field {field_mb:.0f} MB > 129 MB L2")


def lr_chunks(iters: int, schedule: str):
    """The Adam training of the LES mode as (iterations, learning rate) chunks: "const" is lr 1e-3
    throughout; "step" is 1e-3, 3e-4 and 1e-4 over 50 / 30 / 20 % of the iterations (the last chunk
    takes the remainder, so the chunks add up to iters)."""
    sched = [(1.0, 1e-3)] if schedule == "const" else [(0.5, 1e-3), (0.3, 3e-4), (0.2, 1e-4)]
    out, done = [], 0
    for i, (frac, lr) in enumerate(sched):
        it = iters - done if i == len(sched) - 1 else int(round(frac * iters))
        if it > 0:
            out.append((it, lr))
        done += it
    return out


def host_link(h2d: int, d2h: int, stream, e2e_step_ms: float, step_ms: float, reps: int = 3):
    """The host link's copy rates for the e2e leg's byte counts: one pinned -> device and one
    device -> pinned copy of the same sizes (DMA, CUDA events on the solver stream). The
    transfer floor is the time those bytes take at those rates; the e2e step cannot go below
    that floor plus the device step while the transfers and the step run one after the other."""
    import torch
    hb = torch.empty(max(h2d, d2h), dtype=torch.uint8, pin_memory=True)
    db = torch.empty(max(h2d, d2h), dtype=torch.uint8, device="cuda")
    rates = {}
    with torch.cuda.stream(stream):
        for name, nb, dst, src in (("h2d", h2d, db, hb), ("d2h", d2h, hb, db)):
            dst[:nb].copy_(src[:nb], non_blocking=True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                dst[:nb].copy_(src[:nb], non_blocking=True)
            e1.record(stream)
            e1.synchronize()
            rates[name] = reps * nb / (e0.elapsed_time(e1) / 1e3) / 1e9
    floor = h2d / rates["h2d"] / 1e6 + d2h / rates["d2h"] / 1e6
    del hb, db
    return {"h2d_GBps": rates["h2d"], "d2h_GBps": rates["d2h"], "transfer_floor_ms": floor,
            "device_step_ms": step_ms, "e2e_step_ms": e2e_step_ms,
            "frac_of_serial_bound": (floor + step_ms) / e2e_step_ms}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=512)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--shape", type=int, nargs=2, metavar=("VARIANT", "ZFORM"),
                    help="run this tile variant and z-pass form (no autotuning)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--workload", default="forced512",
                    choices=["forced512", "ensemble", "les", "decay256", "closure-infer", "integrators", "fp32err512",
                             "zgemm", "closure-train"])
    ap.add_argument("--err-steps", type=int, default=1000)
    ap.add_argument("--snapshots", type=int, default=2000)
    ap.add_argument("--train-iters", type=int, default=2000)
    ap.add_argument("--les-steps", type=int, default=2000)
    ap.add_argument("--les-seeds", type=int, default=1,
                    help="closure networks trained from seeds 0..n-1 on the same data (the spread of the gain)")
    ap.add_argument("--lr-schedule", default="const", choices=["const", "step"],
                    help="const: lr 1e-3 throughout; step: 1e-3, 3e-4, 1e-4 over 50 / 30 / 20 %% of the iterations")
    ap.add_argument("--decay-steps", type=int, default=1000)
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks for N independent replicas (torch.distributed)."""

    def __init__(self, ws, rank, local, use_cuda):
        self.ws, self.rank = ws, rank
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if use_cuda else "gloo"
            if use_cuda:
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.dist, self.torch = dist, torch
            self.dev = torch.device("cuda", local) if use_cuda else torch.device("cpu")

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_traffic(kernel: str, N: int, prec: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        f = line.split()
        if len(f) >= 4 and f[0] == kernel and f[1] == f"N={N}" and f[2] == prec:
            try:
                return float(f[3].split("=")[1])
            except (IndexError, ValueError):
                return None
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def oracle_for(N: int, nthreads: int = 0):
    """The oracle (CPU FP64 restatement) on the bench's configuration: IF-RK4,
    CFL 0.5, shell k <= 2 forcing, SPECTRUM k0 = 4 seed 0."""
    from oracle import oracle as O
    O.build()
    o = O.Oracle(N, nu=nu_for(N), dt=1e-3, cfl=0.5, forcing=O.FORCE_SHELL, force_k=2, nthreads=nthreads)
    o.ic("SPECTRUM", seed=0, k0=4.0, energy=1.0)
    return o, O.threads()


def cpu_baseline(N: int):
    """The oracle timed on a bounded sample of the workload: one whole RK4
    step at N^3 (four nonlinear evaluations, the stage updates, the CFL step
    and the forcing), after one untimed step."""
    o, cores = oracle_for(N)
    o.step(1)
    t0 = time.perf_counter()
    o.step(1)
    t = time.perf_counter() - t0
    return {"value": N ** 3 / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one whole IF-RK4 step at {N}^3 in FP64 ({t:.1f} s, after one untimed step), "
                      f"oracle restatement with its own FFT (batched Stockham, no FFTW on the host), {cores} threads"}


def run_reference(args, ws, rank):
    """Reference arm: the reference's CPU path on the host cores. The reference
    program needs FFTW3-MPI, MPI and HDF5, which neither machine has, and its
    compiled parts cannot travel to the Arm GPU host, so the arm times the
    oracle restatement (pinned against the reference's own code), all host
    threads. Each bench step is one RK4 stage of the workload (one nonlinear
    evaluation and its stage update; every fourth stage also the final update
    and the forcing): --steps K stages are K/4 RK4 steps, timed back to back
    after --warmup W untimed stages."""
    if rank != 0:
        return
    N = args.N
    o, cores = oracle_for(N)
    for _ in range(args.warmup):
        o.stage()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.stage()
    t = time.perf_counter() - t0
    val = N ** 3 * (args.steps / 4.0) / t
    sample = (f"each bench step = one RK4 stage at {N}^3 in FP64 (1/4 of an RK4 step: a NonlinearRHSBatch and "
              f"its stage update, every fourth with the final update and forcing); {args.steps} stages = "
              f"{args.steps / 4:g} RK4 steps in {t:.1f} s; value = N^3 x (K/4) / t; oracle restatement, "
              f"own FFT (batched Stockham, no FFTW on the host), {cores} threads")
    line = {"impl": "reference", "metric": metric(N), "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload(N),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    pkg.lib()
    torch.cuda.set_device(local)
    dist = Dist(ws, rank, local, True)
    N = args.N
    cfg = dict(nu=nu_for(N), dt=1e-3, cfl=0.5, precision="fp32", forcing="SHELL", force_k=2, device=local)
    tuned = None
    if args.shape:
        pkg.tuning_set(N, args.shape[0], zform=args.shape[1], precision="fp32")
        tuned = {"N": N, "variant": args.shape[0], "zform": args.shape[1], "chosen_by": "--shape"}
    elif not args.no_autotune:
        # the library's autotuner picks the tile / radix variant and z-pass form of this size (untimed)
        tuned, tried = pkg.autotune(N, steps=20, **cfg)
        tuned = dict(tuned, tried=[[t["variant"], t["zform"], round(t["ms_per_step"], 4)] for t in tried])
    s = pkg.Solver(N, **cfg)
    s.InitialConditions("SPECTRUM", seed=0, k0=4.0, energy=1.0)
    stream = torch.cuda.ExternalStream(s.stream)
    s.RK4Step(args.warmup)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the metric's diagnostics: ComputeSystemMeasurables once per SAVE_EVERY = 100 steps (the
    # reference's save cadence), inside the timed region, and at least once in any window
    # (K < 100 steps are charged a whole call)
    saves = max(1, round(args.steps / SAVE_EVERY))
    every = args.steps // saves
    ev0.record(stream)
    done, lib_ms, made = 0, 0.0, 0
    while done < args.steps:
        n = min(args.steps - done, every)
        s.RK4Step(n)
        lib_ms += s.last_step_ms()
        done += n
        if made < saves and (done % every == 0 or done == args.steps):
            s.ComputeSystemMeasurables()
            made += 1
    ev1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max = dist.max(ms)
    value = ws * N ** 3 * args.steps / (ms_max / 1e3)
    tot, _, _ = s.ComputeSystemMeasurables()
    t_sim, dt_sim, iters = s.get_time()

    # per-kernel device times (CUDA events on the solver stream) for the roofline
    prof = s.profile_step(reps=2)
    peak, peak_kind = read_peaks()
    # algorithmic bytes per launch: the per-pass scalar-field counts of the step's byte model
    # (P1 R3 W6, P2 R6 W6, P3 R6 W3, P4 R3 W3, P5 R3 + state: 9/12/12/9 over the 4 stages),
    # each field M = N^3 FP32 words; the design's own compulsory bytes (dealiased subset only)
    # and the measured DRAM traffic are reported beside them
    field = N ** 3 * 4
    model_fields = {"k_xinv": 9, "k_ypass_inv": 12, "k_zline": 9, "k_zpass": 9, "k_ypass_fwd": 6,
                    "k_xfwd": 3 + (9 + 12 + 12 + 9) / 4}
    best = max((p for p in prof if p[0] != "k_misc"), key=lambda p: p[1] * 4)
    alg = model_fields[best[0]] * field
    ach = alg / (best[1] / 1e3) / 1e9
    traffic = read_traffic(best[0], N, "fp32")
    roofline = {"bound": "hbm", "kernel": best[0], "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg, "ms_per_launch": best[1],
                "design_compulsory_bytes_per_launch": best[2],
                "design_compulsory_frac": best[2] / (best[1] / 1e3) / 1e9 / peak,
                "kernels": {p[0]: {"ms": p[1],
                                   "alg_GBps": model_fields[p[0]] * field / (p[1] / 1e3) / 1e9 if p[0] in model_fields else None,
                                   "compulsory_GBps": (p[2] / (p[1] / 1e3) / 1e9) if p[2] else None} for p in prof}}
    step_bytes = sum(p[2] * 4 for p in prof)
    # the per-pass field model: 198 scalar-field passes of N^3 FP32 words per RK4 step
    model_bytes = 198.0 * N ** 3 * 4
    roofline["step_compulsory_GB"] = step_bytes / 1e9
    roofline["step_field_model_GBps"] = model_bytes / (ms_max / args.steps / 1e3) / 1e9

    e2e = None
    if not args.no_e2e:
        # e2e: RK4Step's host-array contract through the C ABI (pinned host buffers,
        # H2D of u_hat, one step, D2H of u_hat, every step)
        fshape = (N, N, N // 2 + 1, 3)
        hin = torch.empty(fshape + (2,), dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)[..., 0]
        hout = torch.empty(fshape + (2,), dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)[..., 0]
        hin[...] = s.get_state()
        for _ in range(2):        # warm: first-touch of the pinned arrays, line plans
            s.step_host(hin, hout)
        ke = max(1, args.e2e_steps)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(ke):
            s.step_host(hin, hout)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = dist.max(e0.elapsed_time(e1))
        nbytes = int(np.prod(fshape)) * 16
        h2d, d2h = s.io_bytes()   # bytes that crossed the host link per call (dealiased modes / their lines)
        e2e = {"value": ws * N ** 3 * ke / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "host_array_bytes": nbytes, "steps": ke,
               "call": "ns3d_step_host(ctx, u_hat_in, u_hat_out), reference layout complex128[N][N][N/2+1][3], "
                       "pinned host arrays",
               "link": host_link(h2d, d2h, stream, e2e_ms / ke, ms_max / args.steps)}
    s.close()

    fp64 = None
    if not args.no_fp64:
        s64 = pkg.Solver(N, nu=nu_for(N), dt=1e-3, cfl=0.5, precision="fp64", forcing="SHELL", force_k=2,
                         device=local)
        s64.InitialConditions("SPECTRUM", seed=0, k0=4.0, energy=1.0)
        s64.RK4Step(1)
        torch.cuda.synchronize()
        k64 = 3
        s64.RK4Step(k64)
        ms64 = s64.last_step_ms()
        v64 = N ** 3 * k64 / (ms64 / 1e3)
        fp64 = {"value": v64, "ms_per_step": ms64 / k64, "steps": k64, "fp32_over_fp64": (value / ws) / v64}
        s64.close()

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(N)
    dist.close()
    if rank != 0:
        return
    line = {"metric": metric(N), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(workload(N), parallelism=f"replicas x{ws}", autotune=tuned,
                           diagnostics=f"ComputeSystemMeasurables once per {SAVE_EVERY} steps inside the timed "
                                       f"steps, at least once per window ({saves} call(s) in {args.steps} steps)"),
            "clocks": clocks, "e2e": e2e, "gpu_launches": s_kernels(pkg, N) * args.steps + 2 * saves,
            "roofline": roofline, "cpu_baseline": cpu, "fp64": fp64,
            "library_ms_per_step": lib_ms / args.steps,
            "state_after": {"t": t_sim, "dt": dt_sim, "iters": iters, "energy": tot["energy"]}}
    print(json.dumps(line), flush=True)


def s_kernels(pkg, N):
    s = pkg.Solver(16, cfl=0.5, precision="fp32", forcing="SHELL", force_k=2)
    k = s.kernels_per_step
    s.close()
    return k


def run_ensemble(args, local):
    """Config C4: 96 independent FP32 runs (32 x 48^3, 32 x 64^3, 24 x 96^3, 8 x 128^3), each with its own
    seeded SPECTRUM initial field (k0 ~ U[2, 6]) and nu log-uniform in [5e-4, 5e-3], CFL 0.5, IF-RK4,
    stepped together (one CUDA graph launch per step). Prints one JSON line."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    rng = np.random.default_rng(2024)
    sizes = [48] * 32 + [64] * 32 + [96] * 24 + [128] * 8
    k0 = rng.uniform(2.0, 6.0, len(sizes))
    nu = np.exp(rng.uniform(np.log(5e-4), np.log(5e-3), len(sizes)))
    members = [dict(N=n, nu=float(v), dt=1e-3, cfl=0.5, precision="fp32", device=local) for n, v in zip(sizes, nu)]
    # autotuner: tile variant and z-pass form per grid size, timed with each size's members
    t0 = time.perf_counter()
    tuned = pkg.autotune_ensemble(members, steps=10)
    tune_s = time.perf_counter() - t0
    ens = pkg.Ensemble(members)
    for i in range(len(sizes)):
        ens.InitialConditions(i, "SPECTRUM", seed=i, k0=float(k0[i]))
    ens.step(args.warmup)
    torch.cuda.synchronize()
    clk = Clocks(local)
    ens.step(args.steps)
    ms_per_launch = ens.last_step_ms()          # one graph launch per step
    ens.run(args.steps)                         # the same steps in one launch (device-side loop)
    clocks = clk.stop()
    ms = ens.last_step_ms()
    groups, kps = ens.info()
    pts = sum(n ** 3 for n in sizes)
    e0 = [ens.measurables(i)[0]["energy"] for i in (0, 32, 64, 88)]
    # per launch group, after the timed steps: each kernel class's device time (ms per launch)
    group_profile = {}
    for g in range(groups):
        n, prof = ens.profile_group(g, reps=3)
        group_profile[str(n)] = {name: round(t, 4) for name, t, _ in prof}
    line = {"metric": "ensemble grid-pt*RK4-steps/s (96 runs: 32x48^3, 32x64^3, 24x96^3, 8x128^3)",
            "value": pts * args.steps / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched ensemble, FP32, IF-RK4, CFL 0.5, the whole run in one graph launch",
                       "members": len(sizes), "launch_groups": groups, "grid_points": pts},
            "clocks": clocks, "gpu_launches": (kps + 1) * args.steps,
            "timing": f"ns3d_ensemble_run: {args.steps} steps in one graph launch (a device-side while loop); "
                      f"one launch per step: {ms_per_launch / args.steps:.4f} ms/step",
            "autotune": {"seconds": tune_s, "choices": tuned},
            "group_profile_ms": group_profile,
            "energy_samples": e0}
    print(json.dumps(line), flush=True)
    ens.close()


def run_les(args, local):
    """Config C5: snapshots of a seeded forced 256^3 FP32 DNS box-filtered to 64^3 train the closure
    network on the GPU; a 64^3 run with the closure and the plain 64^3 solve then start from the filtered
    DNS and are compared with it after the same number of steps (E(k) log error over k = 1..21), with
    their speeds. --snapshots, --train-iters and --les-steps set the sizes."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    pkg.tuning_load(os.path.join(ROOT, "3d_navier_stokes_gb300", "tuning", "gb300.txt"))
    Nf, Nc, nu, dt = 256, 64, 1.5e-3, 1e-3
    dns = pkg.Solver(Nf, nu=nu, dt=dt, precision="fp32", forcing="SHELL", force_k=2, device=local)
    dns.InitialConditions("SPECTRUM", seed=0, k0=3.0)
    dns.RK4Step(500)
    nseed = max(1, args.les_seeds)
    nets = [pkg.LES(Nc, capacity=args.snapshots, seed=s) for s in range(nseed)]
    t0 = time.perf_counter()
    for _ in range(args.snapshots):
        dns.RK4Step(5)
        for les in nets:
            les.add_snapshot(dns)
    t_data = time.perf_counter() - t0
    loss0 = nets[0].dataset_loss()
    t_train, loss_tr, loss1 = [], [], []
    for les in nets:
        t0 = time.perf_counter()
        tail = 0.0
        for it, lr in lr_chunks(args.train_iters, args.lr_schedule):
            tail = les.train(it, lr=lr)
        t_train.append(time.perf_counter() - t0)
        loss_tr.append(tail)
        loss1.append(les.dataset_loss())
    ubar = nets[0].filtered_velocity(dns)
    runs = {}
    for name in ["plain"] + [f"closure{s}" for s in range(nseed)]:
        c = pkg.Solver(Nc, nu=nu, dt=dt, precision="fp32", forcing="SHELL", force_k=2, device=local)
        c.set_state_real(ubar)
        if name != "plain":
            c.attach_closure(nets[int(name[7:])])
        runs[name] = c
    ms = {}
    dns.RK4Step(args.les_steps)
    ms["dns"] = dns.last_step_ms() / args.les_steps
    ms["closure_inference"] = nets[0].profile_infer(20)
    for n, c in runs.items():
        c.RK4Step(args.les_steps)
        ms[n] = c.last_step_ms() / args.les_steps
    ref = pkg.Solver(Nc, nu=nu, dt=dt, precision="fp32", device=local)
    ref.set_state_real(nets[0].filtered_velocity(dns))
    _, Eref, _ = ref.ComputeSystemMeasurables()
    k = np.arange(1, Nc // 3 + 1)
    err = {}
    for n, c in runs.items():
        _, E, _ = c.ComputeSystemMeasurables()
        err[n] = float(np.sqrt(np.mean((np.log(E[k]) - np.log(Eref[k])) ** 2)))
    cl = [err[f"closure{s}"] for s in range(nseed)]
    counters = [runs[f"closure{s}"].closure_counters() for s in range(nseed)]
    line = {"metric": "LES E(k) log-error vs filtered 256^3 DNS (64^3, closure vs plain)",
            "value": float(np.mean(cl)), "unit": "rms log E(k) error", "higher_is_better": False,
            "plain_coarse_error": err["plain"], "closure_error_per_seed": cl,
            "closure_error_range": [min(cl), max(cl)], "margin_vs_plain": err["plain"] - max(cl),
            "n_gpus": 1, "steps": args.les_steps, "dtype": "f32 (bf16 weights)",
            "data": "synthetic", "config": {"workload": "learned closure C5", "dns_N": Nf, "les_N": Nc, "nu": nu,
                                            "dt": dt, "snapshots": args.snapshots, "train_iters": args.train_iters,
                                            "seeds": nseed, "lr_schedule": args.lr_schedule},
            "ms_per_step": {"dns_256": ms["dns"], "les_64_closure": ms["closure0"], "plain_64": ms["plain"],
                            "closure_inference": ms["closure_inference"]},
            "inference_tflops": 126144.0 * Nc ** 3 / (ms["closure_inference"] * 1e-3) / 1e12,
            "speedup_vs_dns": ms["dns"] / ms["closure0"],
            "closure_steps": [c[0] for c in counters], "fallback_steps": [c[1] for c in counters],
            "loss": {"before": loss0, "after": loss1, "train_tail": loss_tr},
            "seconds": {"data": t_data, "train": t_train}}
    print(json.dumps(line), flush=True)
    for les in nets:
        les.close()


def run_closure_infer(args, local):
    """Closure inference alone: the 4-layer network on a 64^3 grid (tensor-core path), random
    weights and input, mean device time of --steps calls after --warmup."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    D = 64
    les = pkg.LES(D, capacity=0, seed=1)
    u = np.random.default_rng(0).standard_normal((3, D, D, D)).astype(np.float32)
    tau = les.infer(u)
    les.profile_infer(max(1, args.warmup))
    ms = les.profile_infer(max(1, args.steps))
    flops = 126144.0 * D ** 3
    print(json.dumps({"metric": "closure inference (64^3, 4 conv layers, tcgen05 BF16 / FP32 accumulate)",
                      "value": ms, "unit": "ms", "higher_is_better": False, "tflops": flops / (ms * 1e-3) / 1e12,
                      "steps": args.steps, "finite": bool(np.isfinite(tau).all())}), flush=True)
    les.close()


def run_closure_train(args, local):
    """Closure training alone at 64^3: 8 box-filtered snapshots of a seeded forced 256^3 FP32
    run, then --warmup untimed and --steps timed Adam iterations on each training path (the
    tensor cores: BF16 operands, FP32 accumulation; and the FP32 CUDA-core kernels), from the
    same initial weights; ms per iteration (wall clock: each iteration reads its loss back)."""
    import importlib
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    pkg.tuning_load(os.path.join(ROOT, "3d_navier_stokes_gb300", "tuning", "gb300.txt"))
    dns = pkg.Solver(256, nu=1.5e-3, dt=1e-3, precision="fp32", forcing="SHELL", force_k=2, device=local)
    dns.InitialConditions("SPECTRUM", seed=0, k0=3.0)
    dns.RK4Step(20)
    out = {}
    for path in ("tc", "fp32"):
        les = pkg.LES(64, capacity=8, seed=0)
        les.set_train_path(path)
        for _ in range(8):
            dns.RK4Step(2)
            les.add_snapshot(dns)
        les.train(max(1, args.warmup), lr=1e-3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = les.train(args.steps, lr=1e-3)
        t = time.perf_counter() - t0
        out[path] = {"ms_per_iteration": 1e3 * t / args.steps, "loss_tail": loss}
        les.close()
    line = {"metric": "closure training ms per Adam iteration (64^3, 4 conv layers, 32 channels)",
            "value": out["tc"]["ms_per_iteration"], "unit": "ms", "higher_is_better": False,
            "steps": args.steps, "warmup": args.warmup, "n_gpus": 1, "data": "synthetic",
            "dtype": "bf16 operands, f32 accumulation (tc); f32 (fp32)", "paths": out,
            "speedup_tc_over_fp32": out["fp32"]["ms_per_iteration"] / out["tc"]["ms_per_iteration"],
            "config": {"workload": "closure training", "Nc": 64, "snapshots": 8, "dns_N": 256}}
    print(json.dumps(line), flush=True)


def run_decay(args, local):
    """Config C2: decaying turbulence at 256^3 (SPECTRUM IC k0 = 4, nu = 2e-3, CFL 0.5, IF-RK4,
    --decay-steps steps) in FP64 and in FP32; reports the FP32 relative errors of the energy, the
    dissipation and E(k) against FP64, and both step rates."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    N, steps = 256, args.decay_steps
    res = {}
    for prec in ("fp64", "fp32"):
        s = pkg.Solver(N, nu=2e-3, dt=1e-3, cfl=0.5, precision=prec, device=local)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s.RK4Step(steps)
        tot, Ek, _ = s.ComputeSystemMeasurables()
        res[prec] = (tot, Ek, s.last_step_ms() / steps, s.get_time())
        s.close()
    t64, t32 = res["fp64"][0], res["fp32"][0]
    E64, E32 = res["fp64"][1], res["fp32"][1]
    kk = np.arange(1, N // 3 + 1)
    line = {"metric": "FP32 vs FP64 relative energy error, 256^3 decaying turbulence",
            "value": abs(t32["energy"] - t64["energy"]) / t64["energy"], "unit": "relative error",
            "higher_is_better": False, "steps": steps, "n_gpus": 1, "data": "synthetic", "dtype": "f32 vs f64",
            "dissipation_rel_err": abs(t32["dissipation"] - t64["dissipation"]) / t64["dissipation"],
            "Ek_max_rel_err_k1_to_85": float(np.max(np.abs(E32[kk] - E64[kk]) / E64[kk])),
            "ms_per_step": {"fp64": res["fp64"][2], "fp32": res["fp32"][2]},
            "fp32_over_fp64_speed": res["fp64"][2] / res["fp32"][2],
            "t_final": {"fp64": res["fp64"][3][0], "fp32": res["fp32"][3][0]},
            "config": {"workload": "decaying turbulence C2", "N": N, "nu": 2e-3, "cfl": 0.5, "k0": 4.0}}
    print(json.dumps(line), flush=True)


def run_fp32err(args, local):
    """Config C3's accuracy bar: forced turbulence at N^3 (default 512^3; SPECTRUM IC k0 = 4 seed 0,
    nu = 1e-3, CFL 0.5, shell k <= 2 forcing, IF-RK4) for --err-steps steps (default 1000) in FP64 and
    in FP32 bulk from the same initial field; the FP32 relative errors of the energy, the dissipation
    and every E(k) shell against FP64, every 100 steps and at the end, and both step rates."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    pkg.tuning_load(os.path.join(ROOT, "3d_navier_stokes_gb300", "tuning", "gb300.txt"))
    N, steps = args.N, args.err_steps
    every = 100 if steps >= 100 else steps
    res = {}
    for prec in ("fp64", "fp32"):
        s = pkg.Solver(N, nu=nu_for(N), dt=1e-3, cfl=0.5, precision=prec, forcing="SHELL", force_k=2, device=local)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        series, ms = [], 0.0
        done = 0
        while done < steps:
            n = min(every, steps - done)
            s.RK4Step(n)
            ms += s.last_step_ms()
            done += n
            tot, Ek, _ = s.ComputeSystemMeasurables()
            series.append((done, s.get_time()[0], tot["energy"], tot["dissipation"], Ek))
        res[prec] = (series, ms / steps)
        s.close()
    kk = np.arange(1, N // 3 + 1)
    rows = []
    for a, b in zip(res["fp64"][0], res["fp32"][0]):
        e64, e32 = a[4][kk], b[4][kk]
        # shells whose FP64 energy is above 1e-10 of the largest: early in the run the
        # highest shells hold energy at the FP32 roundoff level of the total, where a
        # relative error says nothing
        live = e64 > 1e-10 * e64.max()
        rows.append({"steps": a[0], "t_fp64": a[1], "t_fp32": b[1],
                     "energy_rel_err": abs(b[2] - a[2]) / a[2],
                     "dissipation_rel_err": abs(b[3] - a[3]) / a[3],
                     "Ek_max_rel_err": float(np.max(np.abs(e32 - e64) / e64)),
                     "Ek_max_rel_err_live_shells": float(np.max(np.abs(e32[live] - e64[live]) / e64[live])),
                     "live_shells": int(live.sum())})
    last = rows[-1]
    line = {"metric": f"FP32 vs FP64 relative energy error after {steps} steps, {N}^3 forced turbulence",
            "value": last["energy_rel_err"], "unit": "relative error", "higher_is_better": False,
            "target": 1e-5, "steps": steps, "n_gpus": 1, "data": "synthetic", "dtype": "f32 vs f64",
            "dissipation_rel_err": last["dissipation_rel_err"], "Ek_max_rel_err_all_shells": last["Ek_max_rel_err"],
            "max_over_checkpoints": {k: max(r[k] for r in rows) for k in
                                     ("energy_rel_err", "dissipation_rel_err", "Ek_max_rel_err_live_shells")},
            "series": rows, "ms_per_step": {"fp64": res["fp64"][1], "fp32": res["fp32"][1]},
            "fp32_over_fp64_speed": res["fp64"][1] / res["fp32"][1],
            "config": dict(workload(N), shells=f"k = 1..{N // 3}")}
    print(json.dumps(line), flush=True)


def run_zgemm(args, local):
    """The z-pass forms per grid size (N = 32 .. 128; FP32 engine, tile variant 0, IF-RK4,
    forced, CFL 0.5, SPECTRUM IC): device ms per step with the z transforms as FFTs
    (form 0: bulk-copy line kernel, form 1: CTA-synchronous) and as DFT matrix products on
    the tensor cores in split BF16 (form 2), and each form's error against the FP64 engine
    after --steps steps from the same initial field (relative L2 of the state, relative
    energy error)."""
    import importlib
    import numpy as np
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    out = {}
    for N in (32, 48, 64, 96, 128):
        cfg = dict(nu=2e-3, dt=1e-3, cfl=0.5, forcing="SHELL", force_k=2, device=local)
        s64 = pkg.Solver(N, precision="fp64", **cfg)
        s64.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s64.RK4Step(args.steps)
        ref = s64.get_state()
        e_ref = s64.ComputeSystemMeasurables()[0]["energy"]
        s64.close()
        rec = {}
        for z in (0, 1, 2):
            pkg.tuning_set(N, 0, zform=z, precision="fp32")
            s = pkg.Solver(N, precision="fp32", **cfg)
            s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
            s.RK4Step(args.steps)
            st = s.get_state()
            e = s.ComputeSystemMeasurables()[0]["energy"]
            s.RK4Step(max(3, args.warmup))
            s.RK4Step(args.steps)
            ms = s.last_step_ms() / args.steps
            kps = s.kernels_per_step
            s.close()
            rec[f"form{z}"] = {"ms_per_step": ms, "kernels_per_step": kps,
                               "state_rel_l2_vs_fp64": float(np.linalg.norm(st - ref) / np.linalg.norm(ref)),
                               "energy_rel_err_vs_fp64": abs(e - e_ref) / e_ref}
        out[str(N)] = rec
    pkg.tuning_clear()
    line = {"metric": "z-pass forms: ms per step and error vs FP64 (FP32 engine, forced IF-RK4, CFL 0.5)",
            "value": out["128"]["form2"]["ms_per_step"], "unit": "ms per step (128^3, form 2)",
            "higher_is_better": False, "steps": args.steps, "n_gpus": 1, "data": "synthetic", "dtype": "f32",
            "sizes": out,
            "config": {"workload": "z-pass forms", "nu": 2e-3, "cfl": 0.5, "forcing": "shell k<=2", "k0": 4.0,
                       "seed": 0, "tile_variant": 0}}
    print(json.dumps(line), flush=True)


def run_rk5(args, local):
    """The integrators of the step at N^3 (default 512^3) FP32 with shell forcing: IF-RK4,
    RK4CN (CFL 0.5), RK5CN (CFL 0.5, 6 RHS per step) and DP5CN (Dormand-Prince step
    control, 7 RHS per attempt); per integrator the device time per step (CUDA events of the
    library over --steps steps after --warmup) and the simulated time advanced per second."""
    import importlib
    import torch

    pkg = importlib.import_module("3d_navier_stokes_gb300")
    torch.cuda.set_device(local)
    # the shipped GB300 tuning table (the shapes bench's own tuning pass picks)
    pkg.tuning_load(os.path.join(ROOT, "3d_navier_stokes_gb300", "tuning", "gb300.txt"))
    N = args.N
    out = {}
    for integ in ("ifrk4", "rk4cn", "rk5cn", "dp5cn"):
        s = pkg.Solver(N, nu=4e-4 if N >= 1024 else 1e-3, dt=1e-3, cfl=0.0 if integ == "dp5cn" else 0.5,
                       precision="fp32", forcing="SHELL", force_k=2, integrator=integ, device=local)
        s.InitialConditions("SPECTRUM", seed=0, k0=4.0)
        s.RK4Step(args.warmup)
        t0 = s.get_time()[0]
        s.RK4Step(args.steps)
        ms = s.last_step_ms()
        t1, dt, _ = s.get_time()
        rec = {"ms_per_step": ms / args.steps, "grid_pt_steps_per_s": N ** 3 * args.steps / (ms * 1e-3),
               "sim_time_per_s": (t1 - t0) / (ms * 1e-3), "mean_dt": (t1 - t0) / args.steps,
               "kernels_per_step": s.kernels_per_step}
        if integ == "dp5cn":
            err, rej = s.dp_stats()
            rec["rejected_attempts"] = rej
        out[integ] = rec
        s.close()
    line = {"metric": f"grid-pt*steps/s per integrator ({N}^3, FP32 bulk, forced turbulence)",
            "value": out["rk5cn"]["grid_pt_steps_per_s"], "unit": "grid-pt*steps/s (RK5CN)",
            "higher_is_better": True, "steps": args.steps, "warmup": args.warmup, "n_gpus": 1,
            "data": "synthetic", "dtype": "f32", "integrators": out,
            "config": {"workload": "integrators", "N": N, "nu": 4e-4 if N >= 1024 else 1e-3, "cfl": 0.5,
                       "forcing": "shell k<=2", "k0": 4.0, "seed": 0, "dp5cn_tolerances": "1e-7 abs, 1e-7 rel"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload == "ensemble":
        run_ensemble(args, local)
        return
    if args.workload == "les":
        run_les(args, local)
        return
    if args.workload == "decay256":
        run_decay(args, local)
        return
    if args.workload == "closure-infer":
        run_closure_infer(args, local)
        return
    if args.workload == "integrators":
        run_rk5(args, local)
        return
    if args.workload == "fp32err512":
        run_fp32err(args, local)
        return
    if args.workload == "zgemm":
        run_zgemm(args, local)
        return
    if args.workload == "closure-train":
        run_closure_train(args, local)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
