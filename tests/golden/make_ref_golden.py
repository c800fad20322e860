"""Generate tests/golden/ref_N16.npz from the reference's own code.

The reference's Solver/src/solver.c and utils.c are compiled unchanged against
the single-rank MPI / FFTW-MPI stand-ins of oracle/ref_shim (make -C oracle
ref, which reads the reference sources from /root/reference) and called
through oracle/ref.py. The fixture lets the oracle (tests/test_reference_golden.py)
and the GPU path (tests/test_gpu_parity.py) be held to the reference's outputs
where the reference sources are absent.

Contents (N = 16; Fourier arrays complex128[N][N][N/2+1][3]):
  uh          dealiased input: rfftn of seeded normal noise (seed 16), |k| > N/3 zeroed
  rhs         NonlinearRHSBatch(uh) (variant nu; carries D2)
  rk4cn3      uh after 3 RK4Step, nu = 0.02, dt = 2e-3 (variant nu, nu k^2)
  rk4cn3_hyper  the same with the hyper variant (nu k^4)
  tot, Ek, Ok ComputeSystemMeasurables(uh), nu = 0.01, variant nu (tot carries D4/D12)
  tot_hyper   the totals with the hyper variant
  random_ic   InitialConditions with u0 RANDOM (srand(123456789); D2 and D6)

Run: python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref as R  # noqa: E402


def dealiased_field(N, seed):
    rng = np.random.default_rng(seed)
    uh = np.fft.rfftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2))
    k = np.fft.fftfreq(N, 1.0 / N)
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + np.arange(N // 2 + 1)[None, None, :] ** 2
    uh[np.sqrt(K2) > N // 3] = 0
    return uh


def main():
    if not R.build():
        raise SystemExit("the reference sources are needed (make -C oracle ref)")
    N = 16
    uh = dealiased_field(N, 16)
    out = {"uh": uh}
    r = R.Reference(N, nu=0.01, variant="nu")
    out["rhs"] = r.rhs(uh)
    r.set_state(uh)
    out["tot"], out["Ek"], out["Ok"] = r.measurables()
    r.close()
    r = R.Reference(N, nu=0.01, variant="hyper")
    r.set_state(uh)
    out["tot_hyper"] = r.measurables()[0]
    r.close()
    for variant, key in (("nu", "rk4cn3"), ("hyper", "rk4cn3_hyper")):
        r = R.Reference(N, nu=0.02, dt=2e-3, variant=variant)
        r.set_state(uh)
        r.rk4_step(2e-3, 3)
        out[key] = r.get_state()
        r.close()
    r = R.Reference(N, nu=0.01, u0="RANDOM", variant="nu")
    r.initial_conditions()
    out["random_ic"] = r.get_state()
    r.close()
    np.savez_compressed(os.path.join(HERE, f"ref_N{N}.npz"), **out)


if __name__ == "__main__":
    main()
