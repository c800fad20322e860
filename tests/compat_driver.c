/*
 * A reference-shaped driver: the loop of SpectralSolve (solver.c:50-208)
 * written against include/ns3d_compat.h, i.e. the reference's function names
 * and global structs. Used by tests/test_driver_compat.py.
 *   compat_driver N nu dt nsteps integrator(0..3) visc_pow(0..2) out.bin
 * The switches are written into the zero-filled sys_vars as given (0 0 is the
 * reference's default build: RK4 + Crank-Nicolson, nu k^4). Integrators 0
 * and 1 step with RK4Step, 2 and 3 with RK5DPStep (for 3 the step size
 * follows the Dormand-Prince control through sys_vars->dt).
 * Writes u_hat after nsteps (complex double [N][N][N/2+1][3]) followed by the
 * energy/enstrophy series recorded after every step, then sys_vars->t and
 * sys_vars->dt (set by RK5DPStep for integrator 3).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ns3d_compat.h"

int main(int argc, char** argv) {
    if (argc != 8) return 2;
    system_vars_struct sv;
    runtime_data_struct rd;
    RK_data_struct rk;
    memset(&sv, 0, sizeof(sv));
    memset(&rd, 0, sizeof(rd));
    sys_vars = &sv;
    run_data = &rd;
    const long N = atol(argv[1]);
    const int steps = atoi(argv[4]);
    sv.N[0] = sv.N[1] = sv.N[2] = N;
    sv.local_Nx = N;
    sv.NU = atof(argv[2]);
    sv.dt = atof(argv[3]);
    sv.integrator = atoi(argv[5]);
    sv.visc_pow = atoi(argv[6]);
    strcpy(sv.u0, "TAYLOR_GREEN");
    strcpy(sv.forcing, "NONE");
    const long NF = N / 2 + 1;
    for (int d = 0; d < 3; ++d) {
        rd.x[d] = malloc(sizeof(double) * N);
        rd.k[d] = malloc(sizeof(int) * N);
    }
    rd.u_hat = malloc(sizeof(ns3d_fftw_complex) * N * N * NF * 3);
    rd.tot_energy = calloc(steps + 1, sizeof(double));
    rd.tot_enstr = calloc(steps + 1, sizeof(double));
    rd.tot_palin = calloc(steps + 1, sizeof(double));
    rd.tot_heli = calloc(steps + 1, sizeof(double));
    rd.enrg_diss = calloc(steps + 1, sizeof(double));
    InitializeSpaceVariables(rd.x, rd.k, sv.N);
    InitialConditions(rd.u_hat, NULL, sv.N);
    ComputeSystemMeasurables(0);
    for (int it = 1; it <= steps; ++it) {
        if (sv.integrator >= 2)
            RK5DPStep(sv.dt, sv.N, it, sv.local_Nx, &rk);
        else
            RK4Step(sv.dt, sv.N, sv.local_Nx, &rk);
        ComputeSystemMeasurables(it);
    }
    FILE* f = fopen(argv[7], "wb");
    fwrite(rd.u_hat, sizeof(ns3d_fftw_complex), N * N * NF * 3, f);
    fwrite(rd.tot_energy, sizeof(double), steps + 1, f);
    fwrite(rd.tot_enstr, sizeof(double), steps + 1, f);
    const double tdt[2] = {sv.t, sv.dt};
    fwrite(tdt, sizeof(double), 2, f);
    fclose(f);
    ns3d_compat_free();
    return 0;
}
