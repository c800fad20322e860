/*
 * ref_harness.c — ORACLE test infrastructure: a call surface over the
 * reference's own Solver/src/solver.c and utils.c, compiled unchanged
 * against the single-rank MPI / FFTW-MPI stand-ins of oracle/ref_shim.
 * The parity tests (tests/test_reference_parity.py) use it to pin the
 * oracle restatement (ns3d_oracle.c) against the reference's code itself.
 * Never linked into the product library.
 *
 * It defines what the reference's main.c and hdf5_funcs.c would:
 *   - the three global struct pointers (main.c:26-28);
 *   - the three hdf5_funcs.c writers that solver.c calls
 *     (CreateOutputFilesWriteICs, WriteDataToFile,
 *     FinalWriteAndCloseOutputFile), which here record the saved
 *     measurables and the final state in memory instead of writing HDF5.
 * Parameters reach sys_vars through the reference's own GetCMLArgs
 * (utils.c:34-237), given the same flags as the reference binary.
 */
#include <complex.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "data_types.h"
#include "hdf5_funcs.h"
#include "solver.h"
#include "utils.h"

/* main.c:26-28 */
runtime_data_struct* run_data;
system_vars_struct* sys_vars;
HDF_file_info_struct* file_info;

static runtime_data_struct g_run;
static system_vars_struct g_sys;
static HDF_file_info_struct g_file;
static RK_data_struct g_rk;
static long g_n[3];
static int g_ready = 0;

/* what the writer stand-ins record */
static double* g_series = NULL;    /* rows of [t, E, Omega, P, H, eps, Ek[n_spect], Ok[n_spect]] */
static int g_series_rows = 0, g_series_max = 0;
static double* g_final = NULL;     /* u_hat at FinalWriteAndCloseOutputFile */

int ref_n_spect(void) { return g_ready ? sys_vars->n_spect : -1; }
long ref_local_nx(void) { return g_ready ? (long)sys_vars->local_Nx : -1; }
int ref_hyper(void) {
#if defined(HYPER_VISC)
    return 1;
#else
    return 0;
#endif
}

static void record_row(double t, int idx) {
    if (!g_series || g_series_rows >= g_series_max) return;
    const int ns = sys_vars->n_spect;
    double* r = g_series + (size_t)g_series_rows * (6 + 2 * (size_t)ns);
    r[0] = t;
    r[1] = run_data->tot_energy[idx];
    r[2] = run_data->tot_enstr[idx];
    r[3] = run_data->tot_palin[idx];
    r[4] = run_data->tot_heli[idx];
    r[5] = run_data->enrg_diss[idx];
    memcpy(r + 6, run_data->enrg_spect, sizeof(double) * (size_t)ns);
    memcpy(r + 6 + ns, run_data->enst_spect, sizeof(double) * (size_t)ns);
    g_series_rows++;
}

/* hdf5_funcs.c stand-ins (the signatures of hdf5_funcs.h:19-27) */
void CreateOutputFilesWriteICs(const long int* N, double dt) {
    (void)N; (void)dt;
    record_row(sys_vars->t0, 0);
}
void WriteDataToFile(double t, double dt, long int iters) {
    (void)dt;
    record_row(t, (int)iters);
}
void FinalWriteAndCloseOutputFile(const long int* N, int iters, int save_data_indx) {
    (void)iters; (void)save_data_indx;
    if (g_final)
        memcpy(g_final, run_data->u_hat, sizeof(fftw_complex) * 3 * (size_t)(N[0] * N[1] * (N[2] / 2 + 1)));
}

/* main.c:41-67 up to the solver call: globals, rank, GetCMLArgs */
static int parse(int argc, char** argv) {
    memset(&g_run, 0, sizeof(g_run));
    memset(&g_sys, 0, sizeof(g_sys));
    memset(&g_file, 0, sizeof(g_file));
    run_data = &g_run;
    sys_vars = &g_sys;
    file_info = &g_file;
    MPI_Comm_size(MPI_COMM_WORLD, &(sys_vars->num_procs));
    MPI_Comm_rank(MPI_COMM_WORLD, &(sys_vars->rank));
    optind = 0;   /* glibc: a full re-initialisation of getopt for each call */
    GetCMLArgs(argc, argv);
    for (int d = 0; d < 3; ++d) g_n[d] = sys_vars->N[d];
    return 0;
}

void ref_destroy(void) {
    if (!g_ready) return;
    FreeMemory(&g_rk);
    g_ready = 0;
}

/* SpectralSolve's set-up (solver.c:52-105) without the time loop; argv are
   the reference binary's flags (utils.c:74). */
int ref_create(int argc, char** argv) {
    ref_destroy();
    parse(argc, argv);
    const long NB[3] = {g_n[0], g_n[1], g_n[2] / 2 + 1};
    memset(&g_rk, 0, sizeof(g_rk));
    AllocateMemory(NB, &g_rk);
    InitializeFFTWPlans(g_n, NB);
    InitializeSpaceVariables(run_data->x, run_data->k, g_n);
    double t0, t, dt, T;
    long trans;
    InitializeIntegrationVariables(&t0, &t, &dt, &T, &trans);
    InitializeSystemMeasurables(&g_rk);
    g_ready = 1;
    fflush(stdout);   /* the reference prints; flush while the caller's capture is active */
    return 0;
}

static size_t nmodes(void) { return (size_t)(g_n[0] * g_n[1] * (g_n[2] / 2 + 1)); }

void ref_initial_conditions(void) { InitialConditions(run_data->u_hat, run_data->u, g_n); }
void ref_set_state(const double* u_hat) { memcpy(run_data->u_hat, u_hat, sizeof(fftw_complex) * 3 * nmodes()); }
void ref_get_state(double* u_hat) { memcpy(u_hat, run_data->u_hat, sizeof(fftw_complex) * 3 * nmodes()); }

/* NonlinearRHSBatch (solver.c:620-731) on a copy of `in`; `vel`, `vort`
   (optional) receive the real-space arrays it formed, in its transposed
   layout. */
void ref_rhs(const double* in, double* out, double* vel, double* vort) {
    memcpy(g_rk.RK_tmp, in, sizeof(fftw_complex) * 3 * nmodes());
    NonlinearRHSBatch(g_rk.RK_tmp, g_rk.RK1, g_rk.curl, g_rk.vel, g_rk.vort);
    memcpy(out, g_rk.RK1, sizeof(fftw_complex) * 3 * nmodes());
    const size_t nr = (size_t)(g_n[0] * g_n[1] * (g_n[2] + 2)) * 3;
    if (vel) memcpy(vel, g_rk.vel, sizeof(double) * nr);
    if (vort) memcpy(vort, g_rk.vort, sizeof(double) * nr);
}

/* RK4Step (solver.c:505-608), nsteps times on run_data->u_hat */
void ref_rk4_step(double dt, int nsteps) {
    for (int s = 0; s < nsteps; ++s) RK4Step(dt, g_n, sys_vars->local_Nx, &g_rk);
}

/* ApplyDealiasing (solver.c:1709-1756) in place on a caller array */
void ref_dealias(double* arr, int array_dim) { ApplyDealiasing((fftw_complex*)arr, array_dim, g_n); }

/* ComputeSystemMeasurables (solver.c:1142-1276) of run_data->u_hat into slot
   0: tot = [E, Omega, P, H, eps]; Ek, Ok have ref_n_spect() entries */
void ref_measurables(double* tot, double* Ek, double* Ok) {
    ComputeSystemMeasurables(0);
    tot[0] = run_data->tot_energy[0];
    tot[1] = run_data->tot_enstr[0];
    tot[2] = run_data->tot_palin[0];
    tot[3] = run_data->tot_heli[0];
    tot[4] = run_data->enrg_diss[0];
    if (Ek) memcpy(Ek, run_data->enrg_spect, sizeof(double) * (size_t)sys_vars->n_spect);
    if (Ok) memcpy(Ok, run_data->enst_spect, sizeof(double) * (size_t)sys_vars->n_spect);
}

/* InitializeSpaceVariables' wavenumbers and collocation points */
void ref_space(int* kx, int* ky, int* kz, double* x, double* y, double* z) {
    for (long i = 0; i < g_n[0]; ++i) { kx[i] = run_data->k[0][i]; x[i] = run_data->x[0][i]; }
    for (long i = 0; i < g_n[1]; ++i) { ky[i] = run_data->k[1][i]; y[i] = run_data->x[1][i]; }
    for (long i = 0; i < g_n[2] / 2 + 1; ++i) kz[i] = run_data->k[2][i];
    for (long i = 0; i < g_n[2]; ++i) z[i] = run_data->x[2][i];
}

/* The reference program's run: main.c's set-up and SpectralSolve
   (solver.c:50-208) end to end. `series` receives up to max_rows saved rows
   (layout of record_row), `u_hat_final` the state handed to the final
   writer. Returns the number of rows recorded. */
int ref_spectral_solve(int argc, char** argv, double* series, int max_rows, double* u_hat_final) {
    ref_destroy();
    parse(argc, argv);
    g_series = series;
    g_series_max = max_rows;
    g_series_rows = 0;
    g_final = u_hat_final;
    SpectralSolve();
    fflush(stdout);
    g_series = NULL;
    g_final = NULL;
    return g_series_rows;
}
