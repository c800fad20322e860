/*
 * ns3d_compat.c — the reference's hot-path function names over host arrays
 * (include/ns3d_compat.h), each a thin call into the GPU C ABI (ns3d.h).
 * A device context is created on first use from the fields of *sys_vars and
 * recreated when they change. Errors print and exit(1), as the reference's
 * functions do (e.g. solver.c:1394-1397).
 */
#include "../../include/ns3d_compat.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/ns3d.h"

system_vars_struct* sys_vars;
runtime_data_struct* run_data;

static ns3d_ctx* g_ctx;
static ns3d_params g_params;

static void die(const char* what, ns3d_status s) {
    fprintf(stderr, "\n[ERROR] --- %s failed: %s (%s)\n-->> Exiting!!!\n", what, ns3d_status_string(s),
            g_ctx ? ns3d_last_error(g_ctx) : "");
    exit(1);
}

static ns3d_params params_from_sys(double dt) {
    ns3d_params p;
    memset(&p, 0, sizeof(p));
    p.N = (int)sys_vars->N[0];
    p.nu = sys_vars->NU;
    p.dt = dt > 0 ? dt : sys_vars->dt;
    p.t0 = sys_vars->t0;
    /* zero-filled switches select the reference's default build: nu k^4 and
       RK4 + Crank-Nicolson (Makefile:44, data_types.h:57-71) */
    p.visc_pow = sys_vars->visc_pow == 1 ? 1 : 2;
    p.integrator = sys_vars->integrator == 1   ? NS3D_IFRK4
                   : sys_vars->integrator == 2 ? NS3D_RK5CN
                   : sys_vars->integrator == 3 ? NS3D_DP5CN
                                               : NS3D_RK4CN;
    p.precision = sys_vars->precision == 1 ? NS3D_FP32 : NS3D_FP64;
    p.cfl = (sys_vars->adaptive_step && p.integrator != NS3D_DP5CN) ? sys_vars->CFL_CONST : 0.0;
    p.forcing = strcmp(sys_vars->forcing, "SHELL") == 0 ? NS3D_FORCE_SHELL : NS3D_FORCE_NONE;
    p.force_k = sys_vars->force_k > 0 ? sys_vars->force_k : 2;
    p.device = 0;
    p.stream = NULL;
    return p;
}

static ns3d_ctx* ctx_for(double dt) {
    if (!sys_vars) {
        fprintf(stderr, "\n[ERROR] --- sys_vars is not set\n-->> Exiting!!!\n");
        exit(1);
    }
    if (sys_vars->N[0] != sys_vars->N[1] || sys_vars->N[0] != sys_vars->N[2]) {
        fprintf(stderr, "\n[ERROR] --- only cubic grids are supported (N = [%ld,%ld,%ld])\n-->> Exiting!!!\n",
                sys_vars->N[0], sys_vars->N[1], sys_vars->N[2]);
        exit(1);
    }
    ns3d_params want = params_from_sys(dt);
    if (g_ctx) {
        /* the step size is time state, not configuration: an adaptive or
           Dormand-Prince run changes it every step on the same engine */
        ns3d_params same = want;
        same.dt = g_params.dt;
        if (memcmp(&same, &g_params, sizeof(same)) == 0) return g_ctx;
    }
    if (g_ctx) ns3d_destroy(g_ctx);
    g_ctx = NULL;
    ns3d_status s = ns3d_create(&want, &g_ctx);
    if (s != NS3D_OK) die("ns3d_create", s);
    g_params = want;
    return g_ctx;
}

void ns3d_compat_free(void) {
    if (g_ctx) ns3d_destroy(g_ctx);
    g_ctx = NULL;
}

void InitializeSpaceVariables(double** x, int** k, const long int* N) {
    /* solver.c:1764-1826 with local_Nx = N[0], local_Nx_start = 0 */
    const long Nx = N[0], Ny = N[1], Nz = N[2];
    if (sys_vars) {
        sys_vars->dx = 2.0 * M_PI / (double)Nx;
        sys_vars->dy = 2.0 * M_PI / (double)Ny;
        sys_vars->dz = 2.0 * M_PI / (double)Nz;
    }
    for (long i = 0; i < Nx; ++i) {
        x[0][i] = (double)i * 2.0 * M_PI / (double)Nx;
        k[0][i] = (int)(i <= Nx / 2 ? i : i - Nx);
    }
    for (long i = 0; i < Ny; ++i) {
        x[1][i] = (double)i * 2.0 * M_PI / (double)Ny;
        k[1][i] = (int)(i < Ny / 2 + 1 ? i : -Ny + i);
    }
    for (long i = 0; i < Nz; ++i) {
        x[2][i] = (double)i * 2.0 * M_PI / (double)Nz;
        if (i < Nz / 2 + 1) k[2][i] = (int)i;
    }
}

void InitialConditions(ns3d_fftw_complex* u_hat, double* u, const long int* N) {
    (void)N;
    ns3d_ctx* c = ctx_for(0);
    ns3d_status s = ns3d_initial_condition(c, sys_vars->u0, 0, 4.0, 1.0);
    if (s != NS3D_OK) die("InitialConditions", s);
    s = ns3d_get_state_host(c, (double*)u_hat);
    if (s != NS3D_OK) die("InitialConditions", s);
    if (u) {
        s = ns3d_real_space_host(c, u, NULL);
        if (s != NS3D_OK) die("InitialConditions", s);
    }
}

void RK4Step(const double dt, const long int* N, const ptrdiff_t local_Nx, RK_data_struct* RK_data) {
    (void)N;
    (void)local_Nx;
    (void)RK_data;
    ns3d_ctx* c = ctx_for(dt);
    double t = 0, cur_dt = 0;
    long it = 0;
    ns3d_status s = ns3d_get_time(c, &t, &cur_dt, &it);
    if (s == NS3D_OK && cur_dt != dt && !sys_vars->adaptive_step) s = ns3d_set_time(c, t, dt, it);
    if (s == NS3D_OK) s = ns3d_step_host(c, (const double*)run_data->u_hat, (double*)run_data->u_hat);
    if (s != NS3D_OK) die("RK4Step", s);
}

/* RK5DPStep (solver.c:217-421): one RK5CN step (integrator 2), or one accepted
   Dormand-Prince step (integrator 3): the step-size control of SpectralSolve
   (solver.c:134-154) runs inside, and sys_vars->dt and sys_vars->t receive the
   next step size and the new time. */
void RK5DPStep(const double dt, const long int* N, const int iters, const ptrdiff_t local_Nx, RK_data_struct* RK_data) {
    (void)N;
    (void)iters;
    (void)local_Nx;
    (void)RK_data;
    if (!sys_vars || (sys_vars->integrator != 2 && sys_vars->integrator != 3)) {
        fprintf(stderr, "\n[ERROR] --- RK5DPStep needs sys_vars->integrator 2 (RK5) or 3 (DPRK5)\n-->> Exiting!!!\n");
        exit(1);
    }
    ns3d_ctx* c = ctx_for(dt);
    double t = 0, cur_dt = 0;
    long it = 0;
    ns3d_status s = ns3d_get_time(c, &t, &cur_dt, &it);
    if (s == NS3D_OK && sys_vars->integrator == 2 && cur_dt != dt && !sys_vars->adaptive_step)
        s = ns3d_set_time(c, t, dt, it);
    if (s == NS3D_OK) s = ns3d_step_host(c, (const double*)run_data->u_hat, (double*)run_data->u_hat);
    if (s == NS3D_OK && sys_vars->integrator == 3) {
        s = ns3d_get_time(c, &t, &cur_dt, &it);
        sys_vars->dt = cur_dt;
        sys_vars->t = t;
    }
    if (s != NS3D_OK) die("RK5DPStep", s);
}

void NonlinearRHSBatch(ns3d_fftw_complex* u_hat, ns3d_fftw_complex* dw_hat_dt, double* curl, double* u,
                       double* vort) {
    (void)curl;
    (void)u;
    (void)vort;
    ns3d_status s = ns3d_rhs_host(ctx_for(0), (const double*)u_hat, (double*)dw_hat_dt);
    if (s != NS3D_OK) die("NonlinearRHSBatch", s);
}

void ApplyDealiasing(ns3d_fftw_complex* array, int array_dim, const long int* N) {
    ns3d_status s = ns3d_dealias_host((int)N[0], (double*)array, array_dim);
    if (s != NS3D_OK) die("ApplyDealiasing", s);
}

void ComputeSystemMeasurables(int iter) {
    ns3d_ctx* c = ctx_for(0);
    ns3d_measures m;
    double target = 0.0;
    /* loading the array resets the forcing target; keep the running one */
    ns3d_status s = ns3d_get_forcing_target(c, &target);
    if (s == NS3D_OK) s = ns3d_set_state_host(c, (const double*)run_data->u_hat);
    if (s == NS3D_OK) s = ns3d_set_forcing_target(c, target);
    if (s == NS3D_OK) s = ns3d_measurables(c, &m, run_data->enrg_spect, run_data->enst_spect);
    if (s != NS3D_OK) die("ComputeSystemMeasurables", s);
    if (run_data->tot_energy) run_data->tot_energy[iter] = m.energy;
    if (run_data->tot_enstr) run_data->tot_enstr[iter] = m.enstrophy;
    if (run_data->tot_palin) run_data->tot_palin[iter] = m.palinstrophy;
    if (run_data->tot_heli) run_data->tot_heli[iter] = m.helicity;
    if (run_data->enrg_diss) run_data->enrg_diss[iter] = m.dissipation;
}
