/*
 * ns3d_compat.h — the reference solver's hot-path function names and
 * signatures (Solver/src/solver.h:24-55), implemented on top of ns3d.h.
 *
 * The reference's functions work on global structs (data_types.h:147-235,
 * defined in main.c:26-28) whose types pull in FFTW-MPI and HDF5 headers. This
 * header declares reduced structs with the hot-path fields under the same
 * global names, so a reference-shaped driver (SpectralSolve's loop,
 * solver.c:50-208) compiles and links against libns3d.so unchanged apart
 * from the include. Arrays are host arrays in the reference layouts:
 *   Fourier: ns3d_fftw_complex [N][N][N/2+1][3]   (fftw_complex = double[2])
 *   Real:    double             [N][N][N+2][3]
 * As in the reference, a failure prints to stderr and calls exit(1).
 */
#ifndef NS3D_COMPAT_H
#define NS3D_COMPAT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NS3D_SYS_DIM 3

typedef double ns3d_fftw_complex[2];

/* hot-path fields of system_vars_struct (data_types.h:147-185) */
typedef struct system_vars_struct {
    char u0[64];           /* initial condition name                          */
    char forcing[64];      /* "NONE", "ZERO" (no-op, as the reference), "SHELL"  */
    long int N[NS3D_SYS_DIM];
    ptrdiff_t local_Nx;    /* = N[0]: one process holds the whole grid        */
    ptrdiff_t local_Nx_start;
    int num_procs, rank;
    long int num_t_steps, num_print_steps;
    double t0, T, t, dt;
    double dx, dy, dz;
    int n_spect;
    int force_k;
    double CFL_CONST;
    double NU;
    int SAVE_EVERY;
    /* switches that the reference sets at compile time (Makefile:43-53); a
       zero-filled struct gives the reference's default build ("solver":
       -D__NAVIER -D__HYPER with data_types.h's __RK4) */
    int visc_pow;          /* 0: the default build's hyperviscosity nu k^4
                              (HYPER_VISC, VIS_POW 2.0, data_types.h:68-71);
                              1: nu k^2 (the "solver_test" build); 2: nu k^4 */
    int integrator;        /* 0: RK4 + Crank-Nicolson (RK4Step, solver.c:505-608),
                              1: integrating-factor RK4 (no reference counterpart),
                              2: RK5 (__RK5), 3: Dormand-Prince (__DPRK5)      */
    int precision;         /* 0: FP64, 1: FP32 bulk                          */
    int adaptive_step;     /* 1: CFL step (__ADAPTIVE_STEP)                   */
} system_vars_struct;

/* hot-path fields of runtime_data_struct (data_types.h:188-222) */
typedef struct runtime_data_struct {
    double* x[NS3D_SYS_DIM];
    int* k[NS3D_SYS_DIM];
    ns3d_fftw_complex* u_hat;
    ns3d_fftw_complex* w_hat;
    double* u;
    double* w;
    double* tot_energy;
    double* tot_enstr;
    double* tot_palin;
    double* tot_heli;
    double* enrg_diss;
    double* time;
    double* enrg_spect;
    double* enst_spect;
} runtime_data_struct;

/* RK_data_struct (data_types.h:225-240): the GPU keeps its own stage arrays */
typedef struct RK_data_struct {
    int unused;
} RK_data_struct;

extern system_vars_struct* sys_vars;
extern runtime_data_struct* run_data;

/* solver.c:1764-1826 */
void InitializeSpaceVariables(double** x, int** k, const long int* N);
/* solver.c:1537-1648 (TAYLOR_GREEN, SHAPIRO, TESTING, RANDOM/other, SPECTRUM) */
void InitialConditions(ns3d_fftw_complex* u_hat, double* u, const long int* N);
/* solver.c:505-608: one step of run_data->u_hat in place. The device state
   holds only the modes inside the 2/3 sphere: modes outside it in the host
   array are dropped on input and come back as zeros (the reference's RK4Step
   on an array that was never dealiased keeps them and decays them by the
   Crank-Nicolson factor; after any NonlinearRHSBatch the two agree). */
void RK4Step(const double dt, const long int* N, const ptrdiff_t local_Nx, RK_data_struct* RK_data);
/* solver.c:217-421 (integrator 2 or 3; for 3 one accepted adaptive step) */
void RK5DPStep(const double dt, const long int* N, const int iters, const ptrdiff_t local_Nx, RK_data_struct* RK_data);
/* solver.c:620-731 (curl, u, vort are the reference's scratch; unused here) */
void NonlinearRHSBatch(ns3d_fftw_complex* u_hat, ns3d_fftw_complex* dw_hat_dt, double* curl, double* u,
                       double* vort);
/* solver.c:1709-1756 */
void ApplyDealiasing(ns3d_fftw_complex* array, int array_dim, const long int* N);
/* solver.c:1142-1276: fills run_data->tot_*[iter] and the spectra of run_data->u_hat */
void ComputeSystemMeasurables(int iter);
/* releases the device context behind these functions (FreeMemory, solver.c:2078) */
void ns3d_compat_free(void);

#ifdef __cplusplus
}
#endif
#endif
