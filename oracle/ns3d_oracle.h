/*
 * ns3d_oracle.h — ORACLE: test infrastructure only, never product code.
 *
 * CPU FP64 restatement of the time-stepping hot path of the reference
 * pseudospectral 3D Navier–Stokes solver (Solver/src/solver.c). Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it,
 * and only as the checker or the timed CPU baseline. The GPU library never
 * links or calls it.
 *
 * Array layouts follow the reference exactly:
 *   Fourier: complex (re,im doubles) [N][N][N/2+1][3]   (solver.c:644-647)
 *   Real:    double                  [N][N][N+2][3]     (solver.c:667)
 */
#ifndef NS3D_ORACLE_H
#define NS3D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

enum { ORC_IFRK4 = 0, ORC_RK4CN = 1, ORC_RK5CN = 2, ORC_DP5CN = 3 };
enum { ORC_FORCE_NONE = 0, ORC_FORCE_SHELL = 1 };

typedef struct {
    int    N;                  /* grid points per axis (cubic box, even)            */
    double nu;                 /* viscosity NU                                      */
    double dt;                 /* time step (initial step when cfl > 0)             */
    double t0;                 /* start time                                        */
    int    visc_pow;           /* 1: nu k^2, 2: nu k^4 (reference HYPER_VISC)       */
    int    integrator;         /* ORC_IFRK4, ORC_RK4CN, ORC_RK5CN or ORC_DP5CN       */
    double cfl;                /* > 0: dt = cfl*dx/max(|u|+|v|+|w|) every step      */
    int    forcing;            /* ORC_FORCE_NONE / ORC_FORCE_SHELL                  */
    int    force_k;            /* shells round(|k|) <= force_k held at fixed energy */
    int    bugcompat_dealias;  /* reproduce defect D2 (solver.c:1741)               */
    int    bugcompat_measures; /* reproduce defect D4 (solver.c:1232-1235)          */
    int    nthreads;           /* OpenMP threads (<= 0: runtime default)            */
    int    bugcompat_rk5;      /* reproduce defect D19: a32 = 1/2 (solver.c:36)      */
    double dp_atol, dp_rtol;   /* DP5CN error tolerances (<= 0: 1e-7, data_types.h:123-124) */
} orc_params;

orc_ctx* orc_create(const orc_params* p);
void     orc_destroy(orc_ctx* c);
int      orc_n_spect(int N);
int      orc_threads(void);

void orc_set_state(orc_ctx* c, const double* u_hat);
void orc_get_state(const orc_ctx* c, double* u_hat);
void orc_set_time(orc_ctx* c, double t, double dt, long iters);
void orc_get_time(const orc_ctx* c, double* t, double* dt, long* iters);
double orc_forcing_target(const orc_ctx* c);
void   orc_set_forcing_target(orc_ctx* c, double e);

/* transforms, batched over the 3 interleaved components, unnormalised like FFTW */
void orc_fft_r2c(orc_ctx* c, const double* real, double* u_hat);
void orc_fft_c2r(orc_ctx* c, const double* u_hat, double* real);
void orc_fft1d(int n, const double* in, double* out, int inverse);
/* planned 1D complex transform of length n (in != out, contiguous), unnormalised */
typedef struct orc_fft_plan_s orc_fft_plan_t;
orc_fft_plan_t* orc_fft_plan_create(int n);
void orc_fft_plan_exec(const orc_fft_plan_t* q, const double* in, double* out, int inverse);
void orc_fft_plan_destroy(orc_fft_plan_t* q);

void orc_dealias(orc_ctx* c, double* arr, int array_dim);
void orc_rhs(orc_ctx* c, const double* u_hat, double* rhs);
/* returns 0, or 1 when a DP5CN step was rejected DP_MAX_TRY = 50 times in a row */
int  orc_step(orc_ctx* c, int nsteps);
/* One RK4 stage (IF-RK4 or RK4CN): the stage's nonlinear evaluation and its
   stage update; every fourth call also the final update, forcing and time.
   Returns the next stage (0 after a completed step), -1 for other integrators. */
int  orc_stage(orc_ctx* c);
/* DP5CN: error norm of the last attempt, rejected attempts so far */
void orc_dp_stats(const orc_ctx* c, double* last_err, long* rejects);
void orc_measurables(orc_ctx* c, double* totals5, double* Ek, double* Ok);
int  orc_ic(orc_ctx* c, const char* name, uint64_t seed, double k0, double energy);
void orc_real_space(orc_ctx* c, double* u, double* w);
double orc_max_speed_sum(orc_ctx* c);
/* longitudinal velocity-increment statistics (PostProcessing/src/stats.c):
   stats[r][6] = min, max, mean, sd, skew, excess kurtosis; ranges[r][nbins+1];
   counts[r][nbins] */
void orc_increment_stats(orc_ctx* c, const int* incr, int nr, int nbins, double* stats, double* ranges,
                         double* counts);

#ifdef __cplusplus
}
#endif
#endif
