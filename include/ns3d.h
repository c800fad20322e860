/*
 * ns3d.h — C ABI of the GB300 (sm_103a) time-stepping hot path of a 3D periodic
 * pseudospectral Navier–Stokes solver (drop-in for the reference's
 * Solver/src/solver.c hot path).
 *
 * Everything runs on one GPU with hand-written CUDA kernels; there is no CPU
 * fallback. Plain C types only: pointers, sizes, status codes.
 *
 * Host array layouts are the reference's:
 *   Fourier: complex double (re, im) [N][N][N/2+1][3]  (solver.c:644-647)
 *   Real:    double                  [N][N][N+2][3]    (solver.c:667)
 * The device keeps its own layout (one array per component, only the modes
 * inside the 2/3-rule sphere) and converts at these calls.
 *
 * Errors: every call returns an ns3d_status instead of the reference's
 * fprintf + exit(1) (e.g. solver.c:1394-1397, 2047-2050). A context is bound to
 * one CUDA stream and is not thread-safe; separate contexts are independent.
 */
#ifndef NS3D_H
#define NS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    NS3D_OK = 0,
    NS3D_ERR_INVALID = 1,      /* bad argument (size, pointer, name)            */
    NS3D_ERR_UNSUPPORTED = 2,  /* grid size without a compiled FFT plan         */
    NS3D_ERR_CUDA = 3,         /* CUDA runtime error                            */
    NS3D_ERR_NOMEM = 4,        /* device allocation failed                      */
    NS3D_ERR_NUMERIC = 5,      /* health check: NaN/Inf or non-positive dt      */
    NS3D_ERR_TIMEOUT = 6       /* a bounded device wait gave up                 */
} ns3d_status;

typedef enum { NS3D_FP64 = 0, NS3D_FP32 = 1 } ns3d_precision;
/* IFRK4: integrating-factor RK4 (Lawson). RK4CN: the reference's RK4Step
 * (solver.c:505-608). RK5CN: its RK5DPStep built with __RK5 (solver.c:217-421),
 * fixed step. DP5CN: its adaptive Dormand-Prince loop (__DPRK5, solver.c:
 * 134-154), single runs only, cfl must be 0. Both RK5 variants use the
 * published Dormand-Prince table (a32 = 9/40; the reference has 1/2). */
typedef enum { NS3D_IFRK4 = 0, NS3D_RK4CN = 1, NS3D_RK5CN = 2, NS3D_DP5CN = 3 } ns3d_integrator;
typedef enum { NS3D_FORCE_NONE = 0, NS3D_FORCE_SHELL = 1 } ns3d_forcing;

/* Parameters: the hot-path fields of system_vars_struct (data_types.h:147-185)
 * plus the switches that replace the reference's compile-time macros. */
typedef struct {
    int    N;           /* grid points per axis (cubic box, sys_vars->N)               */
    double nu;          /* viscosity (sys_vars->NU, utils.c:150-156)                    */
    double dt;          /* time step (sys_vars->dt); initial step when cfl > 0          */
    double t0;          /* start time (sys_vars->t0)                                    */
    int    visc_pow;    /* 1: nu k^2; 2: nu k^4 (HYPER_VISC, VIS_POW, data_types.h:68-71) */
    int    integrator;  /* ns3d_integrator; RK4CN is the reference's RK4Step           */
    int    precision;   /* ns3d_precision: FP64, or FP32 bulk with FP64 integrating
                           factors, time accumulator and reductions                   */
    double cfl;         /* > 0: dt = cfl * dx / max(|u|+|v|+|w|) every step (CFL_CONST)  */
    int    forcing;     /* ns3d_forcing: SHELL holds the energy of shells
                           1 <= round(|k|) <= force_k at its initial value            */
    int    force_k;     /* forcing shell radius (sys_vars->force_k)                     */
    int    device;      /* CUDA device ordinal                                          */
    void*  stream;      /* cudaStream_t to run on, or NULL for a private stream         */
} ns3d_params;

/* Totals of ComputeSystemMeasurables (solver.c:1142-1276), with the reference's
 * normalisation 8 pi^3 * 0.5 / N^6 and the kz-plane multiplicities. */
typedef struct {
    double energy;        /* tot_energy                                  */
    double enstrophy;     /* tot_enstr                                   */
    double palinstrophy;  /* tot_palin                                   */
    double helicity;      /* tot_heli as Re sum u.conj(w) (see D12)      */
    double dissipation;   /* enrg_diss                                   */
} ns3d_measures;

typedef struct ns3d_ctx ns3d_ctx;

const char* ns3d_status_string(ns3d_status s);
/* 1 when a compiled FFT plan exists for grid size N, else 0: N = 8, 16, 24,
 * 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024 (cubic grids; the
 * reference's GetCMLArgs accepts any even N > 2, utils.c:88-104, and other
 * sizes return NS3D_ERR_UNSUPPORTED from ns3d_create). */
int ns3d_supported_size(int N);
/* Length of the spectrum arrays, sys_vars->n_spect (solver.c:1384). */
int ns3d_n_spect(int N);

/* AllocateMemory + InitializeFFTWPlans + InitializeSpaceVariables
 * (solver.c:1832-2073, 1764-1826): device state, twiddle tables, step graph. */
ns3d_status ns3d_create(const ns3d_params* params, ns3d_ctx** out);
/* FreeMemory (solver.c:2078-2157). */
ns3d_status ns3d_destroy(ns3d_ctx* ctx);
/* Message of the last failure on this context ("" when none). */
const char* ns3d_last_error(const ns3d_ctx* ctx);

/* InitialConditions (solver.c:1537-1648). Names: "TAYLOR_GREEN", "SHAPIRO",
 * "TESTING" (zero field), "RANDOM" (the reference's srand(123456789) modes),
 * "SPECTRUM" (new: seeded random-phase solenoidal field with
 * E(k) ~ k^4 exp(-2 (k/k0)^2), scaled so that 0.5 <|u|^2> = energy).
 * Other names fall back to RANDOM like the reference. Resets t, dt, iters. */
ns3d_status ns3d_initial_condition(ns3d_ctx* ctx, const char* name, uint64_t seed,
                                   double k0, double energy);

/* Copy the state u_hat in or out (reference Fourier layout, FP64 host array).
 * Modes outside the 2/3-rule sphere are dropped on the way in, as
 * ApplyDealiasing does (solver.c:1630). */
ns3d_status ns3d_set_state_host(ns3d_ctx* ctx, const double* u_hat);
ns3d_status ns3d_get_state_host(ns3d_ctx* ctx, double* u_hat);

/* RK4Step (solver.c:505-608) or IF-RK4, nsteps times on the device state,
 * including forcing and the CFL step choice when enabled. */
ns3d_status ns3d_step(ns3d_ctx* ctx, int nsteps);
/* One step through host buffers: u_hat_in -> step -> u_hat_out (either may be
 * NULL to keep the device state). This is RK4Step's host-array contract. */
ns3d_status ns3d_step_host(ns3d_ctx* ctx, const double* u_hat_in, double* u_hat_out);

/* NonlinearRHSBatch (solver.c:620-731): out = P[FFT(u x w)] / N^6, dealiased,
 * for the dealiased part of in. Host arrays in the reference Fourier layout. */
ns3d_status ns3d_rhs_host(ns3d_ctx* ctx, const double* u_hat_in, double* rhs_out);

/* ApplyDealiasing (solver.c:1709-1756) of a host array with array_dim
 * interleaved components (2/3 rule, defect D2 fixed). */
ns3d_status ns3d_dealias_host(int N, double* array, int array_dim);

/* ComputeSystemMeasurables (solver.c:1142-1276), defect D4 fixed. Ek and Ok
 * (n_spect doubles each) may be NULL. Deterministic FP64 reductions. */
ns3d_status ns3d_measurables(ns3d_ctx* ctx, ns3d_measures* out, double* Ek, double* Ok);

/* Real-space velocity and vorticity normalised by 1/N^3 (hdf5_funcs.c:586-600,
 * 662-676), reference real layout; either pointer may be NULL. */
ns3d_status ns3d_real_space_host(ns3d_ctx* ctx, double* u, double* w);

/* ComputeSystemMeasurables for callers that cannot allocate device memory
 * (no counterpart in the reference). Input: a device array in the reference
 * Fourier layout, complex double [N][N][N/2+1][3], 16-byte aligned; every mode
 * counts, as in the reference, except that shells with round(|k|) >= n_spect
 * (corner modes that the reference writes past its spectrum arrays for) are
 * left out of d_Ek / d_Ok while staying in the totals. Outputs (device):
 * d_totals[5] in the order of ns3d_measures, and n_spect doubles each in
 * d_Ek / d_Ok (either may be NULL). Runs asynchronously on `stream` (NULL =
 * default stream). Its partial sums live in a 2 MiB static device array
 * shared by every call, so N <= 512 (larger N: NS3D_ERR_INVALID) and calls
 * that overlap on the GPU race. Outside stream capture each call resolves that
 * array's address in the current context; a call under capture reuses the one
 * resolved earlier in the same context, so make one call per context (again
 * after a cudaDeviceReset) before capturing. Allocates nothing. */
ns3d_status ns3d_measurables_noalloc(int N, double nu, int visc_pow, const double* d_u_hat,
                                     double* d_totals, double* d_Ek, double* d_Ok, void* stream);

/* Time bookkeeping (solver.c:1314-1363): current t, dt and completed steps. */
ns3d_status ns3d_get_time(ns3d_ctx* ctx, double* t, double* dt, long* iters);
ns3d_status ns3d_set_time(ns3d_ctx* ctx, double t, double dt, long iters);
/* Forcing target energy (set by initial conditions / set_state). */
ns3d_status ns3d_get_forcing_target(ns3d_ctx* ctx, double* e);
ns3d_status ns3d_set_forcing_target(ns3d_ctx* ctx, double e);

/* DP5CN step control: error tolerances (default 1e-7 / 1e-7, DP_ABS_TOL and
 * DP_REL_TOL of data_types.h:123-124), and the error norm of the last attempt
 * with the number of rejected attempts so far. With DP5CN, ns3d_step(ctx, n)
 * returns after n accepted steps; n steps rejected DP_MAX_TRY = 50 times in a
 * row end it with NS3D_ERR_NUMERIC. */
ns3d_status ns3d_set_dp_tolerances(ns3d_ctx* ctx, double atol, double rtol);

/* Failure detection (no counterpart in the reference, whose limits
 * MIN_STEP_SIZE, MAX_ITERS and MAX_VORT_LIM at data_types.h:130-136 are
 * defined but never checked). Every wait of the z pass on an asynchronous
 * copy is bounded: after `cycles` SM clock cycles (<= 0: the default, 4e9,
 * about 2 s) the pass records a timeout, lets its copies in flight land and
 * returns, and ns3d_step reports NS3D_ERR_TIMEOUT. A short budget makes that
 * path fire on purpose (tests); ns3d_set_time clears the recorded status.
 * A NaN or Inf in the field is reported by ns3d_step as NS3D_ERR_NUMERIC. */
ns3d_status ns3d_set_wait_budget(ns3d_ctx* ctx, long long cycles);
ns3d_status ns3d_dp_stats(ns3d_ctx* ctx, double* last_err, long* rejects);

/* Longitudinal velocity-increment statistics of the current state, the
 * post-processing of PostProcessing/src/stats.c:22-254 on the GPU. For each
 * increment r (grid points) the samples u_a(x + r e_a) - u_a(x) for a = x, y, z
 * with x_a + r < N (not periodic) are pooled; stats[r][6] = min, max, mean,
 * sample sd, skewness m3/sd^3 and excess kurtosis m4/sd^4 - 3 (GSL rstat);
 * ranges[r][n_bins + 1] = n_bins uniform bins over [min - 0.05, max + 0.05]
 * (GSL's uniform edges); counts[r][n_bins] with edge[b] <= d < edge[b + 1].
 * increments NULL: {1, 2, 4, 8, 16, 32, 64, 128, N/2} (n_incr = 9, the
 * reference's NUM_INCR); ranges / counts may be NULL. n_bins <= 12288. */
ns3d_status ns3d_increment_stats(ns3d_ctx* ctx, const int* increments, int n_incr, int n_bins, double* stats,
                                 double* ranges, double* counts);

/* Largest |u|+|v|+|w| over the grid for the current state (CFL numerator). */
ns3d_status ns3d_max_speed_sum(ns3d_ctx* ctx, double* umax);

/* ------------------------------------------------------------------------
 * Ensembles: many independent runs of (possibly) different grid sizes,
 * viscosities, time steps and initial conditions stepped together. Members
 * with the same N, precision, integrator, visc_pow, forcing and CFL switch
 * share kernel launches; all members advance by one step per CUDA-graph
 * launch. Member operations mirror the single-run calls above.
 * ------------------------------------------------------------------------ */
typedef struct ns3d_ensemble ns3d_ensemble;
ns3d_status ns3d_ensemble_create(const ns3d_params* members, int count, ns3d_ensemble** out);
ns3d_status ns3d_ensemble_destroy(ns3d_ensemble* e);
const char* ns3d_ensemble_last_error(const ns3d_ensemble* e);
ns3d_status ns3d_ensemble_initial_condition(ns3d_ensemble* e, int member, const char* name, uint64_t seed,
                                            double k0, double energy);
ns3d_status ns3d_ensemble_set_state_host(ns3d_ensemble* e, int member, const double* u_hat);
ns3d_status ns3d_ensemble_get_state_host(ns3d_ensemble* e, int member, double* u_hat);
ns3d_status ns3d_ensemble_measurables(ns3d_ensemble* e, int member, ns3d_measures* out, double* Ek, double* Ok);
ns3d_status ns3d_ensemble_get_time(ns3d_ensemble* e, int member, double* t, double* dt, long* iters);
/* every member advances nsteps steps (one graph launch per step) */
ns3d_status ns3d_ensemble_step(ns3d_ensemble* e, int nsteps);
/* The same n steps as ONE graph launch: the captured step sits in a
 * device-side loop (a conditional WHILE graph node whose body ends with a
 * one-thread kernel that counts the steps down), so the host launches once
 * per run instead of once per step. Results equal ns3d_ensemble_step's. */
ns3d_status ns3d_ensemble_run(ns3d_ensemble* e, int nsteps);
/* number of launch groups and kernels launched per ensemble step */
ns3d_status ns3d_ensemble_info(ns3d_ensemble* e, int* groups, int* kernels_per_step);
/* device time of the last ns3d_ensemble_step / ns3d_ensemble_run call, milliseconds */
ns3d_status ns3d_ensemble_last_step_ms(ns3d_ensemble* e, float* ms);
/* ns3d_profile_step for launch group `group` (0 <= group < groups of
 * ns3d_ensemble_info): device time of each kernel class of one step of all the
 * group's members, over `reps` steps that advance those members; grid size N of
 * the group in *n_out. */
ns3d_status ns3d_ensemble_profile(ns3d_ensemble* e, int group, int reps, const char** names, float* ms,
                                  double* bytes, int max_count, int* count, int* n_out);

/* r2c + 2/3 dealiasing of a host velocity in the reference real layout
 * [N][N][N+2][3] into the state (InitialConditions' transform path,
 * solver.c:1573-1599). */
ns3d_status ns3d_set_state_real_host(ns3d_ctx* ctx, const double* u);

/* ------------------------------------------------------------------------
 * Learned subgrid closure (new; no counterpart in the reference). A 3D CNN
 * (3^3 convolutions 3 -> 32 -> 32 -> 32 -> 6, GELU, circular padding, BF16
 * weights, FP32 accumulation) maps the box-filtered velocity ubar to the
 * subgrid stress tau_ij (xx, yy, zz, xy, xz, yz) on an Nc^3 grid (Nc % 8 == 0).
 * Training pairs come from FP32 runs on a finer grid; attached to a coarse
 * FP32 run, -div(tau) enters every step unless the energy-budget check finds
 * that it would add energy, in which case that step is the plain solve.
 * ------------------------------------------------------------------------ */
typedef struct ns3d_les ns3d_les;
int ns3d_les_num_params(void);
ns3d_status ns3d_les_create(int Nc, int capacity, uint64_t seed, ns3d_les** out);
ns3d_status ns3d_les_destroy(ns3d_les* l);
const char* ns3d_les_last_error(const ns3d_les* l);
/* box-filter the current state of a fine FP32 context (N = F * Nc) into the dataset */
ns3d_status ns3d_les_add_snapshot(ns3d_les* l, ns3d_ctx* fine);
ns3d_status ns3d_les_dataset_size(ns3d_les* l, int* count);
/* box-filtered velocity of a fine context, reference real layout [Nc][Nc][Nc+2][3] */
ns3d_status ns3d_les_filtered_velocity_host(ns3d_les* l, ns3d_ctx* fine, double* ubar);
/* input scale s_in and output scale s_out (default: RMS of ubar over the dataset, its square) */
ns3d_status ns3d_les_set_scales(ns3d_les* l, double s_in, double s_out);
ns3d_status ns3d_les_get_scales(ns3d_les* l, double* s_in, double* s_out);
/* Adam over random dataset samples; mean_loss = mean MSE of the last 10% of iterations.
 * For Nc in {16, 32, 64} the forward, input-gradient and weight-gradient
 * convolutions run on the tensor cores (tcgen05, BF16 operands, FP32
 * accumulation; FP32 master weights for Adam); elsewhere, or after
 * ns3d_les_set_train_path(l, 1), on FP32 CUDA cores. */
ns3d_status ns3d_les_train(ns3d_les* l, int iterations, double lr, double* mean_loss);
/* training path: 0 = tensor cores where compiled (default), 1 = FP32 CUDA cores;
 * ns3d_les_train_path returns the path training will take (0 or 1) */
ns3d_status ns3d_les_set_train_path(ns3d_les* l, int path);
int ns3d_les_train_path(const ns3d_les* l);
ns3d_status ns3d_les_dataset_loss(ns3d_les* l, double* mean_loss);
/* FP32 master weights (ns3d_les_num_params floats), get (set = 0) or set */
ns3d_status ns3d_les_weights_host(ns3d_les* l, float* w, int set);
/* loss and weight gradients for one sample (u [3][Nc^3], tau [6][Nc^3] host floats),
 * through the training path */
ns3d_status ns3d_les_gradients_host(ns3d_les* l, const float* u, const float* tau, double* loss, float* grads);
/* tau = network(u) in physical units, the FP32 training network (FP32 activations) */
ns3d_status ns3d_les_forward_host(ns3d_les* l, const float* u, float* tau);
/* tau = network(u) through the inference path an attached coarse run uses: for
 * Nc in {16, 32, 64} tensor-core convolutions (BF16 activations and weights,
 * FP32 accumulation), otherwise the FP32 network */
ns3d_status ns3d_les_infer_host(ns3d_les* l, const float* u, float* tau);
/* mean device time (CUDA events) of one inference on device-resident input over reps calls */
ns3d_status ns3d_les_profile_infer(ns3d_les* l, int reps, float* ms);
/* attach the closure to a coarse FP32 context of grid Nc (NULL detaches) */
ns3d_status ns3d_les_attach(ns3d_ctx* coarse, ns3d_les* l);
/* steps taken with the closure and steps that fell back to the plain solve */
ns3d_status ns3d_les_counters(ns3d_ctx* coarse, long* closure_steps, long* fallback_steps);

/* ------------------------------------------------------------------------
 * Autotuner. An FP32 engine of a grid size exists in several compiled shapes:
 * tile variants 0..6 (pencils per CTA and radix plans of the strided x and y
 * FFT passes) and up to three z-pass forms (0: persistent bulk-copy line
 * kernel, 1: CTA-synchronous pass, 2: for N in {16, 32, 48, 64, 96, 128} the
 * z transforms as dense DFT matrix products on the tensor cores with split-BF16
 * operands, three terms hi*hi + hi*lo + lo*hi accumulated in FP32, relative
 * error ~1e-5 per transform). ns3d_autotune times every shape of params->N / params->precision on
 * the configuration *params (SPECTRUM initial condition, k0 = 4, seed 0;
 * 3 warm-up steps, then `steps` timed steps) and keeps the fastest in a
 * process-wide table; ns3d_create and ns3d_ensemble_create then build engines
 * of that (N, precision) in the chosen shape. The table can be saved to and
 * loaded from a text file; the environment variable NS3D_TUNING_FILE names a
 * file loaded before the first engine is built. *n_tried counts every shape
 * timed; tried[] receives the first max_tried of them. */
typedef struct {
    int   N;
    int   precision;    /* ns3d_precision                          */
    int   variant;      /* tile variant                            */
    int   zform;        /* z-pass form                             */
    float ms_per_step;  /* timed device milliseconds per step      */
} ns3d_tuning;
ns3d_status ns3d_autotune(const ns3d_params* params, int steps, ns3d_tuning* best, ns3d_tuning* tried,
                          int max_tried, int* n_tried);
/* the same for an ensemble: every (N, precision) group of `members` is timed
 * with all of its members in each shape; one best entry per group */
ns3d_status ns3d_autotune_ensemble(const ns3d_params* members, int count, int steps, ns3d_tuning* best,
                                   int max_best, int* n_best);
ns3d_status ns3d_tuning_get(int N, int precision, ns3d_tuning* t);   /* NS3D_ERR_INVALID: no entry */
ns3d_status ns3d_tuning_set(const ns3d_tuning* t);
ns3d_status ns3d_tuning_clear(void);
ns3d_status ns3d_tuning_save(const char* path);
ns3d_status ns3d_tuning_load(const char* path);

/* Instrumentation for benchmarks: the stream the context runs on, the number
 * of kernels one step launches, and the device time of the last ns3d_step
 * call (CUDA events on the context stream), in milliseconds. */
void* ns3d_stream(ns3d_ctx* ctx);
int ns3d_kernels_per_step(ns3d_ctx* ctx);
ns3d_status ns3d_last_step_ms(ns3d_ctx* ctx, float* ms);
/* Device time of each kernel class of one step, for roofline accounting:
 * names[i] / ms[i] for i < *count (max_count entries at most). */
ns3d_status ns3d_profile_step(ns3d_ctx* ctx, int reps, const char** names, float* ms,
                              double* bytes, int max_count, int* count);
/* Bytes that crossed the host link in the last upload (host -> device) and
 * download (device -> host) of a host array. With pinned (page-locked) host
 * arrays the kernels read only the dealiased modes and write only the
 * 128-byte lines that hold them, while host threads zero the rest of the
 * output array during the step; other host memory goes through a full-size
 * staged copy. */
ns3d_status ns3d_io_bytes(ns3d_ctx* ctx, long long* h2d, long long* d2h);

#ifdef __cplusplus
}
#endif
#endif
