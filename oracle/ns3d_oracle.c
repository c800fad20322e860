/*
 * ns3d_oracle.c — ORACLE: test infrastructure only, never product code.
 *
 * CPU FP64 restatement of the reference solver's time-stepping hot path
 * (Solver/src/solver.c). Used by tests/ as the parity checker and by bench.py
 * as the timed CPU baseline. Each function cites the reference lines it
 * restates. The reference program needs FFTW3-MPI, MPI and parallel HDF5,
 * none of which exist on either machine; its hot-path sources solver.c and
 * utils.c do compile unchanged against the single-rank stand-ins of
 * oracle/ref_shim (make -C oracle ref -> oracle/_ref).
 *
 * Parity pinning: (1) the reference's own code: with the bug-compatibility
 * flags below, this restatement agrees with solver.c's NonlinearRHSBatch,
 * RK4Step, ApplyDealiasing, ComputeSystemMeasurables, InitialConditions and
 * the SpectralSolve loop (tests/test_reference_parity.py, and fixtures made
 * from it, tests/golden/ref_N16.npz); (2) its FFT against numpy.fft
 * (pocketfft) and a direct DFT, the stand-in for the reference's FFTW calls
 * (solver.c:656,658,683,1573,1599); (3) the reference's known-answer test,
 * the Shapiro exact solution (solver.c:1654-1702), and the Taylor–Green
 * invariants E = pi^3, Omega = 3 pi^3 at t = 0; (4) an independent numpy
 * restatement of the RHS and the integrators (tests/golden/make_golden.py).
 *
 * Defects of the reference (solver.c) are fixed here, each behind a flag where
 * reproducing it is meaningful:
 *   D1 transform logical size {N,N,N/2+1} (solver.c:55,2067): fixed, {N,N,N}.
 *   D2 dealias keep-branch aliasing (solver.c:1741): fixed; bugcompat_dealias.
 *   D3 TAYLOR_GREEN overwritten by random modes (solver.c:1553-1606): fixed.
 *   D4 2.0*|x|+|y|+|z| precedence (solver.c:1232-1235): fixed; bugcompat_measures.
 *   D12 helicity Re(u.w) without conjugation (solver.c:1227) is identically
 *       zero: fixed to Re(u.conj(w)); bugcompat_measures keeps the old form.
 *   D13 SHAPIRO w = A cos cos cos(Mz) (solver.c:1593, 1686) is not divergence
 *       free: fixed to sin(Mz); bugcompat_measures keeps the old form.
 *   D15-D19 in the RK5 / Dormand-Prince stepper (solver.c:34-42, 85-154,
 *       217-421): see the comment above rk5_attempt.
 *
 * c2r semantics (FFTW's, restated): the two complex axes are inverted as full
 * complex transforms, then each z line is extended by Hermitian symmetry and
 * the imaginary parts of its kz = 0 and kz = N/2 entries are ignored.
 */
#include "ns3d_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ------------------------------------------------------------------------ */
/* Twiddles: e^{-2 pi i m / n}, reduced by quarter turns so that the         */
/* symmetric values (1, -i, -1, i, ...) come out exact.                       */
/* ------------------------------------------------------------------------ */
static cplx twiddle(long m, long n) {
    m %= n;
    if (m < 0) m += n;
    long q = (4 * m) / n;          /* quarter turns */
    long r = 4 * m - q * n;        /* remainder, angle = (pi/2) * r / n */
    const long double half_pi = acosl(-1.0L) / 2.0L;
    long double cs, sn;
    if (2 * r <= n) {
        long double phi = half_pi * (long double)r / (long double)n;
        cs = cosl(phi);
        sn = sinl(phi);
    } else {
        long double phi = half_pi * (long double)(n - r) / (long double)n;
        cs = sinl(phi);
        sn = cosl(phi);
    }
    double c = (double)cs, s = (double)sn;   /* cos(theta), sin(theta) in the quadrant */
    double cr, sr;
    switch (q) {
        case 0: cr = c;  sr = s;  break;
        case 1: cr = -s; sr = c;  break;
        case 2: cr = -c; sr = -s; break;
        default: cr = s; sr = -c; break;
    }
    return cr - I * sr;            /* e^{-i theta} */
}

/* ------------------------------------------------------------------------ */
/* Mixed-radix recursive decimation-in-time FFT (radix 4, 2, 3, 5, generic). */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n;
    int nfac;
    int fac[64];
    cplx* tw;   /* tw[m] = e^{-2 pi i m / n} */
} fft_plan;

static void plan_init(fft_plan* p, int n) {
    p->n = n;
    p->nfac = 0;
    int m = n;
    while (m % 4 == 0) { p->fac[p->nfac++] = 4; m /= 4; }
    while (m % 2 == 0) { p->fac[p->nfac++] = 2; m /= 2; }
    for (int f = 3; f * f <= m; f += 2)
        while (m % f == 0) { p->fac[p->nfac++] = f; m /= f; }
    if (m > 1) p->fac[p->nfac++] = m;
    p->tw = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    for (int i = 0; i < n; ++i) p->tw[i] = twiddle(i, n);
}

static void plan_free(fft_plan* p) { free(p->tw); p->tw = NULL; }

/* out[k] = sum_j in[j*is] * w^{jk}, w = e^{-+2 pi i/n}; twiddle index scale ts */
static void fft_rec(const cplx* in, long is, cplx* out, int n, const int* fac,
                    const cplx* tw, int ts, int inv) {
    if (n == 1) { out[0] = in[0]; return; }
    const int R = fac[0], m = n / R;
    for (int r = 0; r < R; ++r) fft_rec(in + r * is, is * R, out + r * m, m, fac + 1, tw, ts * R, inv);
    const int N = n * ts;   /* size of the twiddle table */
#define TW(e) (inv ? conj(tw[(long)(e) * ts % N]) : tw[(long)(e) * ts % N])
    if (R == 2) {
        for (int k = 0; k < m; ++k) {
            cplx a = out[k], b = out[m + k] * TW(k);
            out[k] = a + b;
            out[m + k] = a - b;
        }
    } else if (R == 4) {
        const cplx mi = inv ? I : -I;   /* w^{n/4} */
        for (int k = 0; k < m; ++k) {
            cplx a0 = out[k];
            cplx a1 = out[m + k] * TW(k);
            cplx a2 = out[2 * m + k] * TW(2 * k);
            cplx a3 = out[3 * m + k] * TW(3 * k);
            cplx s02 = a0 + a2, d02 = a0 - a2, s13 = a1 + a3, d13 = (a1 - a3) * mi;
            out[k] = s02 + s13;
            out[m + k] = d02 + d13;
            out[2 * m + k] = s02 - s13;
            out[3 * m + k] = d02 - d13;
        }
    } else {
        cplx a[64];
        cplx wr[64];
        for (int q = 0; q < R; ++q) wr[q] = inv ? conj(twiddle(q, R)) : twiddle(q, R);
        for (int k = 0; k < m; ++k) {
            for (int r = 0; r < R; ++r) a[r] = out[r * m + k] * TW((long)r * k);
            for (int q = 0; q < R; ++q) {
                cplx s = 0;
                for (int r = 0; r < R; ++r) s += a[r] * wr[(r * q) % R];
                out[q * m + k] = s;
            }
        }
    }
#undef TW
}

static void fft_exec(const fft_plan* p, const cplx* in, cplx* out, int inv) {
    fft_rec(in, 1, out, p->n, p->fac, p->tw, 1, inv);
}

void orc_fft1d(int n, const double* in, double* out, int inverse) {
    fft_plan p;
    plan_init(&p, n);
    fft_exec(&p, (const cplx*)in, (cplx*)out, inverse);
    plan_free(&p);
}

/* Planned form of orc_fft1d, for callers that transform many lines of one
   length (the single-rank FFTW-MPI stand-in under oracle/ref_shim). */
struct orc_fft_plan_s { fft_plan p; };

orc_fft_plan_t* orc_fft_plan_create(int n) {
    if (n < 1) return NULL;
    orc_fft_plan_t* q = (orc_fft_plan_t*)malloc(sizeof(orc_fft_plan_t));
    plan_init(&q->p, n);
    return q;
}

void orc_fft_plan_exec(const orc_fft_plan_t* q, const double* in, double* out, int inverse) {
    fft_exec(&q->p, (const cplx*)in, (cplx*)out, inverse);
}

void orc_fft_plan_destroy(orc_fft_plan_t* q) {
    if (!q) return;
    plan_free(&q->p);
    free(q);
}

/* ------------------------------------------------------------------------ */
/* Batched Stockham FFT (radix 4, 2, 3) of B interleaved lines, x[j * B + b]: */
/* the 3D transforms below gather blocks of B contiguous columns, so every   */
/* memory access is a contiguous run, and each stage reads its twiddles from */
/* a per-stage table. Stage with Ns = product of the earlier radices and      */
/* radix R: element j (j < n / R) reads x[j + r n / R], multiplies by          */
/* W_n^{r (j mod Ns) n / (Ns R)}, takes the R-point DFT and writes output r to */
/* (j / Ns) Ns R + (j mod Ns) + r Ns (the self-sorting Stockham order of       */
/* Govindaraju et al., SC 2008). Complex products are written out in real     */
/* arithmetic. Lengths with another prime factor use the per-line transform. */
/* ------------------------------------------------------------------------ */
#define ORC_BCOLS 16   /* columns per block of the x and y passes */

typedef struct {
    int n, nst, ok;
    int rad[40];
    cplx* tw[40];      /* stage s: tw[r * Ns + jm], r < R, jm < Ns */
} bplan;

static inline cplx mul_i(cplx a) { return CMPLX(-cimag(a), creal(a)); }   /* i a */
static inline cplx cm(cplx a, cplx b) {
    const double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
    return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}

static void bplan_init(bplan* p, int n) {
    memset(p, 0, sizeof *p);
    p->n = n;
    int m = n;
    while (m % 4 == 0) { p->rad[p->nst++] = 4; m /= 4; }
    while (m % 2 == 0) { p->rad[p->nst++] = 2; m /= 2; }
    while (m % 3 == 0) { p->rad[p->nst++] = 3; m /= 3; }
    p->ok = (m == 1);
    if (!p->ok) { p->nst = 0; return; }
    int Ns = 1;
    for (int s = 0; s < p->nst; ++s) {
        const int R = p->rad[s];
        p->tw[s] = (cplx*)malloc(sizeof(cplx) * (size_t)R * Ns);
        for (int r = 0; r < R; ++r)
            for (int jm = 0; jm < Ns; ++jm) p->tw[s][r * Ns + jm] = twiddle((long)r * jm * (n / (Ns * R)), n);
        Ns *= R;
    }
}

static void bplan_free(bplan* p) {
    for (int s = 0; s < p->nst; ++s) free(p->tw[s]);
    p->nst = 0;
}

/* forward transform of the B lines of x (y: scratch of the same size) */
static void bfft(const bplan* p, cplx* x, cplx* y, int B) {
    const int n = p->n;
    cplx* src = x;
    cplx* dst = y;
    int Ns = 1;
    for (int s = 0; s < p->nst; ++s) {
        const int R = p->rad[s], Q = n / R;
        const cplx* tw = p->tw[s];
        const size_t is = (size_t)Q * B, os = (size_t)Ns * B;
        for (int j = 0; j < Q; ++j) {
            const int jm = j % Ns;
            const cplx* in = src + (size_t)j * B;
            cplx* out = dst + ((size_t)(j / Ns) * Ns * R + jm) * B;
            if (R == 4) {
                const cplx w1 = tw[Ns + jm], w2 = tw[2 * Ns + jm], w3 = tw[3 * Ns + jm];
                for (int b = 0; b < B; ++b) {
                    const cplx a0 = in[b], a1 = cm(in[is + b], w1), a2 = cm(in[2 * is + b], w2),
                               a3 = cm(in[3 * is + b], w3);
                    const cplx s02 = a0 + a2, d02 = a0 - a2, s13 = a1 + a3, t = a1 - a3;
                    const cplx d13 = CMPLX(cimag(t), -creal(t));   /* -i (a1 - a3) */
                    out[b] = s02 + s13;
                    out[os + b] = d02 + d13;
                    out[2 * os + b] = s02 - s13;
                    out[3 * os + b] = d02 - d13;
                }
            } else if (R == 2) {
                const cplx w1 = tw[Ns + jm];
                for (int b = 0; b < B; ++b) {
                    const cplx a0 = in[b], a1 = cm(in[is + b], w1);
                    out[b] = a0 + a1;
                    out[os + b] = a0 - a1;
                }
            } else {   /* R == 3: X1,2 = a0 - (a1 + a2) / 2 -+ i (sqrt(3) / 2) (a1 - a2) */
                const cplx w1 = tw[Ns + jm], w2 = tw[2 * Ns + jm];
                const double h = 0.86602540378443864676;
                for (int b = 0; b < B; ++b) {
                    const cplx a0 = in[b], a1 = cm(in[is + b], w1), a2 = cm(in[2 * is + b], w2);
                    const cplx t1 = a1 + a2, t2 = a0 - 0.5 * t1, d = a1 - a2;
                    const cplx t3 = CMPLX(h * cimag(d), -h * creal(d));   /* -i (sqrt 3 / 2) (a1 - a2) */
                    out[b] = a0 + t1;
                    out[os + b] = t2 + t3;
                    out[2 * os + b] = t2 - t3;
                }
            }
        }
        cplx* t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    if (src != x) memcpy(x, src, sizeof(cplx) * (size_t)n * B);
}

/* inverse (unnormalised) as conj(DFT(conj(x))) */
static void bfft_inv(const bplan* p, cplx* x, cplx* y, int B) {
    const size_t nb = (size_t)p->n * B;
    for (size_t q = 0; q < nb; ++q) x[q] = conj(x[q]);
    bfft(p, x, y, B);
    for (size_t q = 0; q < nb; ++q) x[q] = conj(x[q]);
}

/* ------------------------------------------------------------------------ */
/* Context                                                                   */
/* ------------------------------------------------------------------------ */
struct orc_ctx {
    orc_params p;
    int N, NF;               /* NF = N/2+1 */
    long nF, nR;             /* complex / real element counts per component */
    int* kx; int* ky; int* kz;
    double* x;               /* collocation points (solver.c:1786-1823) */
    fft_plan plan;
    bplan bp;                /* batched transform of length N (bp.ok: radix 2 / 3 / 4 factors only) */
    cplx* ftmp;              /* c2r scratch, 3 nF (with bp.ok) */
    cplx* u_hat;             /* state, reference layout */
    cplx *rk1, *rk2, *rk3, *rk4, *rk_tmp, *w_hat;
    cplx *rk5, *rk6, *rk7, *u_new;   /* RK5CN / DP5CN only */
    double *vel, *vort, *curl;
    double dp_err;           /* DP5CN: error norm of the last attempt */
    long dp_rejects;
    double t, dt;
    long iters;
    int stage;               /* next stage of orc_stage (0..3) */
    double force_target;
    double last_umax;        /* max(|u|+|v|+|w|) seen by the last stage-1 RHS */
};

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_n_spect(int N) {
    /* solver.c:1384 (cubic) */
    return (int)sqrt(3.0 * pow((double)N / 2.0, 2.0)) + 1;
}

/* InitializeSpaceVariables, solver.c:1764-1826 (single process: local_Nx = N) */
static void init_space(orc_ctx* c) {
    const int N = c->N;
    for (int i = 0; i < N; ++i) {
        c->kx[i] = (i <= N / 2) ? i : i - N;
        c->ky[i] = (i < N / 2 + 1) ? i : -N + i;
        c->x[i] = (double)i * (2.0 * M_PI / (double)N);
    }
    for (int i = 0; i < c->NF; ++i) c->kz[i] = i;
}

orc_ctx* orc_create(const orc_params* p) {
    if (!p || p->N < 4 || (p->N % 2)) return NULL;
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->p = *p;
    if (c->p.visc_pow < 1) c->p.visc_pow = 1;
#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
    c->N = p->N;
    c->NF = p->N / 2 + 1;
    c->nF = (long)c->N * c->N * c->NF;
    c->nR = (long)c->N * c->N * (c->N + 2);
    c->kx = (int*)malloc(sizeof(int) * c->N);
    c->ky = (int*)malloc(sizeof(int) * c->N);
    c->kz = (int*)malloc(sizeof(int) * c->NF);
    c->x = (double*)malloc(sizeof(double) * c->N);
    init_space(c);
    plan_init(&c->plan, c->N);
    bplan_init(&c->bp, c->N);
    if (c->bp.ok) c->ftmp = (cplx*)malloc(sizeof(cplx) * 3 * (size_t)c->nF);
    size_t fb = sizeof(cplx) * 3 * (size_t)c->nF, rb = sizeof(double) * 3 * (size_t)c->nR;
    c->u_hat = (cplx*)calloc(1, fb);
    c->rk1 = (cplx*)calloc(1, fb);
    c->rk2 = (cplx*)calloc(1, fb);
    c->rk3 = (cplx*)calloc(1, fb);
    c->rk4 = (cplx*)calloc(1, fb);
    c->rk_tmp = (cplx*)calloc(1, fb);
    c->w_hat = (cplx*)calloc(1, fb);
    if (p->integrator == ORC_RK5CN || p->integrator == ORC_DP5CN) {
        c->rk5 = (cplx*)calloc(1, fb);
        c->rk6 = (cplx*)calloc(1, fb);
        c->rk7 = (cplx*)calloc(1, fb);
        c->u_new = (cplx*)calloc(1, fb);
    }
    if (!(c->p.dp_atol > 0.0)) c->p.dp_atol = 1e-7;
    if (!(c->p.dp_rtol > 0.0)) c->p.dp_rtol = 1e-7;
    c->vel = (double*)calloc(1, rb);
    c->vort = (double*)calloc(1, rb);
    c->curl = (double*)calloc(1, rb);
    c->t = p->t0;
    c->dt = p->dt;
    c->iters = 0;
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    free(c->kx); free(c->ky); free(c->kz); free(c->x);
    plan_free(&c->plan);
    bplan_free(&c->bp);
    free(c->ftmp);
    free(c->u_hat); free(c->rk1); free(c->rk2); free(c->rk3); free(c->rk4);
    free(c->rk_tmp); free(c->w_hat); free(c->vel); free(c->vort); free(c->curl);
    free(c->rk5); free(c->rk6); free(c->rk7); free(c->u_new);
    free(c);
}

static double energy_shells(orc_ctx* c, const cplx* u, int kmax_bin);

void orc_set_state(orc_ctx* c, const double* u_hat) {
    memcpy(c->u_hat, u_hat, sizeof(cplx) * 3 * (size_t)c->nF);
    if (c->p.forcing == ORC_FORCE_SHELL) c->force_target = energy_shells(c, c->u_hat, c->p.force_k);
}
void orc_get_state(const orc_ctx* c, double* u_hat) {
    memcpy(u_hat, c->u_hat, sizeof(cplx) * 3 * (size_t)c->nF);
}
void orc_set_time(orc_ctx* c, double t, double dt, long iters) {
    c->t = t;
    c->dt = dt;
    c->iters = iters;
    c->stage = 0;
}
void orc_get_time(const orc_ctx* c, double* t, double* dt, long* iters) {
    if (t) *t = c->t;
    if (dt) *dt = c->dt;
    if (iters) *iters = c->iters;
}
double orc_forcing_target(const orc_ctx* c) { return c->force_target; }
void orc_set_forcing_target(orc_ctx* c, double e) { c->force_target = e; }

/* ------------------------------------------------------------------------ */
/* 3D transforms, batched over 3 interleaved components (replaces the FFTW   */
/* plans of solver.c:2045-2068 with the logical size {N,N,N}, i.e. D1 fixed) */
/* ------------------------------------------------------------------------ */
/* y (along j at fixed i) or x (along i at fixed j) pass over blocks of
   ORC_BCOLS contiguous columns of the C = 3 NF complex values of an (i, j)
   row; inv selects the inverse transform */
static void pass_xy(orc_ctx* c, const cplx* src, cplx* dst, int axis_x, int inv) {
    const int N = c->N, C = 3 * c->NF;
    const int nblk = (C + ORC_BCOLS - 1) / ORC_BCOLS;
    const size_t rs = axis_x ? (size_t)N * C : (size_t)C;   /* row stride along the transformed axis */
#pragma omp parallel
    {
        cplx* x = (cplx*)malloc(sizeof(cplx) * (size_t)N * ORC_BCOLS);
        cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)N * ORC_BCOLS);
#pragma omp for collapse(2) schedule(static)
        for (int o = 0; o < N; ++o)
            for (int blk = 0; blk < nblk; ++blk) {
                const int c0 = blk * ORC_BCOLS, B = C - c0 < ORC_BCOLS ? C - c0 : ORC_BCOLS;
                const size_t off = (axis_x ? (size_t)o * C : (size_t)o * N * C) + c0;
                for (int r = 0; r < N; ++r) memcpy(x + (size_t)r * B, src + off + r * rs, sizeof(cplx) * B);
                if (inv) bfft_inv(&c->bp, x, y, B);
                else bfft(&c->bp, x, y, B);
                for (int r = 0; r < N; ++r) memcpy(dst + off + r * rs, x + (size_t)r * B, sizeof(cplx) * B);
            }
        free(x);
        free(y);
    }
}

/* z lines of one x plane i, JB consecutive j at a time: the 3 JB real lines
   (j, d) packed in pairs as complex lines, z = line 2q + i line 2q+1 */
static int z_block(int N) { return N % 4 == 0 ? 4 : 2; }

static void r2c_fast(orc_ctx* c, const double* real, cplx* out) {
    const int N = c->N, NF = c->NF, JB = z_block(N), B = 3 * JB / 2;
#pragma omp parallel
    {
        cplx* x = (cplx*)malloc(sizeof(cplx) * (size_t)N * B);
        cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)N * B);
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int j0 = 0; j0 < N; j0 += JB) {
                for (int k = 0; k < N; ++k)
                    for (int q = 0; q < B; ++q) {
                        const int la = 2 * q, lb = 2 * q + 1;
                        const double va = real[3 * ((long)(i * N + j0 + la / 3) * (N + 2) + k) + la % 3];
                        const double vb = real[3 * ((long)(i * N + j0 + lb / 3) * (N + 2) + k) + lb % 3];
                        x[(size_t)k * B + q] = CMPLX(va, vb);
                    }
                bfft(&c->bp, x, y, B);
                /* X_a[k] = (Z[k] + conj Z[N-k]) / 2, X_b[k] = (Z[k] - conj Z[N-k]) / (2 i) */
                for (int k = 0; k < NF; ++k)
                    for (int q = 0; q < B; ++q) {
                        const cplx z = x[(size_t)k * B + q], zc = conj(x[(size_t)((N - k) % N) * B + q]);
                        const cplx sa = z + zc, sb = z - zc;
                        const int la = 2 * q, lb = 2 * q + 1;
                        out[3 * ((long)(i * N + j0 + la / 3) * NF + k) + la % 3] = 0.5 * sa;
                        out[3 * ((long)(i * N + j0 + lb / 3) * NF + k) + lb % 3] = CMPLX(0.5 * cimag(sb), -0.5 * creal(sb));
                    }
            }
        free(x);
        free(y);
    }
    pass_xy(c, out, out, 0, 0);   /* y */
    pass_xy(c, out, out, 1, 0);   /* x */
}

static void c2r_fast(orc_ctx* c, const cplx* in, double* real) {
    const int N = c->N, NF = c->NF, JB = z_block(N), B = 3 * JB / 2;
    cplx* tmp = c->ftmp;     /* the input is preserved */
    pass_xy(c, in, tmp, 1, 1);    /* x */
    pass_xy(c, tmp, tmp, 0, 1);   /* y */
#pragma omp parallel
    {
        cplx* x = (cplx*)malloc(sizeof(cplx) * (size_t)N * B);
        cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)N * B);
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int j0 = 0; j0 < N; j0 += JB) {
                /* Z[k] = A[k] + i B[k] over the Hermitian extension of the two half lines;
                   the imaginary parts of their kz = 0 and kz = N/2 entries are ignored */
                for (int q = 0; q < B; ++q) {
                    const int la = 2 * q, lb = 2 * q + 1;
                    const cplx* ha = tmp + 3 * ((long)(i * N + j0 + la / 3) * NF) + la % 3;
                    const cplx* hb = tmp + 3 * ((long)(i * N + j0 + lb / 3) * NF) + lb % 3;
                    for (int k = 0; k < N; ++k) {
                        cplx a, b;
                        if (k == 0 || k == N / 2) {
                            a = creal(ha[3 * k]);
                            b = creal(hb[3 * k]);
                        } else if (k < N / 2) {
                            a = ha[3 * k];
                            b = hb[3 * k];
                        } else {
                            a = conj(ha[3 * (N - k)]);
                            b = conj(hb[3 * (N - k)]);
                        }
                        x[(size_t)k * B + q] = CMPLX(creal(a) - cimag(b), cimag(a) + creal(b));
                    }
                }
                bfft_inv(&c->bp, x, y, B);
                for (int q = 0; q < B; ++q) {
                    const int la = 2 * q, lb = 2 * q + 1;
                    double* ra = real + 3 * ((long)(i * N + j0 + la / 3) * (N + 2)) + la % 3;
                    double* rb = real + 3 * ((long)(i * N + j0 + lb / 3) * (N + 2)) + lb % 3;
                    for (int k = 0; k < N; ++k) {
                        ra[3 * k] = creal(x[(size_t)k * B + q]);
                        rb[3 * k] = cimag(x[(size_t)k * B + q]);
                    }
                    ra[3 * N] = ra[3 * (N + 1)] = 0.0;
                    rb[3 * N] = rb[3 * (N + 1)] = 0.0;
                }
            }
        free(x);
        free(y);
    }
}

void orc_fft_r2c(orc_ctx* c, const double* real, double* u_hat_d) {
    const int N = c->N, NF = c->NF;
    cplx* out = (cplx*)u_hat_d;
    if (c->bp.ok) {
        r2c_fast(c, real, out);
        return;
    }
    /* z: real lines -> half spectrum */
#pragma omp parallel
    {
        cplx* a = (cplx*)malloc(sizeof(cplx) * N);
        cplx* b = (cplx*)malloc(sizeof(cplx) * N);
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int d = 0; d < 3; ++d) {
                    const double* line = real + 3 * ((long)(i * N + j) * (N + 2));
                    for (int k = 0; k < N; ++k) a[k] = line[3 * k + d];
                    fft_exec(&c->plan, a, b, 0);
                    for (int k = 0; k < NF; ++k) out[3 * ((long)(i * N + j) * NF + k) + d] = b[k];
                }
        /* y */
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < NF; ++k)
                for (int d = 0; d < 3; ++d) {
                    for (int j = 0; j < N; ++j) a[j] = out[3 * ((long)(i * N + j) * NF + k) + d];
                    fft_exec(&c->plan, a, b, 0);
                    for (int j = 0; j < N; ++j) out[3 * ((long)(i * N + j) * NF + k) + d] = b[j];
                }
        /* x */
#pragma omp for collapse(2) schedule(static)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k)
                for (int d = 0; d < 3; ++d) {
                    for (int i = 0; i < N; ++i) a[i] = out[3 * ((long)(i * N + j) * NF + k) + d];
                    fft_exec(&c->plan, a, b, 0);
                    for (int i = 0; i < N; ++i) out[3 * ((long)(i * N + j) * NF + k) + d] = b[i];
                }
        free(a);
        free(b);
    }
}

void orc_fft_c2r(orc_ctx* c, const double* u_hat_d, double* real) {
    const int N = c->N, NF = c->NF;
    const cplx* in = (const cplx*)u_hat_d;
    if (c->bp.ok) {
        c2r_fast(c, in, real);
        return;
    }
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * 3 * (size_t)c->nF);   /* preserve input */
#pragma omp parallel
    {
        cplx* a = (cplx*)malloc(sizeof(cplx) * N);
        cplx* b = (cplx*)malloc(sizeof(cplx) * N);
        /* x */
#pragma omp for collapse(2) schedule(static)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k)
                for (int d = 0; d < 3; ++d) {
                    for (int i = 0; i < N; ++i) a[i] = in[3 * ((long)(i * N + j) * NF + k) + d];
                    fft_exec(&c->plan, a, b, 1);
                    for (int i = 0; i < N; ++i) tmp[3 * ((long)(i * N + j) * NF + k) + d] = b[i];
                }
        /* y */
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < NF; ++k)
                for (int d = 0; d < 3; ++d) {
                    for (int j = 0; j < N; ++j) a[j] = tmp[3 * ((long)(i * N + j) * NF + k) + d];
                    fft_exec(&c->plan, a, b, 1);
                    for (int j = 0; j < N; ++j) tmp[3 * ((long)(i * N + j) * NF + k) + d] = b[j];
                }
        /* z: Hermitian extension, imaginary parts of kz = 0 and kz = N/2 ignored */
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int d = 0; d < 3; ++d) {
                    const cplx* h = tmp + 3 * ((long)(i * N + j) * NF);
                    a[0] = creal(h[d]);
                    for (int k = 1; k < N / 2; ++k) {
                        a[k] = h[3 * k + d];
                        a[N - k] = conj(h[3 * k + d]);
                    }
                    a[N / 2] = creal(h[3 * (N / 2) + d]);
                    fft_exec(&c->plan, a, b, 1);
                    double* line = real + 3 * ((long)(i * N + j) * (N + 2));
                    for (int k = 0; k < N; ++k) line[3 * k + d] = creal(b[k]);
                    line[3 * N + d] = 0.0;
                    line[3 * (N + 1) + d] = 0.0;
                }
        free(a);
        free(b);
    }
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* ApplyDealiasing, solver.c:1709-1756 (2/3 rule, __DEALIAS_23)              */
/* ------------------------------------------------------------------------ */
void orc_dealias(orc_ctx* c, double* arr_d, int array_dim) {
    const int N = c->N, NF = c->NF;
    cplx* array = (cplx*)arr_d;
    /* modes are independent unless D2 is reproduced (its copies read other modes in order) */
#pragma omp parallel for collapse(2) schedule(static) if (!c->p.bugcompat_dealias)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long indx = (long)(i * N + j) * NF + k;
                if (sqrt((double)c->kx[i] * c->kx[i] + c->ky[j] * c->ky[j] + c->kz[k] * c->kz[k]) > N / 3) {
                    for (int l = 0; l < array_dim; ++l) array[array_dim * indx + l] = 0.0;
                } else if (c->p.bugcompat_dealias) {
                    /* D2 reproduced: solver.c:1741 copies array[indx+l] */
                    for (int l = 0; l < array_dim; ++l) array[array_dim * indx + l] = array[indx + l];
                }
            }
}

/* ------------------------------------------------------------------------ */
/* NonlinearRHSBatch, solver.c:620-731                                       */
/* ------------------------------------------------------------------------ */
static void rhs_impl(orc_ctx* c, const cplx* u_hat, cplx* dw, int want_umax) {
    const int N = c->N, NF = c->NF;
    const double norm = 1.0 / pow((double)N * N * N, 2.0);
    /* curl in Fourier space (solver.c:637-650) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long indx = (long)(i * N + j) * NF + k;
                const cplx* u = u_hat + 3 * indx;
                dw[3 * indx + 0] = mul_i(c->ky[j] * u[2] - c->kz[k] * u[1]);
                dw[3 * indx + 1] = mul_i(c->kz[k] * u[0] - c->kx[i] * u[2]);
                dw[3 * indx + 2] = mul_i(c->kx[i] * u[1] - c->ky[j] * u[0]);
            }
    /* to real space (solver.c:656-658) */
    orc_fft_c2r(c, (const double*)dw, c->vort);
    orc_fft_c2r(c, (const double*)u_hat, c->vel);
    /* u x w (solver.c:664-677), plus the CFL speed bound on the true velocity */
    const double inv3 = 1.0 / ((double)N * N * N);
    double umax = 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(max : umax)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k) {
                long indx = (long)(i * N + j) * (N + 2) + k;
                const double* u = c->vel + 3 * indx;
                const double* w = c->vort + 3 * indx;
                double* o = c->curl + 3 * indx;
                o[0] = u[1] * w[2] - u[2] * w[1];
                o[1] = u[2] * w[0] - u[0] * w[2];
                o[2] = u[0] * w[1] - u[1] * w[0];
                if (want_umax) {
                    double s = (fabs(u[0]) + fabs(u[1]) + fabs(u[2])) * inv3;
                    if (s > umax) umax = s;
                }
            }
    if (want_umax) c->last_umax = umax;
    /* back to Fourier space (solver.c:683) */
    orc_fft_r2c(c, c->curl, (double*)dw);
    /* normalise + Leray projection (solver.c:689-721) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long indx = (long)(i * N + j) * NF + k;
                cplx* n = dw + 3 * indx;
                n[0] *= norm;
                n[1] *= norm;
                n[2] *= norm;
                if (c->kx[i] != 0 || c->ky[j] != 0 || c->kz[k] != 0) {
                    double kinv = 1.0 / (double)(c->kx[i] * c->kx[i] + c->ky[j] * c->ky[j] + c->kz[k] * c->kz[k]);
                    cplx kdn = c->kx[i] * n[0] + c->ky[j] * n[1] + c->kz[k] * n[2];
                    n[0] -= c->kx[i] * kinv * kdn;
                    n[1] -= c->ky[j] * kinv * kdn;
                    n[2] -= c->kz[k] * kinv * kdn;
                } else {
                    n[0] = n[1] = n[2] = 0.0;
                }
            }
    /* dealias (solver.c:727) */
    orc_dealias(c, (double*)dw, 3);
}

void orc_rhs(orc_ctx* c, const double* u_hat, double* rhs) {
    rhs_impl(c, (const cplx*)u_hat, (cplx*)rhs, 0);
}

double orc_max_speed_sum(orc_ctx* c) {
    rhs_impl(c, c->u_hat, c->rk1, 1);
    return c->last_umax;
}

/* |k|^2 and the viscous operator nu (k^2)^p (solver.c:580-587) */
static inline double visc(const orc_ctx* c, int i, int j, int k) {
    double k2 = (double)(c->kx[i] * c->kx[i] + c->ky[j] * c->ky[j] + c->kz[k] * c->kz[k]);
    return c->p.visc_pow == 2 ? c->p.nu * k2 * k2 : c->p.nu * k2;
}

/* energy in the shells 1 <= round(|k|) <= kb (forcing, new component) */
static double energy_shells(orc_ctx* c, const cplx* u, int kb) {
    const int N = c->N, NF = c->NF;
    const long k2max = (long)kb * (kb + 1);   /* round(sqrt(k2)) <= kb  <=>  k2 <= kb(kb+1) */
    double e = 0.0;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long k2 = (long)c->kx[i] * c->kx[i] + (long)c->ky[j] * c->ky[j] + (long)c->kz[k] * c->kz[k];
                if (k2 == 0 || k2 > k2max) continue;
                long indx = (long)(i * N + j) * NF + k;
                double m = (k == 0 || k == NF - 1) ? 1.0 : 2.0;
                const cplx* v = u + 3 * indx;
                e += m * (creal(v[0] * conj(v[0])) + creal(v[1] * conj(v[1])) + creal(v[2] * conj(v[2])));
            }
    return 8.0 * pow(M_PI, 3.0) * 0.5 / pow((double)N * N * N, 2.0) * e;
}

static void apply_forcing(orc_ctx* c) {
    const int N = c->N, NF = c->NF, kb = c->p.force_k;
    const long k2max = (long)kb * (kb + 1);
    double e = energy_shells(c, c->u_hat, kb);
    if (!(e > 0.0) || !(c->force_target > 0.0)) return;
    double s = sqrt(c->force_target / e);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long k2 = (long)c->kx[i] * c->kx[i] + (long)c->ky[j] * c->ky[j] + (long)c->kz[k] * c->kz[k];
                if (k2 == 0 || k2 > k2max) continue;
                long indx = (long)(i * N + j) * NF + k;
                for (int d = 0; d < 3; ++d) c->u_hat[3 * indx + d] *= s;
            }
}

/* ------------------------------------------------------------------------ */
/* One time step. RK4 + Crank–Nicolson factor restates RK4Step              */
/* (solver.c:505-608). IF-RK4 is Lawson's integrating-factor RK4 (1967):     */
/*   E = exp(-nu k^2p h/2);  k1 = N(u); k2 = N(E(u + h/2 k1));               */
/*   k3 = N(E u + h/2 k2);  k4 = N(E^2 u + h E k3);                          */
/*   u+ = E^2 u + h/6 (E^2 k1 + 2E (k2 + k3) + k4)                           */
/* ------------------------------------------------------------------------ */
#define FOR_MODES                                                   \
    _Pragma("omp parallel for collapse(2) schedule(static)")        \
    for (int i = 0; i < N; ++i)                                     \
        for (int j = 0; j < N; ++j)                                 \
            for (int k = 0; k < NF; ++k)

/* One stage s = 0..3 of a step: the stage's nonlinear evaluation and the
   stage algebra that follows it; stage 3 ends with the final update, the
   forcing and the time bookkeeping. */
static void stage_step(orc_ctx* c, int st) {
    const int N = c->N, NF = c->NF;
    cplx* u = c->u_hat;
    const int cfl = c->p.cfl > 0.0;
    if (st == 0) {
        rhs_impl(c, u, c->rk1, cfl);
        if (cfl) {
            if (c->last_umax > 0.0) c->dt = c->p.cfl * (2.0 * M_PI / (double)N) / c->last_umax;
        }
    }
    const double h = c->dt;
    if (c->p.integrator == ORC_RK4CN) {
        if (st == 0) {
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = u[x + d] + h * 0.5 * c->rk1[x + d];
            }
        } else if (st == 1) {
            rhs_impl(c, c->rk_tmp, c->rk2, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = u[x + d] + h * 0.5 * c->rk2[x + d];
            }
        } else if (st == 2) {
            rhs_impl(c, c->rk_tmp, c->rk3, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = u[x + d] + h * 1.0 * c->rk3[x + d];
            }
        } else {
            rhs_impl(c, c->rk_tmp, c->rk4, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double D = h * visc(c, i, j, k);
                for (int d = 0; d < 3; ++d)
                    u[x + d] = u[x + d] * ((2.0 - D) / (2.0 + D)) +
                               (2.0 * h / (2.0 + D)) * (1.0 / 6.0 * c->rk1[x + d] + 1.0 / 3.0 * c->rk2[x + d] +
                                                        1.0 / 3.0 * c->rk3[x + d] + 1.0 / 6.0 * c->rk4[x + d]);
            }
        }
    } else {
        if (st == 0) {
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double E = exp(-0.5 * h * visc(c, i, j, k));
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = E * (u[x + d] + 0.5 * h * c->rk1[x + d]);
            }
        } else if (st == 1) {
            rhs_impl(c, c->rk_tmp, c->rk2, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double E = exp(-0.5 * h * visc(c, i, j, k));
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = E * u[x + d] + 0.5 * h * c->rk2[x + d];
            }
        } else if (st == 2) {
            rhs_impl(c, c->rk_tmp, c->rk3, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double E = exp(-0.5 * h * visc(c, i, j, k));
                for (int d = 0; d < 3; ++d) c->rk_tmp[x + d] = E * E * u[x + d] + h * E * c->rk3[x + d];
            }
        } else {
            rhs_impl(c, c->rk_tmp, c->rk4, 0);
            FOR_MODES {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double E = exp(-0.5 * h * visc(c, i, j, k));
                double E2 = E * E;
                for (int d = 0; d < 3; ++d)
                    u[x + d] = E2 * u[x + d] +
                               h / 6.0 * (E2 * c->rk1[x + d] + 2.0 * E * (c->rk2[x + d] + c->rk3[x + d]) + c->rk4[x + d]);
            }
        }
    }
    if (st == 3) {
        if (c->p.forcing == ORC_FORCE_SHELL) apply_forcing(c);
        c->iters += 1;
        if (cfl) c->t += h;
        else c->t = c->p.t0 + (double)c->iters * h;
    }
}

static void one_step(orc_ctx* c) {
    for (int st = 0; st < 4; ++st) stage_step(c, st);
}

int orc_stage(orc_ctx* c) {
    if (c->p.integrator != ORC_IFRK4 && c->p.integrator != ORC_RK4CN) return -1;
    stage_step(c, c->stage);
    c->stage = (c->stage + 1) & 3;
    return c->stage;
}

/* ------------------------------------------------------------------------ */
/* RK5 family: RK5DPStep (solver.c:217-421) with the Crank–Nicolson factor   */
/* of the __NAVIER branch (solver.c:356-371), and the adaptive Dormand–      */
/* Prince loop of SpectralSolve (solver.c:134-154).                          */
/*   stages   k_s = N(u + h sum_{j<s} a_sj k_j)      (no viscosity in stages) */
/*   update   u+ = u (2-D)/(2+D) + 2h/(2+D) sum_j b_j k_j,  D = h nu k^2p     */
/* RK5CN evaluates 6 stages; DP5CN a 7th (a_7j = b_j) for the embedded        */
/* 4th-order solution u* = u (2-D)/(2+D) + 2h/(2+D) sum_j b*_j k_j and        */
/*   err = max_d sqrt( sum_modes |u+_d - u*_d|^2 / den_d^2 / (N N (N/2+1)) ), */
/*   den_d = atol + max(|u_d|, |u+_d|) rtol   (solver.c:382-408)             */
/* The step is accepted when err <= 1; either way the next attempt uses      */
/*   h' = h min(1.5, max(0.01, 0.8 err^(-1/5)))   (solver.c:140).            */
/* Defects of the reference fixed here:                                       */
/*   D15 the accept test is inverted (a step with err <= 1 is retried,        */
/*       solver.c:143) and a rejected attempt is not undone (the next attempt */
/*       starts from the already updated u_hat): here err <= 1 accepts and a  */
/*       rejection restarts from the step's initial state.                    */
/*   D16 err_sum_* are used uninitialised (solver.c:229-232) and no error is  */
/*       formed on the first step (iters > 1, solver.c:374): here the sums    */
/*       start at 0 on every attempt.                                         */
/*   D17 the higher-order solution is built from the updated u_hat without    */
/*       the viscous factor (solver.c:376-378), so the "error" is            */
/*       dt sum b*_j k_j, not a difference of two solutions: here u+ - u*.    */
/*   D18 pow() of a complex argument keeps only its real part                 */
/*       (solver.c:387-389): here |.|^2 of the complex difference; the retry  */
/*       counter is never reset (solver.c:91): here 50 tries per step; t is   */
/*       iters*dt with a variable dt (solver.c:193): here t += h.             */
/*   D19 a32 = 1/2 (solver.c:36); Dormand & Prince (1980) have 9/40, which    */
/*       the consistency condition a31 + a32 = c3 = 3/10 requires.           */
/*       bugcompat_rk5 keeps 1/2.                                             */
/* ------------------------------------------------------------------------ */
static const double DP_A[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5.0, 0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
    {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
static const double DP_B[7] = {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0};
static const double DP_BS[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                                187.0 / 2100.0, 1.0 / 40.0};

/* one RK5CN step (dp = 0, written into u_hat) or one DP5CN attempt (dp = 1,
   written into u_new; returns the error norm) */
static double rk5_attempt(orc_ctx* c, double h, int dp) {
    const int N = c->N, NF = c->NF;
    cplx* u = c->u_hat;
    cplx* K[7] = {c->rk1, c->rk2, c->rk3, c->rk4, c->rk5, c->rk6, c->rk7};
    const int S = dp ? 7 : 6;
    double A[7][6];
    memcpy(A, DP_A, sizeof(A));
    if (c->p.bugcompat_rk5) A[2][1] = 0.5;
    rhs_impl(c, u, K[0], 0);
    for (int s = 1; s < S; ++s) {
        FOR_MODES {
            long x = 3 * ((long)(i * N + j) * NF + k);
            for (int d = 0; d < 3; ++d) {
                cplx v = u[x + d];
                for (int q = 0; q < s; ++q) v += h * A[s][q] * K[q][x + d];
                c->rk_tmp[x + d] = v;
            }
        }
        rhs_impl(c, c->rk_tmp, K[s], 0);
    }
    cplx* out = dp ? c->u_new : u;
    const double atol = c->p.dp_atol, rtol = c->p.dp_rtol;
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : e0, e1, e2)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long x = 3 * ((long)(i * N + j) * NF + k);
                double D = h * visc(c, i, j, k);
                double a = (2.0 - D) / (2.0 + D), b = 2.0 * h / (2.0 + D);
                for (int d = 0; d < 3; ++d) {
                    cplx sb = 0.0, se = 0.0;
                    for (int q = 0; q < 6; ++q) sb += DP_B[q] * K[q][x + d];
                    cplx un = u[x + d] * a + b * sb;
                    if (dp) {
                        for (int q = 0; q < 7; ++q) se += (DP_B[q] - DP_BS[q]) * K[q][x + d];
                        cplx diff = b * se;
                        double m0 = cabs(u[x + d]), m1 = cabs(un);
                        double den = atol + (m0 > m1 ? m0 : m1) * rtol;
                        double r = (creal(diff) * creal(diff) + cimag(diff) * cimag(diff)) / (den * den);
                        if (d == 0) e0 += r; else if (d == 1) e1 += r; else e2 += r;
                    }
                    out[x + d] = un;
                }
            }
    if (!dp) return 0.0;
    const double nm = (double)N * N * NF;
    double err = sqrt(e0 / nm);
    if (sqrt(e1 / nm) > err) err = sqrt(e1 / nm);
    if (sqrt(e2 / nm) > err) err = sqrt(e2 / nm);
    return err;
}

static void end_step(orc_ctx* c, double h, int var_dt) {
    if (c->p.forcing == ORC_FORCE_SHELL) apply_forcing(c);
    c->iters += 1;
    if (var_dt) c->t += h;
    else c->t = c->p.t0 + (double)c->iters * h;
}

static int rk5_step(orc_ctx* c) {
    const int N = c->N;
    if (c->p.integrator == ORC_RK5CN) {
        const int cfl = c->p.cfl > 0.0;
        if (cfl) {
            rhs_impl(c, c->u_hat, c->rk1, 1);
            if (c->last_umax > 0.0) c->dt = c->p.cfl * (2.0 * M_PI / (double)N) / c->last_umax;
        }
        rk5_attempt(c, c->dt, 0);
        end_step(c, c->dt, cfl);
        return 0;
    }
    for (int tries = 0; tries < 50; ++tries) {
        const double h = c->dt;
        const double err = rk5_attempt(c, h, 1);
        double fac = 0.8 * pow(1.0 / err, 0.2);
        fac = fac < 0.01 ? 0.01 : fac;
        fac = fac > 1.5 ? 1.5 : fac;
        c->dp_err = err;
        c->dt = h * fac;
        if (err <= 1.0) {
            memcpy(c->u_hat, c->u_new, sizeof(cplx) * 3 * (size_t)c->nF);
            end_step(c, h, 1);
            return 0;
        }
        c->dp_rejects++;
    }
    return 1;
}

void orc_dp_stats(const orc_ctx* c, double* last_err, long* rejects) {
    if (last_err) *last_err = c->dp_err;
    if (rejects) *rejects = c->dp_rejects;
}

int orc_step(orc_ctx* c, int nsteps) {
    const int rk5 = c->p.integrator == ORC_RK5CN || c->p.integrator == ORC_DP5CN;
    for (int s = 0; s < nsteps; ++s) {
        if (!rk5) one_step(c);
        else if (rk5_step(c)) return 1;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* ComputeSystemMeasurables, solver.c:1142-1276 (D4 fixed unless bugcompat)  */
/* totals: [energy, enstrophy, palinstrophy, helicity, energy dissipation]   */
/* ------------------------------------------------------------------------ */
void orc_measurables(orc_ctx* c, double* tot, double* Ek, double* Ok) {
    const int N = c->N, NF = c->NF, ns = orc_n_spect(N);
    const double norm_fac = 0.5 / pow((double)N * N * N, 2.0);
    const double const_fac = 8.0 * pow(M_PI, 3.0);
    double s_diss = 0, s_enst = 0, s_pal = 0, s_hel = 0, s_en = 0;
    if (Ek) memset(Ek, 0, sizeof(double) * ns);
    if (Ok) memset(Ok, 0, sizeof(double) * ns);
    const int bug = c->p.bugcompat_measures;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < NF; ++k) {
                long indx = (long)(i * N + j) * NF + k;
                const cplx* u = c->u_hat + 3 * indx;
                double kx = c->kx[i], ky = c->ky[j], kz = c->kz[k];
                cplx wx = I * (ky * u[2] - kz * u[1]);
                cplx wy = I * (kz * u[0] - kx * u[2]);
                cplx wz = I * (kx * u[1] - ky * u[0]);
                cplx cx = I * (ky * wz - kz * wy);
                cplx cy = I * (kz * wx - kx * wz);
                cplx cz = I * (kx * wy - ky * wx);
                double k2 = kx * kx + ky * ky + kz * kz;
                double pre = c->p.visc_pow == 2 ? c->p.nu * k2 * k2 : c->p.nu * k2;
                double ux2 = cabs(u[0] * conj(u[0])), uy2 = cabs(u[1] * conj(u[1])), uz2 = cabs(u[2] * conj(u[2]));
                double wx2 = cabs(wx * conj(wx)), wy2 = cabs(wy * conj(wy)), wz2 = cabs(wz * conj(wz));
                double cx2 = cabs(cx * conj(cx)), cy2 = cabs(cy * conj(cy)), cz2 = cabs(cz * conj(cz));
                /* D12: the reference's Re(u.w) (solver.c:1227) is identically zero since
                 * u.(k x u) = 0; the Parseval form of the helicity conjugates w. */
                double hel = bug ? creal(u[0] * wx + u[1] * wy + u[2] * wz)
                                 : creal(u[0] * conj(wx) + u[1] * conj(wy) + u[2] * conj(wz));
                if (k == 0 || k == NF - 1) {
                    s_diss += pre * (ux2 + uy2 + uz2);
                    s_enst += wx2 + wy2 + wz2;
                    s_pal += cx2 + cy2 + cz2;
                    s_hel += hel;
                    s_en += ux2 + uy2 + uz2;
                } else if (bug) {
                    s_diss += 2.0 * pre * (ux2 + uy2 + uz2);
                    s_enst += 2.0 * wx2 + wy2 + wz2;
                    s_pal += 2.0 * cx2 + cy2 + cz2;
                    s_hel += 2.0 * hel;
                    s_en += 2.0 * ux2 + uy2 + uz2;
                } else {
                    s_diss += 2.0 * pre * (ux2 + uy2 + uz2);
                    s_enst += 2.0 * (wx2 + wy2 + wz2);
                    s_pal += 2.0 * (cx2 + cy2 + cz2);
                    s_hel += 2.0 * hel;
                    s_en += 2.0 * (ux2 + uy2 + uz2);
                }
                /* D14: round(|k|) reaches n_spect for the corner modes when the
                 * fraction of sqrt(3)N/2 is >= 1/2 (e.g. N = 8); the reference
                 * writes past the end there (solver.c:1242-1250). Dropped here. */
                int b = (int)round(sqrt(k2));
                double m = (k == 0 || k == NF - 1) ? 1.0 : 2.0;
                if (b >= ns) continue;
                if (Ek) Ek[b] += m * const_fac * norm_fac * (ux2 + uy2 + uz2);
                if (Ok) Ok[b] += m * const_fac * norm_fac * (wx2 + wy2 + wz2);
            }
    tot[0] = s_en * const_fac * norm_fac;
    tot[1] = s_enst * const_fac * norm_fac;
    tot[2] = s_pal * const_fac * norm_fac;
    tot[3] = s_hel * const_fac * norm_fac;
    tot[4] = s_diss * 2.0 * const_fac * norm_fac;
}

/* ------------------------------------------------------------------------ */
/* Initial conditions, solver.c:1537-1648 (D3 fixed: if / else-if chain)     */
/* ------------------------------------------------------------------------ */
static uint64_t splitmix64(uint64_t x) {
    /* SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) finaliser on x + golden gamma */
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double uniform01(uint64_t key, uint64_t id, int r) {
    return (double)(splitmix64(key ^ (id * 8u + (uint64_t)r)) >> 11) * 0x1.0p-53;
}

int orc_ic(orc_ctx* c, const char* name, uint64_t seed, double k0, double energy) {
    const int N = c->N, NF = c->NF;
    cplx* uh = c->u_hat;
    double* u = c->vel;
    if (!strcmp(name, "TAYLOR_GREEN")) {
        /* solver.c:1557-1573, KAPPA = 1 */
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < N; ++k) {
                    long indx = (long)(i * N + j) * (N + 2) + k;
                    u[3 * indx + 0] = sin(c->x[i]) * cos(c->x[j]) * cos(c->x[k]);
                    u[3 * indx + 1] = -cos(c->x[i]) * sin(c->x[j]) * cos(c->x[k]);
                    u[3 * indx + 2] = 0.0;
                }
        orc_fft_r2c(c, u, (double*)uh);
    } else if (!strcmp(name, "SHAPIRO")) {
        /* solver.c:1579-1599 with A = 2, K = L = M = 2 (data_types.h:138-142), t = 0.
         * D13 fixed: the w component is A cos(Kx) cos(Ly) sin(Mz) (Shapiro 1993);
         * the reference's cos(Mz) (solver.c:1593, 1686) is neither solenoidal nor
         * a Beltrami field, so it is not an exact solution. */
        const double A = 2.0, K = 2.0, L = 2.0, M = 2.0;
        const double lam = sqrt(K * K + L * L + M * M);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < N; ++k) {
                    long indx = (long)(i * N + j) * (N + 2) + k;
                    double x = c->x[i], y = c->x[j], z = c->x[k];
                    u[3 * indx + 0] = -A / (K * K + L * L) * (lam * L * cos(K * x) * sin(L * y) * sin(M * z) + M * K * sin(K * x) * cos(L * y) * cos(M * z));
                    u[3 * indx + 1] = A / (K * K + L * L) * (lam * K * sin(K * x) * cos(L * y) * sin(M * z) - M * L * cos(K * x) * sin(L * y) * cos(M * z));
                    u[3 * indx + 2] = A * cos(K * x) * cos(L * y) * (c->p.bugcompat_measures ? cos(M * z) : sin(M * z));
                }
        orc_fft_r2c(c, u, (double*)uh);
    } else if (!strcmp(name, "SPECTRUM")) {
        /* New component: seeded random-phase solenoidal field with
         * E(k) ~ k^4 exp(-2 (k/k0)^2), Hermitian on the kz = 0 plane, scaled
         * to the requested energy. */
        const long kc2 = (long)(N / 3) * (N / 3);
        const uint64_t key = splitmix64(seed);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < NF; ++k) {
                    long indx = (long)(i * N + j) * NF + k;
                    int kx = c->kx[i], ky = c->ky[j], kz = c->kz[k];
                    long k2 = (long)kx * kx + (long)ky * ky + (long)kz * kz;
                    cplx* o = uh + 3 * indx;
                    o[0] = o[1] = o[2] = 0.0;
                    if (k2 == 0 || k2 > kc2) continue;
                    int conj_of = 0;
                    int ci = i, cj = j;
                    if (kz == 0 && !(kx > 0 || (kx == 0 && ky > 0))) {
                        conj_of = 1;
                        ci = (N - i) % N;
                        cj = (N - j) % N;
                    }
                    uint64_t id = (uint64_t)((long)(ci * N + cj) * NF + k);
                    cplx v[3];
                    for (int d = 0; d < 3; ++d)
                        v[d] = (2.0 * uniform01(key, id, 2 * d) - 1.0) + I * (2.0 * uniform01(key, id, 2 * d + 1) - 1.0);
                    double ckx = c->kx[ci], cky = c->ky[cj], ckz = kz;
                    cplx kv = ckx * v[0] + cky * v[1] + ckz * v[2];
                    double kk = (double)k2;
                    v[0] -= ckx * kv / kk;
                    v[1] -= cky * kv / kk;
                    v[2] -= ckz * kv / kk;
                    double vn = sqrt(creal(v[0] * conj(v[0])) + creal(v[1] * conj(v[1])) + creal(v[2] * conj(v[2])));
                    if (!(vn > 1e-300)) continue;
                    double amp = sqrt(kk) * exp(-kk / (k0 * k0)) / vn;
                    for (int d = 0; d < 3; ++d) o[d] = conj_of ? conj(amp * v[d]) : amp * v[d];
                }
        double tot[5];
        orc_measurables(c, tot, NULL, NULL);
        double target = 8.0 * pow(M_PI, 3.0) * energy;
        if (tot[0] > 0.0) {
            double s = sqrt(target / tot[0]);
            for (long n = 0; n < 3 * c->nF; ++n) uh[n] *= s;
        }
    } else if (!strcmp(name, "TESTING")) {
        /* solver.c:1600-1604: no field is set */
        memset(uh, 0, sizeof(cplx) * 3 * (size_t)c->nF);
    } else {
        /* RANDOM and unrecognised names: solver.c:1606-1625 with srand(123456789), D6 kept */
        srand(123456789);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < NF; ++k) {
                    long indx = (long)(i * N + j) * NF + k;
                    for (int d = 0; d < 3; ++d) {
                        double a = (double)rand() / (double)RAND_MAX;
                        double ph = (double)rand() / (double)RAND_MAX;
                        uh[3 * indx + d] = a * cexp(ph * 2.0 * M_PI * I);
                    }
                }
    }
    orc_dealias(c, (double*)uh, 3);
    c->t = c->p.t0;
    c->dt = c->p.dt;
    c->iters = 0;
    c->stage = 0;
    if (c->p.forcing == ORC_FORCE_SHELL) c->force_target = energy_shells(c, uh, c->p.force_k);
    return 0;
}

/* Real-space u and w, normalised by 1/N^3 (hdf5_funcs.c:586-600, 662-676) */
void orc_real_space(orc_ctx* c, double* u, double* w) {
    const int N = c->N, NF = c->NF;
    const double s = 1.0 / ((double)N * N * N);
    if (u) {
        orc_fft_c2r(c, (const double*)c->u_hat, u);
        for (long n = 0; n < 3 * c->nR; ++n) u[n] *= s;
    }
    if (w) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int k = 0; k < NF; ++k) {
                    long indx = (long)(i * N + j) * NF + k;
                    const cplx* v = c->u_hat + 3 * indx;
                    c->w_hat[3 * indx + 0] = I * (c->ky[j] * v[2] - c->kz[k] * v[1]);
                    c->w_hat[3 * indx + 1] = I * (c->kz[k] * v[0] - c->kx[i] * v[2]);
                    c->w_hat[3 * indx + 2] = I * (c->kx[i] * v[1] - c->ky[j] * v[0]);
                }
        orc_fft_c2r(c, (const double*)c->w_hat, w);
        for (long n = 0; n < 3 * c->nR; ++n) w[n] *= s;
    }
}

/* ------------------------------------------------------------------------ */
/* Longitudinal velocity-increment statistics, restating the post-processing */
/* PostProcessing/src/stats.c:22-254 (Precompute, ComputeStats) and          */
/* AllocateStatsObjects (:404-418): for each increment r the samples         */
/* u_a(x + r e_a) - u_a(x), a = x, y, z, with x_a + r < N, pooled. GSL's      */
/* running statistics give min, max, mean, sample sd, skewness m3/sd^3 and    */
/* excess kurtosis m4/sd^4 - 3; here they come from two passes with long      */
/* double sums. Bins: gsl_histogram_set_ranges_uniform over                  */
/* [min - 0.05, max + 0.05], edge b = ((n-b)/n) lo + (b/n) hi, sample d in   */
/* bin b when edge[b] <= d < edge[b+1] (binary search).                      */
/* ------------------------------------------------------------------------ */
static double incr_edge(double lo, double hi, int b, int n) {
    return ((double)(n - b) / (double)n) * lo + ((double)b / (double)n) * hi;
}

void orc_increment_stats(orc_ctx* c, const int* incr, int nr, int nbins, double* stats, double* ranges,
                         double* counts) {
    const int N = c->N;
    const long NP = N + 2;
    double* u = (double*)malloc(sizeof(double) * 3 * (size_t)c->nR);
    orc_real_space(c, u, NULL);
    /* u[((i*N + j)*(N+2) + k)*3 + a] */
#define UAT(i, j, k, a) u[(((long)(i) * N + (j)) * NP + (k)) * 3 + (a)]
    double* edges = (double*)malloc(sizeof(double) * (nbins + 1));
    for (int r = 0; r < nr; ++r) {
        const int dr = incr[r];
        long double n = 0, s1 = 0;
        double mn = 0, mx = 0;
        int first = 1;
        for (int pass = 0; pass < 3; ++pass) {
            long double m2 = 0, m3 = 0, m4 = 0;
            const double mean = n > 0 ? (double)(s1 / n) : 0.0;
            const double lo = mn - 0.05, hi = mx + 0.05;
            if (pass == 2)
                for (int b = 0; b <= nbins; ++b) edges[b] = incr_edge(lo, hi, b, nbins);
            if (pass == 2 && counts)
                for (int b = 0; b < nbins; ++b) counts[(long)r * nbins + b] = 0.0;
            for (int i = 0; i < N; ++i)
                for (int j = 0; j < N; ++j)
                    for (int k = 0; k < N; ++k) {
                        for (int a = 0; a < 3; ++a) {
                            const int ca = a == 0 ? i : a == 1 ? j : k;
                            if (ca + dr >= N) continue;
                            const double d = (a == 0 ? UAT(i + dr, j, k, 0) : a == 1 ? UAT(i, j + dr, k, 1)
                                                                                      : UAT(i, j, k + dr, 2)) -
                                             UAT(i, j, k, a);
                            if (pass == 0) {
                                n += 1;
                                s1 += d;
                                if (first || d < mn) mn = d;
                                if (first || d > mx) mx = d;
                                first = 0;
                            } else if (pass == 1) {
                                const long double e = (long double)d - mean;
                                m2 += e * e;
                                m3 += e * e * e;
                                m4 += e * e * e * e;
                            } else if (counts) {
                                /* binary search for edge[b] <= d < edge[b+1] */
                                int lo_b = 0, hi_b = nbins;
                                while (hi_b - lo_b > 1) {
                                    const int mid = (lo_b + hi_b) / 2;
                                    if (d >= edges[mid]) lo_b = mid;
                                    else hi_b = mid;
                                }
                                counts[(long)r * nbins + lo_b] += 1.0;
                            }
                        }
                    }
            if (pass == 1) {
                const double nn = (double)n;
                const double var = nn > 1 ? (double)(m2 / (n - 1)) : 0.0;
                double* sr = stats + 6 * r;
                sr[0] = n > 0 ? mn : 0.0;
                sr[1] = n > 0 ? mx : 0.0;
                sr[2] = mean;
                sr[3] = sqrt(var);
                sr[4] = var > 0 ? (double)(m3 / n) / pow(var, 1.5) : 0.0;
                sr[5] = var > 0 ? (double)(m4 / n) / (var * var) - 3.0 : 0.0;
                if (n == 0) mn = mx = 0.0;
            }
        }
        if (ranges)
            for (int b = 0; b <= nbins; ++b) ranges[(long)r * (nbins + 1) + b] = edges[b];
    }
#undef UAT
    free(edges);
    free(u);
}
