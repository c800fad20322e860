// ns3d_api.cu — the extern "C" boundary (include/ns3d.h): argument checks,
// context lifetime, status codes and the reference-layout host entry points.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <complex>
#include <vector>

#include "ns3d_base.h"

namespace ns3d {

__global__ void k_dealias_ref_entry(double2* a, int N, int dim);

bool supported_n(int N) {
    switch (N) {
        case 8: case 16: case 24: case 32: case 48: case 64: case 96: case 128: case 192: case 256: case 384: case 512:
        case 768: case 1024:
            return true;
        default:
            return false;
    }
}

// e^{-2 pi i m / n}: quarter-turn reduction so that 1, -i, -1, i are exact,
// then cos/sin of the residual angle evaluated in long double.
void twiddle_table(int n, double* re, double* im) {
    const long double half_pi = acosl(-1.0L) / 2.0L;
    for (long m = 0; m < n; ++m) {
        long q = (4 * m) / n;
        long r = 4 * m - q * n;
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
        double c = (double)cs, s = (double)sn, cr, sr;
        switch (q) {
            case 0: cr = c; sr = s; break;
            case 1: cr = -s; sr = c; break;
            case 2: cr = -c; sr = -s; break;
            default: cr = s; sr = -c; break;
        }
        re[m] = cr;
        im[m] = -sr;
    }
}

// InitialConditions (solver.c:1537-1648) for the selected member of an engine,
// with the if / else-if chain (D3 fixed).
ns3d_status ic_dispatch(Base* impl, int N, const char* name, uint64_t seed, double k0, double energy) {
    if (!strcmp(name, "TAYLOR_GREEN")) return impl->ic_real(0);
    if (!strcmp(name, "SHAPIRO")) return impl->ic_real(1);
    if (!strcmp(name, "TESTING")) return impl->ic_zero();
    if (!strcmp(name, "SPECTRUM")) {
        if (!(k0 > 0) || !(energy > 0)) {
            impl->set_err("SPECTRUM needs k0 > 0 and energy > 0");
            return NS3D_ERR_INVALID;
        }
        return impl->ic_spectrum(seed, k0, energy);
    }
    // RANDOM and unrecognised names: the reference's random modes
    // (solver.c:1606-1625): srand(123456789), amplitude then phase per
    // component, loop order i, j, k; dealiased on upload.
    const int NF = N / 2 + 1;
    std::vector<double> h((size_t)N * N * NF * 3 * 2);
    srand(123456789);
    for (size_t q = 0; q < (size_t)N * N * NF * 3; ++q) {
        const double a = (double)rand() / (double)RAND_MAX;
        const double ph = (double)rand() / (double)RAND_MAX;
        const std::complex<double> v = a * std::exp(std::complex<double>(0.0, ph * 2.0 * M_PI));
        h[2 * q] = v.real();
        h[2 * q + 1] = v.imag();
    }
    return impl->ic_host(h.data());
}

}  // namespace ns3d

#include "ns3d_ctx.h"

static ns3d_status fail(ns3d_ctx* c, ns3d_status s, const char* msg) {
    if (c) snprintf(c->err, sizeof(c->err), "%s", msg);
    return s;
}
static ns3d_status pass(ns3d_ctx* c, ns3d_status s) {
    if (c && s != NS3D_OK && c->impl) snprintf(c->err, sizeof(c->err), "%s", c->impl->err());
    return s;
}

extern "C" {

const char* ns3d_status_string(ns3d_status s) {
    switch (s) {
        case NS3D_OK: return "ok";
        case NS3D_ERR_INVALID: return "invalid argument";
        case NS3D_ERR_UNSUPPORTED: return "unsupported grid size";
        case NS3D_ERR_CUDA: return "CUDA error";
        case NS3D_ERR_NOMEM: return "out of device memory";
        case NS3D_ERR_NUMERIC: return "numeric health check failed";
        case NS3D_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

int ns3d_supported_size(int N) { return ns3d::supported_n(N) ? 1 : 0; }

int ns3d_n_spect(int N) {
    // solver.c:1384 for a cubic grid
    return (int)sqrt(3.0 * pow((double)N / 2.0, 2.0)) + 1;
}

ns3d_status ns3d_create(const ns3d_params* p, ns3d_ctx** out) {
    if (!p || !out) return NS3D_ERR_INVALID;
    *out = nullptr;
    // argument checks of GetCMLArgs (utils.c:87-160)
    if (p->N <= 2 || (p->N % 2) != 0) return NS3D_ERR_INVALID;
    if (!ns3d::supported_n(p->N)) return NS3D_ERR_UNSUPPORTED;
    if (!(p->nu > 0) || !(p->dt > 0) || p->t0 < 0) return NS3D_ERR_INVALID;
    if (p->visc_pow != 1 && p->visc_pow != 2) return NS3D_ERR_INVALID;
    if (p->integrator < NS3D_IFRK4 || p->integrator > NS3D_DP5CN) return NS3D_ERR_INVALID;
    if (p->integrator == NS3D_DP5CN && p->cfl > 0) return NS3D_ERR_INVALID;   // DP5CN chooses its own step
    if (p->precision != NS3D_FP64 && p->precision != NS3D_FP32) return NS3D_ERR_INVALID;
    if (p->forcing != NS3D_FORCE_NONE && p->forcing != NS3D_FORCE_SHELL) return NS3D_ERR_INVALID;
    if (p->forcing == NS3D_FORCE_SHELL && (p->force_k < 1 || p->force_k > p->N / 3)) return NS3D_ERR_INVALID;
    if (p->cfl < 0) return NS3D_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return NS3D_ERR_CUDA;
    if (p->device < 0 || p->device >= ndev) return NS3D_ERR_INVALID;
    if (cudaSetDevice(p->device) != cudaSuccess) return NS3D_ERR_CUDA;

    ns3d_ctx* c = (ns3d_ctx*)calloc(1, sizeof(ns3d_ctx));
    if (!c) return NS3D_ERR_NOMEM;
    c->p = *p;
    if (p->stream) {
        c->stream = (cudaStream_t)p->stream;
        c->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            free(c);
            return NS3D_ERR_CUDA;
        }
        c->own_stream = true;
    }
    c->impl = p->precision == NS3D_FP32 ? ns3d::make_f32(p->N, p, 1, c->stream) : ns3d::make_f64(p->N, p, 1, c->stream);
    if (!c->impl) {
        if (c->own_stream) cudaStreamDestroy(c->stream);
        free(c);
        return NS3D_ERR_UNSUPPORTED;
    }
    ns3d_status s = c->impl->init();
    if (s != NS3D_OK) {
        const bool oom = strstr(c->impl->err(), "out of memory") != nullptr;
        delete c->impl;
        if (c->own_stream) cudaStreamDestroy(c->stream);
        free(c);
        cudaGetLastError();
        return oom ? NS3D_ERR_NOMEM : s;
    }
    *out = c;
    return NS3D_OK;
}

ns3d_status ns3d_destroy(ns3d_ctx* c) {
    if (!c) return NS3D_ERR_INVALID;
    cudaStreamSynchronize(c->stream);
    delete c->impl;
    if (c->own_stream) cudaStreamDestroy(c->stream);
    free(c);
    return NS3D_OK;
}

const char* ns3d_last_error(const ns3d_ctx* c) { return c ? c->err : "null context"; }

ns3d_status ns3d_initial_condition(ns3d_ctx* c, const char* name, uint64_t seed, double k0, double energy) {
    if (!c || !name) return NS3D_ERR_INVALID;
    return pass(c, ns3d::ic_dispatch(c->impl, c->p.N, name, seed, k0, energy));
}

ns3d_status ns3d_set_state_host(ns3d_ctx* c, const double* u) {
    if (!c || !u) return NS3D_ERR_INVALID;
    return pass(c, c->impl->set_state_host(u));
}

ns3d_status ns3d_get_state_host(ns3d_ctx* c, double* u) {
    if (!c || !u) return NS3D_ERR_INVALID;
    return pass(c, c->impl->get_state_host(u));
}

ns3d_status ns3d_step(ns3d_ctx* c, int nsteps) {
    if (!c || nsteps < 0) return NS3D_ERR_INVALID;
    return pass(c, c->impl->step(nsteps));
}

ns3d_status ns3d_step_host(ns3d_ctx* c, const double* in, double* out) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->step_host(in, out));
}

ns3d_status ns3d_rhs_host(ns3d_ctx* c, const double* in, double* out) {
    if (!c || !in || !out) return NS3D_ERR_INVALID;
    return pass(c, c->impl->rhs_host(in, out));
}

ns3d_status ns3d_dealias_host(int N, double* a, int dim) {
    if (!a || N <= 2 || (N % 2) || dim < 1) return NS3D_ERR_INVALID;
    const size_t bytes = sizeof(double2) * (size_t)N * N * (N / 2 + 1) * dim;
    double2* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return NS3D_ERR_NOMEM;
    cudaError_t e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        long long total = (long long)N * N * (N / 2 + 1);
        long long g = (total + 255) / 256;
        if (g > 4864) g = 4864;
        ns3d::k_dealias_ref_entry<<<(unsigned)g, 256>>>(d, N, dim);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(a, d, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? NS3D_OK : NS3D_ERR_CUDA;
}

ns3d_status ns3d_measurables(ns3d_ctx* c, ns3d_measures* m, double* Ek, double* Ok) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->measurables(m, Ek, Ok));
}

ns3d_status ns3d_real_space_host(ns3d_ctx* c, double* u, double* w) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->real_space_host(u, w));
}

ns3d_status ns3d_get_time(ns3d_ctx* c, double* t, double* dt, long* iters) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->get_time(t, dt, iters));
}

ns3d_status ns3d_set_time(ns3d_ctx* c, double t, double dt, long iters) {
    if (!c || !(dt > 0) || iters < 0) return NS3D_ERR_INVALID;
    return pass(c, c->impl->set_time(t, dt, iters));
}

ns3d_status ns3d_get_forcing_target(ns3d_ctx* c, double* e) {
    if (!c || !e) return NS3D_ERR_INVALID;
    return pass(c, c->impl->get_forcing_target(e));
}

ns3d_status ns3d_set_forcing_target(ns3d_ctx* c, double e) {
    if (!c || e < 0) return NS3D_ERR_INVALID;
    return pass(c, c->impl->set_forcing_target(e));
}

ns3d_status ns3d_set_dp_tolerances(ns3d_ctx* c, double atol, double rtol) {
    if (!c || !(atol > 0) || !(rtol >= 0)) return NS3D_ERR_INVALID;
    return pass(c, c->impl->set_dp_tolerances(atol, rtol));
}

ns3d_status ns3d_increment_stats(ns3d_ctx* c, const int* increments, int n_incr, int n_bins, double* stats,
                                 double* ranges, double* counts) {
    if (!c || !stats || n_bins < 1 || n_bins > 12288) return NS3D_ERR_INVALID;
    const int N = c->p.N;
    const int deflt[9] = {1, 2, 4, 8, 16, 32, 64, 128, N / 2};   // stats.c:411-413
    if (!increments) {
        increments = deflt;
        n_incr = 9;
    }
    if (n_incr < 1) return NS3D_ERR_INVALID;
    for (int r = 0; r < n_incr; ++r)
        if (increments[r] < 1) return NS3D_ERR_INVALID;
    return pass(c, c->impl->increment_stats(increments, n_incr, n_bins, stats, ranges, counts));
}

ns3d_status ns3d_io_bytes(ns3d_ctx* c, long long* h2d, long long* d2h) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->io_bytes(h2d, d2h));
}

ns3d_status ns3d_set_wait_budget(ns3d_ctx* c, long long cycles) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->set_wait_budget(cycles));
}

ns3d_status ns3d_dp_stats(ns3d_ctx* c, double* last_err, long* rejects) {
    if (!c) return NS3D_ERR_INVALID;
    return pass(c, c->impl->dp_stats(last_err, rejects));
}

ns3d_status ns3d_max_speed_sum(ns3d_ctx* c, double* umax) {
    if (!c || !umax) return NS3D_ERR_INVALID;
    return pass(c, c->impl->max_speed_sum(umax));
}

void* ns3d_stream(ns3d_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ns3d_kernels_per_step(ns3d_ctx* c) { return c ? c->impl->kernels_per_step() : 0; }

ns3d_status ns3d_last_step_ms(ns3d_ctx* c, float* ms) {
    if (!c || !ms) return NS3D_ERR_INVALID;
    return pass(c, c->impl->last_step_ms(ms));
}

ns3d_status ns3d_profile_step(ns3d_ctx* c, int reps, const char** names, float* ms, double* bytes, int maxc,
                              int* count) {
    if (!c || !names || !ms || !count || reps <= 0) return NS3D_ERR_INVALID;
    return pass(c, c->impl->profile(reps, names, ms, bytes, maxc, count));
}

}  // extern "C"
