// ns3d_base.h — type-erased engine interface behind the C ABI. One concrete
// engine exists per (precision, grid size); see ns3d_impl.cuh.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/ns3d.h"

namespace ns3d {

// The learned subgrid closure as seen by an engine: tau[6][N^3] from the
// real-space velocity u[3][N^3], enqueued on stream s (FP32 device arrays).
struct LesHook {
    virtual ~LesHook() {}
    virtual void forward(const float* u, float* tau, int N, cudaStream_t s) = 0;
    // device word that the closure's kernels set to a non-zero status on failure
    virtual int* status_word() = 0;
};

class Base {
  public:
    Base(const ns3d_params& p, cudaStream_t s) : p_(p), s_(s) { err_[0] = 0; }
    virtual ~Base() {}
    virtual ns3d_status init() = 0;
    virtual int kernels_per_step() const = 0;
    virtual ns3d_status step(int nsteps) = 0;
    virtual ns3d_status step_host(const double* in, double* out) = 0;
    virtual ns3d_status last_step_ms(float* ms) = 0;
    virtual ns3d_status profile(int reps, const char** names, float* ms, double* bytes, int maxc, int* count) = 0;
    virtual ns3d_status rhs_host(const double* in, double* out) = 0;
    virtual ns3d_status set_state_host(const double* u) = 0;
    virtual ns3d_status get_state_host(double* u) = 0;
    virtual ns3d_status measurables(ns3d_measures* m, double* Ek, double* Ok) = 0;
    virtual ns3d_status ic_real(int kind) = 0;
    virtual ns3d_status ic_spectrum(uint64_t seed, double k0, double energy) = 0;
    virtual ns3d_status ic_host(const double* u) = 0;
    virtual ns3d_status ic_zero() = 0;
    virtual ns3d_status real_space_host(double* u, double* w) = 0;
    virtual ns3d_status max_speed_sum(double* umax) = 0;
    virtual ns3d_status get_time(double* t, double* dt, long* iters) = 0;
    virtual ns3d_status set_time(double t, double dt, long iters) = 0;
    virtual ns3d_status get_forcing_target(double* e) = 0;
    virtual ns3d_status set_forcing_target(double e) = 0;
    virtual ns3d_status set_dp_tolerances(double atol, double rtol) = 0;
    virtual ns3d_status dp_stats(double* err, long* rejects) = 0;
    // clock-cycle budget of the z pass's bounded waits (<= 0: the default)
    virtual ns3d_status set_wait_budget(long long cycles) = 0;
    virtual ns3d_status io_bytes(long long* h2d, long long* d2h) = 0;
    virtual ns3d_status increment_stats(const int* incr, int nr, int nbins, double* stats, double* ranges,
                                        double* counts) = 0;
    virtual void* state_ptr() = 0;
    // ensembles: number of members, selection of the member that single-run
    // calls act on, enqueueing one step of every member on the engine's
    // stream (for graph capture), and the health check of all members
    virtual int members() const = 0;
    virtual ns3d_status select(int m) = 0;
    virtual void enqueue_step() = 0;
    virtual ns3d_status status() = 0;
    // learned closure: attach (NULL detaches), step counters, the real-space
    // velocity for filtering, r2c of a host real-layout velocity
    virtual ns3d_status attach_les(LesHook* h) = 0;
    virtual ns3d_status les_counters(long* on, long* off) = 0;
    virtual const float* real_velocity_f32(ns3d_status* st) = 0;
    virtual ns3d_status set_state_real_host(const double* u) = 0;
    // z-pass form: 0 the persistent line kernel where compiled, 1 the CTA-synchronous pass,
    // 2 the tensor-core GEMMs where compiled
    virtual void set_zform(int z) = 0;
    virtual int zform() const = 0;
    virtual int variant() const = 0;

    const char* err() const { return err_; }
    void set_err(const char* fmt, ...) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err_, sizeof(err_), fmt, ap);
        va_end(ap);
    }
    cudaStream_t stream() const { return s_; }

  protected:
    ns3d_params p_;
    cudaStream_t s_;
    char err_[512];
};

// Factories, one per precision (ns3d_tune.cu): an engine for M members of
// grid size N with parameters ps[0..M-1], built with the tile variant and
// z-pass form the tuning table holds for (N, precision).
Base* make_f32(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f64(int N, const ns3d_params* ps, int M, cudaStream_t s);
// one compiled tile variant (nullptr where that variant is not compiled for N)
Base* make_f32_v0(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v1(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v2(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v3(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v4(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v5(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v3_large(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f64_large(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v6(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f64_v0(int N, const ns3d_params* ps, int M, cudaStream_t s);
bool supported_n(int N);
// z-pass form 2 (tensor-core GEMMs, zgemm.cuh) exists for FP32 and N in {16, 32, 48, 64, 96, 128}
inline bool zgemm_size(int N, int precision) {
    return precision == NS3D_FP32 && N >= 16 && N <= 128 && N % 16 == 0;
}
constexpr int kTileVariants = 7;   // TileVar<0..6>, PlansV (ns3d_kernels.cuh)

inline unsigned long long host_splitmix64(unsigned long long x) {
    unsigned long long z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace ns3d
