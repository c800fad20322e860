// stats.cuh — longitudinal velocity-increment statistics of a real-space
// velocity field (the post-processing of PostProcessing/src/stats.c:22-254):
// for each increment r, the pooled samples
//     u_x(i + r, j, k) - u_x(i, j, k)   (i + r < N)
//     u_y(i, j + r, k) - u_y(i, j, k)   (j + r < N)
//     u_z(i, j, k + r) - u_z(i, j, k)   (k + r < N)
// (not periodic, as there), their moments and a histogram over
// [min - 0.05, max + 0.05] in nbins uniform bins (the reference's two passes:
// Precompute, then ComputeStats).
//
// Per increment three kernels over every point, each with per-CTA partials
// reduced in a fixed order (bit-reproducible): pass 0 count / sum / min /
// max, pass 1 the centred sums of powers 2, 3, 4; the histogram pass counts
// in shared memory with integer atomics (order-independent) and adds each
// CTA's counts to the global ones.
#pragma once
#include <cuda_runtime.h>
#include <float.h>

namespace ns3d {

constexpr int kIncrParts = 512;   // CTAs of the moment passes
constexpr int kIncrThreads = 256;

// the increment of component a at point q (x slowest), or false outside the box
template <typename T, int N>
__device__ __forceinline__ bool incr_at(const T* __restrict__ R, long long q, int a, int dr, double& d) {
    constexpr long long M = (long long)N * N * N;
    const int c = a == 0 ? (int)(q / ((long long)N * N)) : a == 1 ? (int)((q / N) % N) : (int)(q % N);
    if (c + dr >= N) return false;
    const long long st = a == 0 ? (long long)N * N : a == 1 ? N : 1;
    d = (double)R[a * M + q + dr * st] - (double)R[a * M + q];
    return true;
}

// pass 0: part[cta][4] = (count, sum, min, max); pass 1: part[cta][4] =
// (sum e^2, sum e^3, sum e^4, 0), e = d - mean. R: u as [3][N^3].
template <typename T, int N>
__global__ void __launch_bounds__(kIncrThreads)
k_incr_moments(const T* __restrict__ R, int dr, int pass, const double* __restrict__ mean, double* __restrict__ part) {
    constexpr long long M = (long long)N * N * N;
    __shared__ double red[4][kIncrThreads];
    double acc[4] = {0.0, 0.0, pass == 0 ? DBL_MAX : 0.0, pass == 0 ? -DBL_MAX : 0.0};
    const double mu = pass == 1 ? *mean : 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M; q += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            double d;
            if (!incr_at<T, N>(R, q, a, dr, d)) continue;
            if (pass == 0) {
                acc[0] += 1.0;
                acc[1] += d;
                acc[2] = fmin(acc[2], d);
                acc[3] = fmax(acc[3], d);
            } else {
                const double e = d - mu, e2 = e * e;
                acc[0] += e2;
                acc[1] += e2 * e;
                acc[2] += e2 * e2;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) red[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = kIncrThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const int t = threadIdx.x;
            red[0][t] += red[0][t + o];
            red[1][t] += red[1][t + o];
            if (pass == 0) {
                red[2][t] = fmin(red[2][t], red[2][t + o]);
                red[3][t] = fmax(red[3][t], red[3][t + o]);
            } else {
                red[2][t] += red[2][t + o];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 4) part[(long long)blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// sum the CTA partials in CTA order: out[4] (one thread per component)
template <int Unused = 0>
__global__ void k_incr_reduce(const double* __restrict__ part, int nparts, int pass, double* __restrict__ out) {
    const int c = threadIdx.x;
    if (c >= 4) return;
    double v = (pass == 0 && c == 2) ? DBL_MAX : (pass == 0 && c == 3) ? -DBL_MAX : 0.0;
    for (int b = 0; b < nparts; ++b) {
        const double x = part[(long long)b * 4 + c];
        v = (pass == 0 && c == 2) ? fmin(v, x) : (pass == 0 && c == 3) ? fmax(v, x) : v + x;
    }
    out[c] = v;
}

// edge b of nbins uniform bins over [lo, hi]: ((nbins - b) / nbins) lo + (b / nbins) hi,
// GSL's uniform-range rule (exact at both ends), which the reference's
// gsl_histogram_set_ranges_uniform uses
__host__ __device__ inline double incr_edge(double lo, double hi, int b, int nbins) {
    return ((double)(nbins - b) / (double)nbins) * lo + ((double)b / (double)nbins) * hi;
}

// histogram over those edges: bin b holds edge[b] <= d < edge[b + 1] (the
// binary-search rule of a range array)
template <typename T, int N>
__global__ void __launch_bounds__(kIncrThreads)
k_incr_hist(const T* __restrict__ R, int dr, const double* __restrict__ lohi, int nbins,
            unsigned long long* __restrict__ counts) {
    constexpr long long M = (long long)N * N * N;
    extern __shared__ unsigned int hist[];   // [nbins]
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    const double xl = lohi[0], xh = lohi[1], scale = (double)nbins / (xh - xl);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M; q += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            double d;
            if (!incr_at<T, N>(R, q, a, dr, d)) continue;
            int b = (int)((d - xl) * scale);   // first guess; the edge tests below decide
            b = b < 0 ? 0 : (b >= nbins ? nbins - 1 : b);
            while (b > 0 && d < incr_edge(xl, xh, b, nbins)) --b;
            while (b < nbins - 1 && d >= incr_edge(xl, xh, b + 1, nbins)) ++b;
            atomicAdd(&hist[b], 1u);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
        if (hist[b]) atomicAdd(&counts[b], (unsigned long long)hist[b]);
}

}  // namespace ns3d
