// cnn.cuh — kernels of the learned subgrid closure: a 3D convolutional
// network on a periodic D^3 grid (3^3 kernels, GELU, circular padding),
// BF16 weights with FP32 accumulation, and its training kernels.
//
// Layout: activations [C][D][D][D] float (z fastest, like the solver's real
// fields); weights W[cout][cin][27] with tap k = (dx+1)*9 + (dy+1)*3 + (dz+1),
// i.e. torch's [cout][cin][3][3][3] for a cross-correlation.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns3d {
namespace cnn {

constexpr int TX = 8, TY = 8, TZ = 4;            // output tile per CTA (256 threads)
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int HALO = HX * HY * HZ;
constexpr int CCH = 8;                           // input channels staged per round

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// y[co][p] = epi( b[co] + sum_{ci,k} W[co][ci][k] * in(x[ci][p + off_k]) )
//   IN_GELU : in(v) = gelu(v)  (x holds the previous layer's pre-activation)
//   IN_SCALE: in(v) = v * in_scale
//   OUT_MUL : y = acc * gelu'(z[co][p])   (backward through the activation)
//   FLIP    : use taps mirrored (k -> 26-k) and weights transposed, i.e. the
//             gradient with respect to the input of a layer with weights w
template <int CIN, int COUT, bool IN_GELU, bool OUT_MUL, bool FLIP>
__global__ void __launch_bounds__(256)
k_conv3(const float* __restrict__ x, const __nv_bfloat16* __restrict__ w, const float* __restrict__ b,
        const float* __restrict__ z, float* __restrict__ y, int D, float in_scale, float out_scale) {
    __shared__ float sx[CCH][HALO];
    __shared__ __nv_bfloat16 sw[COUT][CCH][27];
    const int tx = threadIdx.x / (TY * TZ), ty = (threadIdx.x / TZ) % TY, tz = threadIdx.x % TZ;
    const int ntz = D / TZ, nty = D / TY;
    const int bz = blockIdx.x % ntz, by = (blockIdx.x / ntz) % nty, bx = blockIdx.x / (ntz * nty);
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * TZ;
    const long long D3 = (long long)D * D * D;
    float acc[COUT];
#pragma unroll
    for (int c = 0; c < COUT; ++c) acc[c] = b ? b[c] : 0.0f;
    for (int c0 = 0; c0 < CIN; c0 += CCH) {
        __syncthreads();
        for (int q = threadIdx.x; q < CCH * HALO; q += blockDim.x) {
            const int ci = c0 + q / HALO, h = q % HALO;
            float v = 0.0f;
            if (ci < CIN) {
                const int hx = h / (HY * HZ), hy = (h / HZ) % HY, hz = h % HZ;
                const int gx = (x0 + hx - 1 + D) % D, gy = (y0 + hy - 1 + D) % D, gz = (z0 + hz - 1 + D) % D;
                v = x[ci * D3 + ((long long)gx * D + gy) * D + gz];
                if (IN_GELU) v = gelu(v);
                v *= in_scale;
            }
            sx[q / HALO][h] = v;
        }
        for (int q = threadIdx.x; q < COUT * CCH * 27; q += blockDim.x) {
            const int co = q / (CCH * 27), ci = c0 + (q / 27) % CCH, k = q % 27;
            __nv_bfloat16 v = __float2bfloat16(0.0f);
            if (ci < CIN) v = FLIP ? w[((long long)ci * COUT + co) * 27 + (26 - k)] : w[((long long)co * CIN + ci) * 27 + k];
            sw[co][(q / 27) % CCH][k] = v;
        }
        __syncthreads();
#pragma unroll 1
        for (int cc = 0; cc < CCH; ++cc) {
            if (c0 + cc >= CIN) break;
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int dx = k / 9, dy = (k / 3) % 3, dz = k % 3;
                const float v = sx[cc][((tx + dx) * HY + (ty + dy)) * HZ + (tz + dz)];
#pragma unroll
                for (int c = 0; c < COUT; ++c) acc[c] = fmaf(v, __bfloat162float(sw[c][cc][k]), acc[c]);
            }
        }
    }
    const long long p = ((long long)(x0 + tx) * D + (y0 + ty)) * D + (z0 + tz);
#pragma unroll
    for (int c = 0; c < COUT; ++c) {
        float v = acc[c] * out_scale;
        if (OUT_MUL) v *= gelu_grad(z[c * D3 + p]);
        y[c * D3 + p] = v;
    }
}

// dW[co][ci][k] = sum_p g[co][p] * in(a[ci][p + off_k]),  db[co] = sum_p g[co][p]
// one CTA per (co, ci); fixed-order block reduction (deterministic)
template <bool IN_GELU>
__global__ void __launch_bounds__(256)
k_conv3_wgrad(const float* __restrict__ g, const float* __restrict__ a, float* __restrict__ dw, float* __restrict__ db,
              int CIN, int D, float in_scale) {
    __shared__ float red[256];
    const int co = blockIdx.x / CIN, ci = blockIdx.x % CIN;
    const long long D3 = (long long)D * D * D;
    float s[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) s[k] = 0.0f;
    float sb = 0.0f;
    for (long long p = threadIdx.x; p < D3; p += blockDim.x) {
        const int px = (int)(p / ((long long)D * D)), py = (int)((p / D) % D), pz = (int)(p % D);
        const float gv = g[co * D3 + p];
        sb += gv;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            const int gx = (px + k / 9 - 1 + D) % D, gy = (py + (k / 3) % 3 - 1 + D) % D, gz = (pz + k % 3 - 1 + D) % D;
            float v = a[ci * D3 + ((long long)gx * D + gy) * D + gz];
            if (IN_GELU) v = gelu(v);
            s[k] = fmaf(gv, v * in_scale, s[k]);
        }
    }
    for (int k = 0; k < 28; ++k) {
        red[threadIdx.x] = k < 27 ? s[k] : sb;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (k < 27) dw[((long long)co * CIN + ci) * 27 + k] = red[0];
            else if (ci == 0 && db) db[co] = red[0];
        }
        __syncthreads();
    }
}

// mean-squared-error gradient and per-CTA partial losses against the target
// t * tscale: g = 2 (y - t tscale) / n
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, float tscale, float* __restrict__ g,
                      long long n, double* __restrict__ part) {
    __shared__ double red[256];
    double s = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const float d = y[q] - t[q] * tscale;
        if (g) g[q] = 2.0f * d / (float)n;
        s += (double)d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// the loss of one sample: the k_mse partial sums in block order, / denom
__global__ void k_loss_store(const double* __restrict__ part, int nparts, double denom, double* __restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < nparts; ++i) s += part[i];
        *out = s / denom;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights, then their BF16 copy.
// No update once *halt is set, nor when this sample's loss is not finite or a
// bounded wait of its kernels gave up (*stat != 0): the first such sample sets
// *halt, so the weights stay those before it.
__global__ void k_adam(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, const double* __restrict__ loss, const int* __restrict__ stat,
                       int* __restrict__ halt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (*halt != 0 || !isfinite(*loss) || *stat != 0) {
        if (i == 0) *halt = 1;
        return;
    }
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16(w[i]);
}

}  // namespace cnn
}  // namespace ns3d
