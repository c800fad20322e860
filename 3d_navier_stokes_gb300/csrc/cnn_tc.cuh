// cnn_tc.cuh — inference of the closure network on the 5th-generation tensor
// cores. A 3^3 convolution
//     out[p][co] = b[co] + sum_{dx,dy,dz} sum_ci in[p + (dx,dy,dz)][ci] W[co][ci][dx,dy,dz]
// is computed as nine GEMMs over the (dx, dy) taps whose N dimension holds the
// three dz taps side by side:
//     G[q][dz*NO + co] = sum_{dx,dy} sum_ci in[q + (dx,dy,0)][ci] W[co][ci][dx,dy,dz]
//     out[p][co] = G[p - 1z][0*NO + co] + G[p][1*NO + co] + G[p + 1z][2*NO + co]
// M = 128 grid points per tile (R = 128/D whole z-lines at one x, D in
// {16, 32, 64}), so the z neighbours of every row, periodic wrap included,
// are rows of the same tile; N = 3 NO (96 for the 32-channel layers, 48 for
// the 6-channel output padded to 16); K = the input channels, 16 per
// tcgen05.mma kind::f16 (BF16 operands from shared memory, FP32 accumulator in
// tensor memory), 9 x CIN/16 MMAs per tile issued by one thread.
//
// Shared-memory operand layout (SWIZZLE_NONE, K-major canonical form): a
// "core matrix" is 8 rows x 16 bytes (8 rows of 8 BF16 channels), stored
// contiguously; the KC core matrices of one 8-row group (the K direction)
// are adjacent, so the descriptor's leading byte offset (K step) is 128 bytes
// and its stride byte offset (next 8 rows) is KC * 128 bytes.
//   A: [x plane 3][y row R+2][z group D/8][kchunk KC][8 points][16 B]  (x2, double buffered)
//   B: [(dx,dy) 9][n group 3 NO/8][kchunk KC][8 (dz, co)][16 B]
// Activations between layers are BF16 in the blocked layout
// [x][y][z group][kchunk][8 points][8 channels], so every (x, y) line of the
// halo block is one contiguous run identical to its place in A: one thread
// stages a tile with 3 (R+2) cp.async.bulk copies completed on an mbarrier.
// The copies for tile i+2 are issued as soon as the MMAs of tile i have
// released its buffer, and the MMAs of tile i+1 before the epilogue of tile i
// (tensor memory -> registers, the dz combination through a shared exchange
// of the dz = -1 and +1 blocks, bias, GELU), which the other warps run while
// the tensor cores work; two accumulators live in tensor memory. Layers
// write GELU(z) in the blocked layout; k_to_blocked converts the FP32
// velocity [3][D^3] (x in_scale) into the blocked form of layer 1, and the
// output layer writes FP32 [6][D^3] (x out_scale). Every wait is bounded; on
// a timeout the kernel records kStatusTimeout in *status, waits once more
// (bounded) for its own copies and MMAs, frees its tensor memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tcgen05.cuh"
#include "tma.cuh"

namespace ns3d {
namespace cnn {

using tc::idesc_bf16;
using tc::idesc_bf16_mn;
using tc::mma_bf16;
using tc::mma_commit;
using tc::pack_bf16x2;
using tc::smem_desc;
using tc::tc_fence_after;
using tc::tc_fence_before;
using tc::tmem_alloc;
using tc::tmem_dealloc;
using tc::tmem_ld16;
using tc::tmem_ld8;
using tc::tmem_relinquish;
using tc::tmem_wait_ld;

__device__ __forceinline__ float gelu_tc(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_tc(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    return cdf + x * 0.39894228040143268f * __expf(-0.5f * x * x);
}

constexpr int kTcTmemCols = 256;   // two accumulators of up to 96 columns, at 0 and 128

__host__ __device__ constexpr bool tc_grid_ok(int D) { return D == 16 || D == 32 || D == 64; }
__host__ __device__ constexpr uint32_t tc_a_bytes(int KC, int D) {
    return 3u * (uint32_t)(128 / D + 2) * (uint32_t)D * (uint32_t)KC * 16u;
}
__host__ __device__ constexpr uint32_t tc_b_bytes(int KC, int NO) { return 9u * 3u * (uint32_t)NO * (uint32_t)KC * 16u; }
__host__ __device__ constexpr uint32_t tc_x_bytes(int NO) { return 2u * (uint32_t)NO * 128u * 4u; }
__host__ __device__ constexpr uint32_t tc_smem_bytes(int KC, int NO, int D) {
    return tc_b_bytes(KC, NO) + 2u * tc_a_bytes(KC, D) + tc_x_bytes(NO) + 64u;
}

// blocked activation index (in 16-byte units) of point (x, y, z), chunk kc
template <int LOGD, int KC>
__device__ __forceinline__ long long blk_index(int x, int y, int z, int kc) {
    constexpr int ZG = (1 << LOGD) / 8;
    return (((((long long)x << LOGD) + y) * ZG + (z >> 3)) * KC + kc) * 8 + (z & 7);
}

// Operand copies of the weight-gradient kernel, in 16-byte units (8 BF16
// channels of one point). wg-A [x][y][c/8][z]: the NC channels of one (x, y)
// line are NC/8 runs of D points. wg-B [x][y][j][c/8][r]: three copies of
// that, copy j holding the line shifted by dz = j - 1, row r = d[r + 1 - j]
// (periodic in z), so that one operand of 3 NC rows covers the three dz taps.
template <int LOGD, int NC>
__device__ __forceinline__ long long wga_index(int x, int y, int c8, int z) {
    return ((((long long)x << LOGD) + y) * (NC / 8) + c8) * (1 << LOGD) + z;
}
template <int LOGD, int NC>
__device__ __forceinline__ long long wgb_index(int x, int y, int j, int c8, int r) {
    return (((((long long)x << LOGD) + y) * 3 + j) * (NC / 8) + c8) * (1 << LOGD) + r;
}
// point z's 8 channels c8 into the three copies (rows z - 1, z, z + 1)
template <int LOGD, int NC>
__device__ __forceinline__ void wgb_store(uint4* dst, int x, int y, int c8, int z, uint4 v) {
    constexpr int D = 1 << LOGD;
#pragma unroll
    for (int j = 0; j < 3; ++j) dst[wgb_index<LOGD, NC>(x, y, j, c8, (z - 1 + j) & (D - 1))] = v;
}

// FP32 velocity [3][D^3] x in_scale -> blocked BF16 with 16 channels (KC = 2)
template <int LOGD>
__global__ void k_to_blocked(const float* __restrict__ u, float in_scale, uint4* __restrict__ dst) {
    constexpr int D = 1 << LOGD;
    constexpr long long D3 = (long long)D * D * D;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < D3; p += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(p & (D - 1)), y = (int)((p >> LOGD) & (D - 1)), x = (int)(p >> (2 * LOGD));
        uint4 v;
        v.x = pack_bf16x2(u[p] * in_scale, u[D3 + p] * in_scale);
        v.y = pack_bf16x2(u[2 * D3 + p] * in_scale, 0.0f);
        v.z = 0u;
        v.w = 0u;
        dst[blk_index<LOGD, 2>(x, y, z, 0)] = v;
        dst[blk_index<LOGD, 2>(x, y, z, 1)] = make_uint4(0u, 0u, 0u, 0u);
    }
}


// One layer. KC: 16-byte channel chunks of the input (CIN padded to 8 KC);
// NO: output channels per dz block (32, or 16 for the output layer);
// D = 1 << LOGD; input BF16 blocked with KC chunks; OUT_MODE 0: GELU(out + b)
// as BF16 blocked with 4 chunks, 1: (out + b) * out_scale as FP32
// [cout][D^3]; training: 2: z = out + b to zbuf (FP32 [32][D^3]) and
// a = GELU(z) blocked and as the wg-A copy (cm) of the weight-gradient kernel;
// 3 (the input gradient, weights packed transposed and mirrored by
// k_pack_jobs with transposed = 1, no bias): d = out * GELU'(zbuf) blocked and as the wg-B copies
// (cm). Warp-specialised, 17 warps: lane 0 of warp 16 (the producer) issues the
// copies and the MMAs; warps 0..15 (the epilogue) each take tensor-memory lane
// quarter w % 4 and output channels [8 (w / 4), 8 (w / 4) + 8). Handoffs run on
// mbarriers only: full[b] (the copies of A buffer b landed), done[b] (the MMAs
// into accumulator b completed, also freeing A buffer b), aempty[b] (the 16
// epilogue warps have read accumulator b); the epilogue warps synchronise among
// themselves on a named barrier, so the producer keeps the MMAs of tile i + 1
// running while tile i's epilogue runs.
constexpr int kConvWarps = 16;                        // epilogue warps
constexpr int kConvThreads = 32 * (kConvWarps + 1);   // and the producer warp
constexpr int kTcThreads = 256;                       // the weight-gradient kernel

// the epilogue warps' named barrier 1 (512 threads), and the same with an AND
// of a predicate across them
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * kConvWarps) : "memory"); }
__device__ __forceinline__ bool epi_sync_and(bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, 1, %2, q;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(32 * kConvWarps)
        : "memory");
    return r != 0;
}

template <int KC, int NO, int LOGD, int OUT_MODE>
__global__ void __launch_bounds__(kConvThreads, 1)
k_conv3_tc(const uint4* __restrict__ in, const uint4* __restrict__ wpk, const float* __restrict__ bias,
           void* __restrict__ out, int cout, float out_scale, int* __restrict__ status,
           float* __restrict__ zbuf = nullptr, __nv_bfloat16* __restrict__ cm = nullptr) {
    static_assert(KC % 2 == 0 && (NO == 16 || NO == 32), "tile shape");
    static_assert(OUT_MODE < 2 || NO == 32, "the training modes write 32 channels");
    constexpr int D = 1 << LOGD, R = 128 / D, rows = R + 2, ZG = D / 8, NB = 3 * NO;
    static_assert(R >= 1 && R <= D, "grid size");
    constexpr uint32_t b_bytes = tc_b_bytes(KC, NO), a_bytes = tc_a_bytes(KC, D);
    constexpr uint32_t line_bytes = (uint32_t)D * KC * 16;   // one (x, y) line of the blocked input
    constexpr long long D3 = (long long)D * D * D;
    constexpr int tiles_per_x = D / R, ntiles = D * tiles_per_x;
    constexpr uint32_t idesc = idesc_bf16(128, NB);
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sB = smem;
    unsigned char* sA = smem + b_bytes;                                        // two buffers
    float* sX = reinterpret_cast<float*>(sA + 2 * a_bytes);                    // [2][NO][128]
    uint64_t* done = reinterpret_cast<uint64_t*>(sA + 2 * a_bytes + tc_x_bytes(NO));   // MMAs into accumulator b done
    uint64_t* full = done + 2;                                                 // copies into buffer b landed
    uint64_t* aempty = full + 2;                                               // accumulator b read by the epilogue
    uint32_t* holder = reinterpret_cast<uint32_t*>(aempty + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int first = blockIdx.x, stride = gridDim.x;
    const int nmine = first < ntiles ? (ntiles - first + stride - 1) / stride : 0;

    for (uint32_t q = tid; q < b_bytes / 16; q += kConvThreads) reinterpret_cast<uint4*>(sB)[q] = wpk[q];
    fence_proxy_async_smem();   // B (generic stores) -> visible to the tensor cores
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&done[b], 1);
            mbar_init(&full[b], 1);
            mbar_init(&aempty[b], kConvWarps);
        }
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(holder, kTcTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *holder;

    if (warp == kConvWarps) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            const uint32_t sA_u = smem_u32(sA), sB_u = smem_u32(sB);
            uint32_t ph_full = 0u, ph_done = 0u, ph_empty = 0u;   // bit b: parity of the next completion
            uint32_t pend_copy = 0u, pend_mma = 0u;               // bit b: in flight
            bool ok = true;
            // the halo block of tile t into buffer b: 3 (R+2) line copies
            auto load = [&](int t, int b) {
                const int x = t / tiles_per_x, y0 = (t % tiles_per_x) * R;
                mbar_arrive_expect_tx(&full[b], a_bytes);
#pragma unroll 1
                for (int l = 0; l < 3 * rows; ++l) {
                    const int xp = l / rows, yr = l % rows;
                    const int gx = (x + xp - 1) & (D - 1), gy = (y0 + yr - 1) & (D - 1);
                    bulk_g2s(sA + b * a_bytes + l * line_bytes, in + (((long long)gx << LOGD) + gy) * (D * KC),
                             line_bytes, &full[b]);
                }
                pend_copy |= 1u << b;
            };
            if (nmine > 0) load(first, 0);
            if (nmine > 1) load(first + stride, 1);
#pragma unroll 1
            for (int i = 0; i < nmine; ++i) {
                const int b = i & 1;
                ok = mbar_wait(&full[b], (ph_full >> b) & 1u);
                if (!ok) break;
                ph_full ^= 1u << b;
                pend_copy &= ~(1u << b);
                if (i >= 2) {   // the epilogue of tile i - 2 has read accumulator b
                    ok = mbar_wait(&aempty[b], (ph_empty >> b) & 1u);
                    if (!ok) break;
                    ph_empty ^= 1u << b;
                }
                tc_fence_after();
                const uint32_t a_base = sA_u + b * a_bytes, d = tmem + 128u * b;
                uint32_t acc = 0;
#pragma unroll 1
                for (int t9 = 0; t9 < 9; ++t9) {
                    const int dx = t9 / 3, dy = t9 % 3;   // offsets + 1
                    const uint32_t a0 = a_base + ((dx * rows + dy) * ZG) * KC * 128;
                    const uint32_t b0 = sB_u + (uint32_t)(t9 * (NB / 8) * KC) * 128;
#pragma unroll
                    for (int ks = 0; ks < KC / 2; ++ks) {
                        mma_bf16(d, smem_desc(a0 + ks * 256, 128, KC * 128), smem_desc(b0 + ks * 256, 128, KC * 128),
                                 idesc, acc);
                        acc = 1;
                    }
                }
                mma_commit(&done[b]);
                pend_mma |= 1u << b;
                // those MMAs read A buffer b: refill it with tile i + 2 once they are done
                // (refilling the other buffer with tile i + 1 right after issuing these
                // instead measured slower: its copies then land too late)
                if (i + 2 < nmine) {
                    ok = mbar_wait(&done[b], (ph_done >> b) & 1u);
                    if (!ok) break;
                    ph_done ^= 1u << b;
                    pend_mma &= ~(1u << b);
                    load(first + (i + 2) * stride, b);
                }
            }
            if (!ok) atomicExch(status, kStatusTimeout);
            // the copies and MMAs still in flight complete before the CTA exits
            for (int b = 0; b < 2; ++b) {
                if (pend_copy & (1u << b)) (void)mbar_wait(&full[b], (ph_full >> b) & 1u);
                if (pend_mma & (1u << b)) (void)mbar_wait(&done[b], (ph_done >> b) & 1u);
            }
        }
    } else {
        // ------------------------------------------------------------ epilogue warps
        const int quarter = warp & 3, part = warp >> 2;   // lane quarter, 8-channel group
        const int m = quarter * 32 + lane;
        const bool active = (NO == 32) || part < 2;
        float bv[8];   // this thread's 8 biases, once
#pragma unroll
        for (int j = 0; j < 8; ++j) bv[j] = bias[8 * part + j < cout ? 8 * part + j : 0];
        uint32_t ph_done = 0u;
#pragma unroll 1
        for (int i = 0; i < nmine; ++i) {
            const int b = i & 1, tile = first + i * stride;
            // tile i's MMAs are done (every epilogue thread waits; all agree on the
            // outcome); this barrier also ends every read of sX for tile i - 1
            const bool got = mbar_wait(&done[b], (ph_done >> b) & 1u);
            if (!epi_sync_and(got)) {
                if (tid == 0) atomicExch(status, kStatusTimeout);
                break;
            }
            ph_done ^= 1u << b;
            tc_fence_after();
            const int x = tile / tiles_per_x, y0 = (tile % tiles_per_x) * R;
            const uint32_t tl = tmem + 128u * b + ((uint32_t)(quarter * 32) << 16) + 8u * part;
            uint32_t gm[8], g0[8], gp[8];
            if (active) {
                tmem_ld8(tl, gm);
                tmem_ld8(tl + NO, g0);
                tmem_ld8(tl + 2 * NO, gp);
                tmem_wait_ld(gm);
                tmem_wait_ld(g0);
                tmem_wait_ld(gp);
            }
            // accumulator b may be overwritten (the MMAs of tile i + 2)
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&aempty[b]);
            if (active) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    sX[(8 * part + j) * 128 + m] = __uint_as_float(gm[j]);
                    sX[(NO + 8 * part + j) * 128 + m] = __uint_as_float(gp[j]);
                }
            }
            epi_sync();
            if (active) {
                const int line = m & ~(D - 1), zz = m & (D - 1), yy = y0 + (m >> LOGD);
                const int left = line | ((zz - 1) & (D - 1)), right = line | ((zz + 1) & (D - 1));
                float v[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int co = 8 * part + j;
                    v[j] = sX[co * 128 + left] + __uint_as_float(g0[j]) + sX[(NO + co) * 128 + right] + bv[j];
                }
                if constexpr (OUT_MODE == 0) {
                    uint4* dst = reinterpret_cast<uint4*>(out);
                    dst[blk_index<LOGD, 4>(x, yy, zz, part)] =
                        make_uint4(pack_bf16x2(gelu_tc(v[0]), gelu_tc(v[1])), pack_bf16x2(gelu_tc(v[2]), gelu_tc(v[3])),
                                   pack_bf16x2(gelu_tc(v[4]), gelu_tc(v[5])), pack_bf16x2(gelu_tc(v[6]), gelu_tc(v[7])));
                } else if constexpr (OUT_MODE == 2 || OUT_MODE == 3) {
                    const long long p = ((((long long)x << LOGD) + yy) << LOGD) | zz;
                    float o[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const long long qi = (long long)(8 * part + j) * D3 + p;
                        if constexpr (OUT_MODE == 2) {
                            zbuf[qi] = v[j];
                            o[j] = gelu_tc(v[j]);
                        } else {
                            o[j] = v[j] * gelu_grad_tc(zbuf[qi]);
                        }
                    }
                    uint4* dst = reinterpret_cast<uint4*>(out);
                    uint4* wg = reinterpret_cast<uint4*>(cm);
                    const uint4 pk = make_uint4(pack_bf16x2(o[0], o[1]), pack_bf16x2(o[2], o[3]), pack_bf16x2(o[4], o[5]),
                                                pack_bf16x2(o[6], o[7]));
                    dst[blk_index<LOGD, 4>(x, yy, zz, part)] = pk;
                    if constexpr (OUT_MODE == 2)
                        wg[wga_index<LOGD, 32>(x, yy, part, zz)] = pk;
                    else
                        wgb_store<LOGD, 32>(wg, x, yy, part, zz, pk);
                } else {
                    float* dst = reinterpret_cast<float*>(out);
                    const long long p = ((((long long)x << LOGD) + yy) << LOGD) | zz;
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (8 * part + j < cout) dst[(8 * part + j) * D3 + p] = v[j] * out_scale;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTcTmemCols);
}

// ------------------------------------------------------------------ training
// Tensor-core training of the network (BF16 operands, FP32 accumulation,
// FP32 master weights and Adam outside). Notation for layer L: z_L = conv(a_{L-1},
// W_L) + b_L, a_L = GELU(z_L) (L = 1..3), y = z_4; the loss gradient
// d_4 = dloss/dy, d_L = conv^T(d_{L+1}, W_{L+1}) * GELU'(z_L),
// dW_L[co][ci][t] = sum_p d_L[co][p] a_{L-1}[ci][p + off_t], db_L = sum_p d_L.
// The forward convolutions (OUT_MODE 2) and the input gradients (OUT_MODE 3,
// a convolution with the weights transposed and mirrored) run on k_conv3_tc;
// the weight and bias gradients on k_wgrad_tc, whose operands are the wg-A
// copies of the activations and the wg-B copies of the gradients that those
// kernels also write.


// B operands of the layers from W[cout][cin][27] (BF16), several in one launch
// (job blockIdx.y), in the shared-memory order [(dx,dy) 9][n group][kchunk][8 n][8
// channels], n = dz * NO + output channel, zero padding to NO output and 8 KC input
// channels. transposed = 0: the layer's own kernel, output channels co, input
// channels ci; transposed = 1: the B operand of its input-gradient convolution,
// the kernel transposed and mirrored, W'[ci][co][t] = W[co][ci][26 - t] (input
// channels co in KC chunks, output channels ci < NO).
struct PackJob {
    const __nv_bfloat16* w;
    __nv_bfloat16* dst;
    int cout, cin, KC, NO, transposed;
};
struct PackJobs {
    PackJob job[8];
};
__global__ void k_pack_jobs(const PackJobs jobs) {
    const PackJob J = jobs.job[blockIdx.y];
    const int NG = 3 * J.NO / 8;
    const int n_all = 9 * NG * J.KC * 64;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n_all; q += gridDim.x * blockDim.x) {
        const int j = q % 8;
        int r = q / 8;
        const int n8 = r % 8;
        r /= 8;
        const int kc = r % J.KC;
        r /= J.KC;
        const int ng = r % NG;
        const int t9 = r / NG;
        const int n = ng * 8 + n8, dz = n / J.NO, a = n % J.NO, b = kc * 8 + j;
        const int t = t9 * 3 + dz;
        if (J.transposed)
            J.dst[q] = (a < J.cin && b < J.cout) ? J.w[((long long)b * J.cin + a) * 27 + (26 - t)] : __float2bfloat16(0.0f);
        else
            J.dst[q] = (a < J.cout && b < J.cin) ? J.w[((long long)a * J.cin + b) * 27 + t] : __float2bfloat16(0.0f);
    }
}

// per-channel sums of an FP32 [nch][n] array in two fixed-order levels:
// partial[c][blockIdx.x] over a strided share, then the partials in order
__global__ void k_chan_partial(const float* __restrict__ x, long long n, float* __restrict__ partial) {
    __shared__ float red[256];
    const int c = blockIdx.y;
    const float* xc = x + (long long)c * n;
    float s = 0.0f;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        s += xc[p];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = red[0];
}
__global__ void k_chan_final(const float* __restrict__ partial, int nparts, int nch, float* __restrict__ out) {
    const int c = threadIdx.x;
    if (c >= nch) return;
    float s = 0.0f;
    for (int q = 0; q < nparts; ++q) s += partial[c * nparts + q];
    out[c] = s;
}

// FP32 velocity [3][D^3] x in_scale -> wg-A BF16 with 8 channels (3..7 zero);
// with one run per line the wg-A index of point p is p
template <int LOGD>
__global__ void k_to_wga(const float* __restrict__ u, float in_scale, uint4* __restrict__ dst) {
    constexpr long long D3 = 1ll << (3 * LOGD);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < D3; p += (long long)gridDim.x * blockDim.x)
        dst[p] = make_uint4(pack_bf16x2(u[p] * in_scale, u[D3 + p] * in_scale), pack_bf16x2(u[2 * D3 + p] * in_scale, 0.0f),
                            0u, 0u);
}

// the output gradient d_4 (FP32 [6][D^3]) -> blocked BF16 with 2 chunks (16
// channels, 6 used) and its wg-B copies (channels 6..15 zero)
template <int LOGD>
__global__ void k_grad_pack(const float* __restrict__ g, uint4* __restrict__ blk, uint4* __restrict__ wg) {
    constexpr int D = 1 << LOGD;
    constexpr long long D3 = (long long)D * D * D;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < D3; p += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(p & (D - 1)), y = (int)((p >> LOGD) & (D - 1)), x = (int)(p >> (2 * LOGD));
        float v[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = c < 6 ? g[c * D3 + p] : 0.0f;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint4 pk =
                make_uint4(pack_bf16x2(v[q * 8 + 0], v[q * 8 + 1]), pack_bf16x2(v[q * 8 + 2], v[q * 8 + 3]),
                           pack_bf16x2(v[q * 8 + 4], v[q * 8 + 5]), pack_bf16x2(v[q * 8 + 6], v[q * 8 + 7]));
            blk[blk_index<LOGD, 2>(x, y, z, q)] = pk;
            wgb_store<LOGD, 16>(wg, x, y, q, z, pk);
        }
    }
}


__host__ __device__ constexpr int tc_pow2(int v) {
    int p = 32;
    while (p < v) p <<= 1;
    return p;
}
// byte offset of the 16-byte chunk (row r, K elements 8 k8 ..) of a canonical K-major operand with K columns
__host__ __device__ constexpr uint32_t tc_chunk(int r, int k8, int K) {
    return (uint32_t)(((r >> 3) * (K >> 3) + k8) * 128 + (r & 7) * 16);
}

// Weight gradient on the tensor cores. For one z line (x, y) of D points, the
// GEMM D[(t, ci)][(j, co)] += sum_z a[ci][x + dx_t][y + dy_t][z] d[co][x][y][z - (j - 1)]
// accumulates dW[co][ci][(t, j)] (t = the (dx, dy) tap, j = dz + 1). M = 128
// rows: TG = 128 / CI taps of CI channels per tap group, NGRP = ceil(9 / TG)
// groups; N = 3 NB: the three dz copies of the NB output channels; K = the D
// points of the line. Both operands are MN-major (8 channels of one point per
// 16-byte row, the K rows of a run 16 bytes apart): A is the nine tap lines of
// the wg-A copy, one bulk copy each, placed so that the 8-row groups of a tap
// group are SBO = 16 D bytes apart; B is the wg-B line, one bulk copy. A
// padding row of the last tap group holds ones, so its j = 1 columns sum to
// the bias gradient sum_p d[co][p]. Persistent CTAs walk the D^2 lines; thread
// 0 keeps NST stages of copies in flight and issues the MMAs (bounded waits);
// each CTA writes its FP32 partial sums [group][128][3 NB] to part, reduced in
// a fixed order by k_wgrad_reduce.
template <int CI, int NB, int LOGD>
struct WgGeo {
    static constexpr int D = 1 << LOGD, TG = 128 / CI, NGRP = (9 + TG - 1) / TG, NN = 3 * NB;
    static constexpr uint32_t TAP_BYTES = (uint32_t)CI * D * 2;       // one wg-A line
    static constexpr uint32_t A_BYTES = 128u * D * 2;                 // one tap group
    static constexpr uint32_t B_BYTES = 3u * NB * D * 2;              // one wg-B line
    // the last group holds its taps and the ones slot; the rows of its unused slots are
    // read from whatever follows (the B line, discarded rows), as long as the stage holds
    // the group's full 128 rows
    static constexpr uint32_t LAST_SLOTS = 9 - (NGRP - 1) * TG + 1;
    static constexpr uint32_t A_REGION = (NGRP - 1) * A_BYTES + LAST_SLOTS * TAP_BYTES;
    static constexpr uint32_t STAGE =
        A_REGION + B_BYTES > NGRP * A_BYTES ? A_REGION + B_BYTES : NGRP * A_BYTES;
    static constexpr int NST = 225280u / STAGE >= 4 ? 4 : (225280u / STAGE >= 3 ? 3 : 2);
    static constexpr int ONES = (9 - (NGRP - 1) * TG) * CI;          // first padding row of the last group
    static constexpr int TCOLS = tc_pow2(NGRP * NN);
    static constexpr uint32_t need = NST * STAGE + 2 * NST * 8 + 16;
    // at least enough shared memory that no more CTAs share an SM than its 512 tensor-memory columns hold
    static constexpr uint32_t floor_bytes = 233472u / (512u / (uint32_t)TCOLS + 1u) - 1024u + 16u;
    static constexpr uint32_t SMEM = need > floor_bytes ? need : floor_bytes;
    static constexpr int PART = NGRP * 128 * NN;   // floats of one CTA's partial sums
    static_assert(CI % 8 == 0 && NB % 16 == 0 && NGRP * TG > 9, "tile shape");
    static_assert(LAST_SLOTS <= (uint32_t)TG && A_REGION % 16 == 0, "last tap group");
    static_assert(STAGE % 16 == 0 && TAP_BYTES % 16 == 0 && B_BYTES % 16 == 0, "bulk copy sizes");
    static_assert(NST * STAGE + 2 * NST * 8 + 16 <= 232448u, "shared memory");
};

template <int CI, int NB, int LOGD>
__global__ void __launch_bounds__(kTcThreads, 1)
k_wgrad_tc(const uint4* __restrict__ a, const uint4* __restrict__ d, float* __restrict__ part,
           int* __restrict__ status) {
    using WG = WgGeo<CI, NB, LOGD>;
    constexpr int D = WG::D, TG = WG::TG, NGRP = WG::NGRP, NN = WG::NN, NST = WG::NST;
    constexpr int nlines = D * D;
    constexpr uint32_t SBO = (uint32_t)D * 16;
    constexpr uint32_t idesc = idesc_bf16_mn(128, NN);
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * WG::STAGE);
    uint64_t* done = full + NST;
    uint32_t* holder = reinterpret_cast<uint32_t*>(done + NST);
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // zero every stage (the tap slots past the ninth stay zero), then the ones row
    for (uint32_t q = tid; q < NST * WG::STAGE / 16; q += kTcThreads)
        reinterpret_cast<uint4*>(smem)[q] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int q = tid; q < NST * D; q += kTcThreads) {
        unsigned char* row = smem + (q / D) * WG::STAGE + (NGRP - 1) * WG::A_BYTES + (WG::ONES / 8) * SBO + (q % D) * 16;
        *reinterpret_cast<uint32_t*>(row) = 0x3F80u;   // BF16 1.0 in channel slot 0 of the row group
    }
    fence_proxy_async_smem();
    if (tid == 0) {
        for (int st = 0; st < NST; ++st) {
            mbar_init(&full[st], 1);
            mbar_init(&done[st], 1);
        }
        fence_barrier_init();
        s_ok = 1;
    }
    if (warp == 0) {
        tmem_alloc(holder, WG::TCOLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *holder;
    if (tid == 0) {
        const uint32_t s_u = smem_u32(smem);
        const int first = blockIdx.x, stride = gridDim.x;
        const int nmine = first < nlines ? (nlines - first + stride - 1) / stride : 0;
        uint32_t ph_full = 0u, ph_done = 0u, pend_full = 0u, pend_done = 0u;   // one bit per stage
        auto load = [&](int line, int st) {
            const int x = line >> LOGD, y = line & (D - 1);
            unsigned char* sa = smem + st * WG::STAGE;
            mbar_arrive_expect_tx(&full[st], 9u * WG::TAP_BYTES + WG::B_BYTES);
#pragma unroll 1
            for (int t9 = 0; t9 < 9; ++t9) {
                const int gx = (x + t9 / 3 - 1) & (D - 1), gy = (y + t9 % 3 - 1) & (D - 1);
                bulk_g2s(sa + (t9 / TG) * WG::A_BYTES + (t9 % TG) * WG::TAP_BYTES,
                         a + ((((long long)gx << LOGD) + gy) * (CI / 8)) * D, WG::TAP_BYTES, &full[st]);
            }
            bulk_g2s(sa + WG::A_REGION, d + (((long long)x << LOGD) + y) * 3 * (NB / 8) * D, WG::B_BYTES,
                     &full[st]);
            pend_full |= 1u << st;
        };
        bool ok = true;
        for (int st = 0; st < NST && st < nmine; ++st) load(first + st * stride, st);
#pragma unroll 1
        for (int i = 0; i < nmine && ok; ++i) {
            const int st = i % NST;
            ok = mbar_wait(&full[st], (ph_full >> st) & 1u);
            if (!ok) break;
            ph_full ^= 1u << st;
            pend_full &= ~(1u << st);
            tc_fence_after();
            const uint32_t a0 = s_u + st * WG::STAGE, b0 = a0 + WG::A_REGION;
#pragma unroll 1
            for (int g = 0; g < NGRP; ++g)
#pragma unroll 1
                for (int ks = 0; ks < D / 16; ++ks)
                    mma_bf16(tmem + g * NN, smem_desc(a0 + g * WG::A_BYTES + ks * 256, 128, SBO),
                             smem_desc(b0 + ks * 256, 128, SBO), idesc, (i > 0 || ks > 0) ? 1u : 0u);
            mma_commit(&done[st]);
            pend_done |= 1u << st;
            // the MMAs of line i - 1 (queued before these) are done: refill their stage
            if (i >= 1) {
                const int ps = (i - 1) % NST;
                ok = mbar_wait(&done[ps], (ph_done >> ps) & 1u);
                if (!ok) break;
                ph_done ^= 1u << ps;
                pend_done &= ~(1u << ps);
                if (i - 1 + NST < nmine) load(first + (i - 1 + NST) * stride, ps);
            }
        }
        if (ok && nmine > 0) {
            const int ls = (nmine - 1) % NST;
            ok = mbar_wait(&done[ls], (ph_done >> ls) & 1u);
            if (ok) pend_done &= ~(1u << ls);
        }
        if (!ok) {
            s_ok = 0;
            atomicExch(status, kStatusTimeout);
            // one more bounded wait for the copies and MMAs in flight
            for (int st = 0; st < NST; ++st) {
                if (pend_full & (1u << st)) (void)mbar_wait(&full[st], (ph_full >> st) & 1u);
                if (pend_done & (1u << st)) (void)mbar_wait(&done[st], (ph_done >> st) & 1u);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (s_ok) {
        const int quarter = warp & 3, hh = warp >> 2;
        const int row = quarter * 32 + lane;
        float* dst = part + (long long)blockIdx.x * WG::PART;
#pragma unroll 1
        for (int i = hh; i < NGRP * (NN / 16); i += 2) {
            const int g = i / (NN / 16), c = i % (NN / 16);
            uint32_t r[16];
            tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + g * NN + c * 16, r);
            tmem_wait_ld(r);
            float4* o = reinterpret_cast<float4*>(dst + ((long long)g * 128 + row) * NN + c * 16);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                o[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]), __uint_as_float(r[4 * j + 2]),
                                   __uint_as_float(r[4 * j + 3]));
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, WG::TCOLS);
}

// sum of the CTAs' partials in CTA order, scattered to dW[co][ci][27]; the
// ones row's dz = 0 columns to db[co] when db is given
__global__ void k_wgrad_reduce(const float* __restrict__ part, int nparts, int CI, int NB, int ngrp, int cin,
                               int cout, float* __restrict__ dw, float* __restrict__ db) {
    const int NN = 3 * NB, TG = 128 / CI, width = ngrp * 128 * NN, ones = (9 - (ngrp - 1) * TG) * CI;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= width) return;
    const int g = e / (128 * NN), r = (e / NN) % 128, n = e % NN;
    const int t9 = g * TG + r / CI, ci = r % CI, j = n / NB, co = n % NB;
    const bool bias = db != nullptr && g == ngrp - 1 && r == ones && j == 1 && co < cout;
    if (!bias && (t9 >= 9 || ci >= cin || co >= cout)) return;
    float s = 0.0f;
    for (int q = 0; q < nparts; ++q) s += part[(long long)q * width + e];
    if (bias)
        db[co] = s;
    else
        dw[((long long)co * cin + ci) * 27 + t9 * 3 + j] = s;
}

}  // namespace cnn
}  // namespace ns3d
