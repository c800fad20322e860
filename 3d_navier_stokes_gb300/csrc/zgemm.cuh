// zgemm.cuh — the z pass (P3) of the FP32 engines for N <= 128 as two
// tensor-core GEMMs with split-BF16 operands (z-pass form 2).
//
// The z transforms are dense matrix products over the kz / z index of each
// stored (x, y) line:
//   inverse (c2r of the six fields u, w):
//     u[line][z] = sum_k A[line][k] Binv[z][k],  A = the line's stored
//     complex modes kz = 0..KC as 2 (KC + 1) interleaved (re, im) floats,
//     Binv[z][2 kz] = m_kz cos(2 pi kz z / N), Binv[z][2 kz + 1] =
//     -m_kz sin(2 pi kz z / N), m_0 = 1 (and the kz = 0 imaginary part
//     ignored, as FFTW's c2r does), m_kz = 2 otherwise;
//   u x w per point in the epilogue (with the CFL speed bound);
//   forward (r2c of the three products):
//     out[line][k'] = sum_z p[line][z] Bfwd[k'][z], Bfwd[2 kz][z] =
//     cos(2 pi kz z / N), Bfwd[2 kz + 1][z] = -sin(2 pi kz z / N),
//     written back as the interleaved complex modes kz = 0..KC.
// Both are unnormalised like the FFT form (the 1/N^6 is applied by P5).
//
// Precision: every operand is split into BF16 hi + lo (x = hi + lo + O(2^-16 x))
// and each product is the three-term sum Ah Bh + Ah Bl + Al Bh accumulated in
// FP32 in tensor memory (tcgen05.mma kind::f16, M = 128 lines per tile).
// Expected relative error of a transform ~1e-5; the tests state the bar.
//
// Layout: operands in shared memory in the SWIZZLE_NONE K-major canonical
// form of tcgen05.cuh. The DFT matrices (hi then lo) are built on the host in
// that order and copied into shared memory once per CTA; A tiles are read
// from global memory as FP32, split and stored by all 256 threads, double
// buffered so that the MMAs of one field run while the next one is staged.
// Persistent CTAs (one per SM) walk the 128-line tiles. Inverse: the six
// fields of a sweep of ZQ z columns accumulate in 6 ZQ tensor-memory columns;
// the epilogue (8 warps: lane quarter x column half) forms u x w and writes
// the three products to the workspace P [member][3][N*N lines][N]. Forward:
// the three product tiles accumulate in 3 KI columns, and the epilogue writes
// the modes into fields 0..2 of W. Every wait is bounded; on a timeout the
// kernel records kStatusTimeout, waits (full budget) for its MMAs in flight,
// frees its tensor memory and returns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tcgen05.cuh"
#include "tma.cuh"

namespace ns3d {

__host__ __device__ constexpr int pow2_at_least(int v) {
    int p = 32;
    while (p < v) p <<= 1;
    return p;
}

template <int N>
struct ZGeo {
    static constexpr int KC = N / 3;
    static constexpr int KIN = 2 * (KC + 1);             // floats of a stored z line that can be non-zero
    static constexpr int KI = (KIN + 15) / 16 * 16;      // K of the inverse GEMM, N of the forward GEMM
    // z columns per inverse sweep: the six fields must fit the 512 tensor-memory columns
    static constexpr int ZQ = N <= 64 ? N : (N % 64 == 0 ? 64 : 48);
    static constexpr int NH = N / ZQ;
    static constexpr int TC_INV = pow2_at_least(6 * ZQ);
    static constexpr int TC_FWD = pow2_at_least(3 * KI);
    static constexpr uint32_t BI = (uint32_t)N * KI * 2;     // bytes of Binv (hi, or lo)
    static constexpr uint32_t AI = 128u * KI * 2;            // bytes of one inverse A tile (hi, or lo)
    static constexpr uint32_t BF = (uint32_t)KI * N * 2;     // bytes of Bfwd (hi, or lo)
    static constexpr uint32_t AF = 128u * N * 2;             // bytes of one forward A tile (hi, or lo)
    // shared memory requested per CTA: the operands, and at least enough that no
    // more CTAs fit on an SM (228 KB, 1 KB reserved per CTA) than its tensor
    // memory (512 columns) can hold, so that no tcgen05.alloc has to wait
    static constexpr uint32_t smem_for(uint32_t need, int tcols) {
        const uint32_t k = 512u / (uint32_t)tcols;
        const uint32_t floor_bytes = 233472u / (k + 1u) - 1024u + 16u;
        return need > floor_bytes ? need : floor_bytes;
    }
    static constexpr uint32_t SMEM_INV = smem_for(2 * BI + 4 * AI + 64, TC_INV);
    static constexpr uint32_t SMEM_FWD = smem_for(2 * BF + 4 * AF + 64, TC_FWD);
};

// grids the tensor-core z pass is compiled for: MMA N and K steps of 16, 128-line tiles
template <typename T, int N>
constexpr bool zgemm_ok() {
    return sizeof(T) == 4 && N >= 16 && N <= 128 && N % 16 == 0 && ((long long)N * N) % 128 == 0;
}

constexpr int kZgThreads = 256;

// The four DFT matrices of grid N as BF16 bit patterns in the canonical
// operand order: Binv hi, Binv lo ([N][KI]), Bfwd hi, Bfwd lo ([KI][N])
// (host, ns3d_misc.cu).
void zgemm_matrices(int N, int KI, uint16_t* out);

// byte offset of the 16-byte chunk (row r, K elements 8 k8 .. 8 k8 + 7) of a
// canonical K-major operand with K columns
__host__ __device__ constexpr uint32_t zg_chunk(int r, int k8, int K) {
    return (uint32_t)(((r >> 3) * (K >> 3) + k8) * 128 + (r & 7) * 16);
}

// FP32 x8 -> BF16 hi x8 and lo x8 (x = hi + lo + O(2^-16 x))
__device__ __forceinline__ void zg_split8(const float (&v)[8], uint4& hi, uint4& lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const __nv_bfloat16 a = __float2bfloat16_rn(v[2 * j]), b = __float2bfloat16_rn(v[2 * j + 1]);
        const float ra = v[2 * j] - __bfloat162float(a), rb = v[2 * j + 1] - __bfloat162float(b);
        __nv_bfloat162 hp;
        hp.x = a;
        hp.y = b;
        h[j] = *reinterpret_cast<uint32_t*>(&hp);
        l[j] = tc::pack_bf16x2(ra, rb);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// three-term split product of one K = 16 step into accumulator d
__device__ __forceinline__ void zg_mma3(uint32_t d, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl, uint32_t sbo_a,
                                        uint32_t sbo_b, uint32_t idesc, uint32_t first) {
    tc::mma_bf16(d, tc::smem_desc(ah, 128, sbo_a), tc::smem_desc(bh, 128, sbo_b), idesc, first ? 0u : 1u);
    tc::mma_bf16(d, tc::smem_desc(ah, 128, sbo_a), tc::smem_desc(bl, 128, sbo_b), idesc, 1u);
    tc::mma_bf16(d, tc::smem_desc(al, 128, sbo_a), tc::smem_desc(bh, 128, sbo_b), idesc, 1u);
}

// Inverse z transforms of the six fields of W, u x w and the CFL bound; products to P.
template <int N>
__global__ void __launch_bounds__(kZgThreads, 1)
k_zgemm_inv(const float* __restrict__ W, const uint4* __restrict__ bpk, float* __restrict__ P,
            StepDev* __restrict__ sd, int want_umax, int nmem) {
    using Z = ZGeo<N>;
    using G = Geo<N>;
    constexpr int KI = Z::KI, ZQ = Z::ZQ, K8 = KI / 8;
    constexpr long long LPM = (long long)N * N;   // lines per member
    constexpr uint32_t SBO = K8 * 128;
    constexpr uint32_t idesc = tc::idesc_bf16(128, ZQ);
    const long long ntiles = LPM * nmem / 128;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sB = smem;                 // Binv hi [N][KI], then lo
    unsigned char* sA = smem + 2 * Z::BI;     // [buffer 2][hi, lo]
    uint64_t* done = reinterpret_cast<uint64_t*>(sA + 4 * Z::AI);
    uint32_t* holder = reinterpret_cast<uint32_t*>(done + 2);
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long budget = sd[0].wait_cycles > 0 ? sd[0].wait_cycles : kWaitCycles;

    for (uint32_t q = tid; q < 2 * Z::BI / 16; q += kZgThreads) reinterpret_cast<uint4*>(sB)[q] = bpk[q];
    fence_proxy_async_smem();
    if (tid == 0) {
        mbar_init(&done[0], 1);
        mbar_init(&done[1], 1);
        fence_barrier_init();
        s_ok = 1;
    }
    if (warp == 0) {
        tc::tmem_alloc(holder, Z::TC_INV);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *holder;
    const uint32_t sA_u = smem_u32(sA), sB_u = smem_u32(sB);
    uint32_t ph[2] = {0u, 0u};          // thread 0: phase to wait for on done[b]
    bool pend[2] = {false, false};      // thread 0: a commit on done[b] not yet waited for
    bool ok = true;
    int use = 0, last = 0;
    const int quarter = warp & 3, hh = warp >> 2;
    const uint32_t lrow = (uint32_t)(quarter * 32) << 16;

    for (long long tile = blockIdx.x; tile < ntiles && s_ok; tile += gridDim.x) {
        const long long line0 = tile * 128;
        const long long mem = line0 / LPM, l0 = line0 % LPM;
        float um = 0.f;
        for (int h = 0; h < Z::NH && s_ok; ++h) {
            for (int f = 0; f < 6; ++f, ++use) {
                const int b = use & 1;
                if (tid == 0 && pend[b]) {   // buffer b is free once the MMAs of its last use completed
                    if (ok) ok = mbar_wait(&done[b], ph[b], budget);
                    if (ok) {
                        ph[b] ^= 1u;
                        pend[b] = false;
                    } else {
                        s_ok = 0;
                        atomicExch(&sd[mem].status, kStatusTimeout);
                    }
                }
                __syncthreads();
                if (!s_ok) break;
                const float* src = W + ((mem * 6 + f) * G::FS + l0 * G::NZP) * 2;
                unsigned char* aH = sA + b * 2 * Z::AI;
                for (int q = tid; q < 128 * K8; q += kZgThreads) {
                    const int r = q / K8, k8 = q % K8;
                    const float* rp = src + (long long)r * 2 * G::NZP + k8 * 8;
                    float v[8];
                    if (k8 * 8 + 8 <= Z::KIN) {
                        const float4 a = reinterpret_cast<const float4*>(rp)[0];
                        const float4 c = reinterpret_cast<const float4*>(rp)[1];
                        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                        v[4] = c.x; v[5] = c.y; v[6] = c.z; v[7] = c.w;
                    } else {
#pragma unroll
                        for (int j = 0; j < 8; ++j) v[j] = (k8 * 8 + j < Z::KIN) ? rp[j] : 0.f;
                    }
                    uint4 hi, lo;
                    zg_split8(v, hi, lo);
                    const uint32_t off = zg_chunk(r, k8, KI);
                    *reinterpret_cast<uint4*>(aH + off) = hi;
                    *reinterpret_cast<uint4*>(aH + Z::AI + off) = lo;
                }
                fence_proxy_async_smem();
                __syncthreads();
                if (tid == 0) {
                    tc::tc_fence_after();
                    const uint32_t ah = sA_u + b * 2 * Z::AI, al = ah + Z::AI;
                    const uint32_t bh = sB_u + (uint32_t)(h * ZQ / 8) * SBO, bl = bh + Z::BI;
#pragma unroll 1
                    for (int ks = 0; ks < KI / 16; ++ks)
                        zg_mma3(tmem + f * ZQ, ah + ks * 256, al + ks * 256, bh + ks * 256, bl + ks * 256, SBO, SBO,
                                idesc, ks == 0);
                    tc::mma_commit(&done[b]);
                    pend[b] = true;
                    last = b;
                }
            }
            // the sweep's accumulators are complete once its last commit has arrived
            if (tid == 0 && s_ok) {
                if (ok) ok = mbar_wait(&done[last], ph[last], budget);
                if (ok) {
                    ph[last] ^= 1u;
                    pend[last] = false;
                } else {
                    s_ok = 0;
                    atomicExch(&sd[mem].status, kStatusTimeout);
                }
            }
            __syncthreads();
            if (!s_ok) break;
            tc::tc_fence_after();
            const long long line = l0 + quarter * 32 + lane;
            float* pout = P + (mem * 3 * LPM + line) * N + h * ZQ;
#pragma unroll 1
            for (int c = hh; c < ZQ / 16; c += 2) {
                uint32_t r0[16], r1[16], r2[16], r3[16], r4[16], r5[16];
                const uint32_t ta = tmem + lrow + c * 16;
                tc::tmem_ld16(ta, r0);
                tc::tmem_ld16(ta + ZQ, r1);
                tc::tmem_ld16(ta + 2 * ZQ, r2);
                tc::tmem_ld16(ta + 3 * ZQ, r3);
                tc::tmem_ld16(ta + 4 * ZQ, r4);
                tc::tmem_ld16(ta + 5 * ZQ, r5);
                tc::tmem_wait_ld(r0);
                tc::tmem_wait_ld(r1);
                tc::tmem_wait_ld(r2);
                tc::tmem_wait_ld(r3);
                tc::tmem_wait_ld(r4);
                tc::tmem_wait_ld(r5);
                float px[16], py[16], pz[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float ux = __uint_as_float(r0[j]), uy = __uint_as_float(r1[j]), uz = __uint_as_float(r2[j]);
                    const float wx = __uint_as_float(r3[j]), wy = __uint_as_float(r4[j]), wz = __uint_as_float(r5[j]);
                    um = fmaxf(um, fabsf(ux) + fabsf(uy) + fabsf(uz));
                    px[j] = uy * wz - uz * wy;
                    py[j] = uz * wx - ux * wz;
                    pz[j] = ux * wy - uy * wx;
                }
                float4* dx = reinterpret_cast<float4*>(pout + c * 16);
                float4* dy = reinterpret_cast<float4*>(pout + LPM * N + c * 16);
                float4* dz = reinterpret_cast<float4*>(pout + 2 * LPM * N + c * 16);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    dx[j] = make_float4(px[4 * j], px[4 * j + 1], px[4 * j + 2], px[4 * j + 3]);
                    dy[j] = make_float4(py[4 * j], py[4 * j + 1], py[4 * j + 2], py[4 * j + 3]);
                    dz[j] = make_float4(pz[4 * j], pz[4 * j + 1], pz[4 * j + 2], pz[4 * j + 3]);
                }
            }
            // the accumulators are read before the next sweep's MMAs overwrite them
            tc::tc_fence_before();
            __syncthreads();
        }
        if (want_umax) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) um = fmaxf(um, __shfl_xor_sync(0xffffffffu, um, o));
            if (lane == 0) Bits<float>::amax(&sd[mem].umax_bits, um);
        }
    }
    // a failed wait: wait (full budget) for the MMAs still in flight before the tensor memory goes
    if (tid == 0) {
#pragma unroll
        for (int b = 0; b < 2; ++b)
            if (pend[b]) (void)mbar_wait(&done[b], ph[b], kWaitCycles);
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, Z::TC_INV);
}

// Forward z transforms of the three products in P; modes kz = 0..KC into fields 0..2 of W.
template <int N>
__global__ void __launch_bounds__(kZgThreads, 1)
k_zgemm_fwd(const float* __restrict__ P, const uint4* __restrict__ bpk, float* __restrict__ W,
            StepDev* __restrict__ sd, int nmem) {
    using Z = ZGeo<N>;
    using G = Geo<N>;
    constexpr int KI = Z::KI, N8 = N / 8;
    constexpr long long LPM = (long long)N * N;
    constexpr uint32_t SBO_A = N8 * 128, SBO_B = N8 * 128;
    constexpr uint32_t idesc = tc::idesc_bf16(128, KI);
    const long long ntiles = LPM * nmem / 128;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sB = smem;                 // Bfwd hi [KI][N], then lo
    unsigned char* sA = smem + 2 * Z::BF;     // [buffer 2][hi, lo]
    uint64_t* done = reinterpret_cast<uint64_t*>(sA + 4 * Z::AF);
    uint32_t* holder = reinterpret_cast<uint32_t*>(done + 2);
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long budget = sd[0].wait_cycles > 0 ? sd[0].wait_cycles : kWaitCycles;

    for (uint32_t q = tid; q < 2 * Z::BF / 16; q += kZgThreads) reinterpret_cast<uint4*>(sB)[q] = bpk[q];
    fence_proxy_async_smem();
    if (tid == 0) {
        mbar_init(&done[0], 1);
        mbar_init(&done[1], 1);
        fence_barrier_init();
        s_ok = 1;
    }
    if (warp == 0) {
        tc::tmem_alloc(holder, Z::TC_FWD);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *holder;
    const uint32_t sA_u = smem_u32(sA), sB_u = smem_u32(sB);
    uint32_t ph[2] = {0u, 0u};
    bool pend[2] = {false, false};
    bool ok = true;
    int use = 0, last = 0;
    const int quarter = warp & 3, hh = warp >> 2;
    const uint32_t lrow = (uint32_t)(quarter * 32) << 16;

    for (long long tile = blockIdx.x; tile < ntiles && s_ok; tile += gridDim.x) {
        const long long line0 = tile * 128;
        const long long mem = line0 / LPM, l0 = line0 % LPM;
        for (int f = 0; f < 3; ++f, ++use) {
            const int b = use & 1;
            if (tid == 0 && pend[b]) {
                if (ok) ok = mbar_wait(&done[b], ph[b], budget);
                if (ok) {
                    ph[b] ^= 1u;
                    pend[b] = false;
                } else {
                    s_ok = 0;
                    atomicExch(&sd[mem].status, kStatusTimeout);
                }
            }
            __syncthreads();
            if (!s_ok) break;
            const float* src = P + ((mem * 3 + f) * LPM + l0) * N;
            unsigned char* aH = sA + b * 2 * Z::AF;
            for (int q = tid; q < 128 * N8; q += kZgThreads) {
                const int r = q / N8, k8 = q % N8;
                const float4* rp = reinterpret_cast<const float4*>(src + (long long)r * N + k8 * 8);
                const float4 a = rp[0], c = rp[1];
                const float v[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
                uint4 hi, lo;
                zg_split8(v, hi, lo);
                const uint32_t off = zg_chunk(r, k8, N);
                *reinterpret_cast<uint4*>(aH + off) = hi;
                *reinterpret_cast<uint4*>(aH + Z::AF + off) = lo;
            }
            fence_proxy_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::tc_fence_after();
                const uint32_t ah = sA_u + b * 2 * Z::AF, al = ah + Z::AF;
                const uint32_t bh = sB_u, bl = sB_u + Z::BF;
#pragma unroll 1
                for (int ks = 0; ks < N / 16; ++ks)
                    zg_mma3(tmem + f * KI, ah + ks * 256, al + ks * 256, bh + ks * 256, bl + ks * 256, SBO_A, SBO_B,
                            idesc, ks == 0);
                tc::mma_commit(&done[b]);
                pend[b] = true;
                last = b;
            }
        }
        if (tid == 0 && s_ok) {
            if (ok) ok = mbar_wait(&done[last], ph[last], budget);
            if (ok) {
                ph[last] ^= 1u;
                pend[last] = false;
            } else {
                s_ok = 0;
                atomicExch(&sd[mem].status, kStatusTimeout);
            }
        }
        __syncthreads();
        if (!s_ok) break;
        tc::tc_fence_after();
        const long long line = l0 + quarter * 32 + lane;
#pragma unroll 1
        for (int i = hh; i < 3 * (KI / 16); i += 2) {
            const int f = i / (KI / 16), c = i % (KI / 16);
            uint32_t r[16];
            tc::tmem_ld16(tmem + lrow + f * KI + c * 16, r);
            tc::tmem_wait_ld(r);
            float* dst = W + ((mem * 6 + f) * G::FS + line * G::NZP) * 2 + c * 16;
            if (c * 16 + 16 <= Z::KIN) {
                float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    d4[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                                        __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (c * 16 + j < Z::KIN) dst[j] = __uint_as_float(r[j]);
            }
        }
        tc::tc_fence_before();
        __syncthreads();
    }
    if (tid == 0) {
#pragma unroll
        for (int b = 0; b < 2; ++b)
            if (pend[b]) (void)mbar_wait(&done[b], ph[b], kWaitCycles);
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, Z::TC_FWD);
}

}  // namespace ns3d
