// ns3d_kernels.cuh — CUDA kernels of the hot path (templated on precision T
// and grid size N; instantiated in ns3d_inst_*.cu).
//
// Device layout. Every Fourier quantity is stored per component as
// complex [N (x or kx)][N (y or ky)][NZP (kz)] with only kz <= KC = N/3 used
// (NZP = KC+1 rounded up to 8). The 2/3 rule zeroes every mode with
// |k| > N/3 (solver.c:1709-1756), so the Nyquist plane and all modes outside
// the dealiasing sphere are never stored, loaded or transformed: loads of
// known-zero inputs are predicated off and stores of outputs that the next
// pass never reads are skipped.
//
// One nonlinear-term evaluation N(u) (NonlinearRHSBatch, solver.c:620-731)
// is five passes over HBM:
//   P1 k_xinv  : inverse FFT along kx of u_hat with the curl w_hat = i k x u_hat
//                formed on load (solver.c:637-650); 3 fields in, 6 out.
//   P2 k_ypass : inverse FFT along ky (6 fields, in place).
//   P3 k_zpass : per z line: c2r of the 6 fields (two real lines per complex
//                FFT), u x w in shared memory (solver.c:664-677), r2c of the 3
//                products; in place. Also max(|u|+|v|+|w|) for the CFL step.
//   P4 k_ypass : forward FFT along y (3 fields, in place).
//   P5 k_xfwd  : forward FFT along x, then per mode the Leray projection
//                (solver.c:689-721), the dealias mask and the RK stage
//                algebra, written straight into the integrator's arrays.
// The inverse passes scale by 1/N^3 on load, so real-space fields are the true
// velocity/vorticity and the forward transform yields the reference's
// FFT(u x w)/N^6 directly.
#pragma once
#include <type_traits>

#include "fft_engine.cuh"
#include "stats.cuh"
#include "tma.cuh"

namespace ns3d {

// ---------------------------------------------------------------------------
// Geometry and FFT plans
// ---------------------------------------------------------------------------
template <int N_>
struct Geo {
    static constexpr int N = N_;
    static constexpr int KC = N_ / 3;               // dealias radius, integer N/3 (solver.c:1732)
    static constexpr int KC2 = KC * KC;
    static constexpr int NZ1 = KC + 1;              // kz columns in use
    static constexpr int NZP = (NZ1 + 7) / 8 * 8;   // stored kz columns
    static constexpr long long FS = (long long)N_ * N_ * NZP;   // elements per field
    static constexpr int NKY = 2 * KC + 1;          // ky rows with |ky| <= KC
    static constexpr int NSP = KC + 1;              // spectrum bins that can be non-zero
};

// wavenumber of storage index i (InitializeSpaceVariables, solver.c:1786-1812)
template <int N> __device__ __forceinline__ int kof(int i) { return i <= N / 2 ? i : i - N; }

template <int N> struct Plans;
template <> struct Plans<8>    { using A = Plan<8, 8, 8>;            using X = A; };
template <> struct Plans<16>   { using A = Plan<16, 16, 16>;         using X = A; };
template <> struct Plans<24>   { using A = Plan<24, 12, 12, 2>;      using X = A; };
template <> struct Plans<32>   { using A = Plan<32, 8, 4, 8>;        using X = A; };
template <> struct Plans<48>   { using A = Plan<48, 12, 4, 12>;     using X = A; };
template <> struct Plans<64>   { using A = Plan<64, 8, 8, 8>;        using X = A; };
template <> struct Plans<96>   { using A = Plan<96, 12, 4, 4, 6>;    using X = A; };
template <> struct Plans<128>  { using A = Plan<128, 16, 16, 8>;     using X = Plan<128, 8, 8, 4, 4>; };
template <> struct Plans<256>  { using A = Plan<256, 16, 16, 16>;    using X = Plan<256, 8, 8, 8, 4>; };
template <> struct Plans<512>  { using A = Plan<512, 16, 8, 8, 8>;   using X = Plan<512, 8, 8, 8, 8>; };
template <> struct Plans<1024> { using A = Plan<1024, 16, 16, 16, 4>; using X = Plan<1024, 8, 8, 8, 4, 4>; };
// sizes with a factor 3 (the reference accepts any even N, utils.c:88-104): 12 elements per thread
template <> struct Plans<192>  { using A = Plan<192, 12, 4, 4, 12>;    using X = A; };
template <> struct Plans<384>  { using A = Plan<384, 12, 4, 4, 4, 6>;  using X = A; };
template <> struct Plans<768>  { using A = Plan<768, 12, 4, 4, 4, 4, 3>; using X = A; };

// Tile width (pencils per CTA along kz) of the strided passes: one 128-byte
// row segment per pencil row where the thread count allows. Variant V of the
// FP32 engines asks for other widths (clipped to 512 threads per CTA); the
// autotuner times the compiled variants of a grid size and keeps the fastest.
#ifndef NS3D_TILE_A32
#define NS3D_TILE_A32 8
#endif
#ifndef NS3D_TILE_X32
#define NS3D_TILE_X32 16
#endif
// A / AF: pencils per CTA of the inverse / forward y pass; X / XF: of the
// inverse / forward x pass.
// MINB / MINB_XI: CTAs per SM the x-forward / x-inverse passes are compiled
// for (registers capped to fit); BATCH: the x-forward epilogue issues all of a
// thread's state loads of a component before their updates (more registers);
// STAGE: velocity components the x-inverse pass stages in shared memory (2:
// y and z, two live arrays instead of four, 11 % faster at 256^3; 1: z only,
// three live arrays, for the 16-element plan of variant 3; 0: none)
template <int V> struct TileVar;
template <> struct TileVar<0> { static constexpr int A = NS3D_TILE_A32, AF = NS3D_TILE_A32, X = NS3D_TILE_X32, XF = NS3D_TILE_X32, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 2; };
template <> struct TileVar<1> { static constexpr int A = 4, AF = 4, X = 8, XF = 8, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 2; };
template <> struct TileVar<2> { static constexpr int A = 16, AF = 16, X = 8, XF = 8, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 2; };
template <> struct TileVar<3> { static constexpr int A = NS3D_TILE_A32, AF = 16, X = 16, XF = 16, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 1; };
template <> struct TileVar<4> { static constexpr int A = NS3D_TILE_A32, AF = NS3D_TILE_A32, X = 4, XF = 4, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 2; };
template <> struct TileVar<5> { static constexpr int A = NS3D_TILE_A32, AF = NS3D_TILE_A32, X = NS3D_TILE_X32, XF = NS3D_TILE_X32, MINB = 2, MINB_XI = 1; static constexpr bool BATCH = false; static constexpr int STAGE = 2; };
template <> struct TileVar<6> { static constexpr int A = 16, AF = 16, X = 8, XF = NS3D_TILE_X32, MINB = 1, MINB_XI = 1; static constexpr bool BATCH = true; static constexpr int STAGE = 2; };

// Variant 5: the default tiles and plans with the x-forward pass compiled for
// two CTAs per SM, so one CTA's FFT overlaps another's loads (the x-inverse
// pass spills too much at 64 registers to gain from the same).
// Variant 4: 4-pencil x tiles (half-size CTAs, twice as many per SM).
// Variant 6: variant 2's 16-pencil y tiles and 8-pencil x-inverse tiles with
// 16-pencil x-forward tiles (the per-kernel best of variants 0 and 2 at 256^3).
// Plans of variant V: variant 3 gives the x passes a plan with twice the
// elements per thread (half the threads per pencil), with 16 pencils per CTA
// (every row access a full 128-byte segment).
// Plan of a y pass: the z-line plan, except for the inverse pass at 96 points in
// FP32, where a y line (one field per pencil) affords 24 elements per thread and
// two stages (12 x 8, one exchange) instead of three (4 x 4 x 6, two exchanges):
// 0.155 -> 0.145-0.148 ms per launch for 24 members; the forward pass measured slower
// with it (0.058 -> 0.060 ms). The z lines hold three fields per line and keep 12.
template <typename T, int N, bool INV> struct YPlan { using A = typename Plans<N>::A; };
template <> struct YPlan<float, 96, true> { using A = Plan<96, 24, 12, 8>; };
template <int N> struct AltX { using X = typename Plans<N>::X; };
template <> struct AltX<64> { using X = Plan<64, 16, 16, 4>; };
template <> struct AltX<128> { using X = Plan<128, 16, 16, 8>; };
template <> struct AltX<256> { using X = Plan<256, 16, 16, 16>; };
template <> struct AltX<512> { using X = Plan<512, 16, 8, 8, 8>; };
template <> struct AltX<1024> { using X = Plan<1024, 16, 8, 8, 4, 4>; };
template <int N, int V> struct PlansV {
    using A = typename Plans<N>::A;
    using X = typename std::conditional<(V == 3), typename AltX<N>::X, typename Plans<N>::X>::type;
};
template <int P, int W> constexpr int clip_tile() { return P * W <= 512 ? W : (P * 8 <= 512 ? 8 : (P * 4 <= 512 ? 4 : 2)); }
template <typename T, int N, int V = 0, bool INV = true> constexpr int tile_a() {
    return sizeof(T) == 4 ? clip_tile<YPlan<T, N, INV>::A::P, (INV ? TileVar<V>::A : TileVar<V>::AF)>()
                          : (YPlan<T, N, INV>::A::P * 8 <= 512 ? 8 : 4);
}
template <typename T, int N, int V = 0, bool FWD = false> constexpr int tile_x() {
    constexpr int P = PlansV<N, V>::X::P;
    return sizeof(T) == 4 ? clip_tile<P, (FWD ? TileVar<V>::XF : TileVar<V>::X)>()
                          : (P * 8 <= 256 ? 8 : (P * 4 <= 512 ? 4 : 2));
}
// line pairs per CTA of the z pass (>= 96 threads)
template <int N> constexpr int zpairs() {
    return (3 * Plans<N>::A::P >= 96) ? 1 : (96 + 3 * Plans<N>::A::P - 1) / (3 * Plans<N>::A::P);
}

struct SyncBlock {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
// Exchange slot of element m of pencil t: [m'][TT] with the row m' = m XOR
// ((m / R1) mod G), G = 32 / TT pencil groups per warp (G < R1, power-of-two
// R1; identity otherwise). The first stage's writes of a warp's G groups go
// to rows R1 apart (R1 * TT complex, a multiple of 128 bytes) and would share
// one bank range; the XOR spreads them over the banks. The reads of
// consecutive rows stay consecutive (a permutation inside each aligned block
// of R1 rows), so neither side has bank conflicts.
template <int TT, int R1 = 1>
struct StridedIdx {
    static constexpr int G = TT < 16 ? 32 / TT : 1;
    static constexpr bool kSwz = G > 1 && (R1 & (R1 - 1)) == 0 && R1 >= G;
    static constexpr int kShift = (R1 >= 16) ? 4 : (R1 >= 8) ? 3 : (R1 >= 4) ? 2 : (R1 >= 2) ? 1 : 0;
    int t;
    __device__ __forceinline__ int operator()(int m) const {
        if constexpr (kSwz) m ^= (m >> kShift) & (G - 1);
        return m * TT + t;
    }
};
struct PaddedIdx {    // exchange slot of element m of one line: one pad slot per 16
    __device__ __forceinline__ int operator()(int m) const { return m + (m >> 4); }
};

// ---------------------------------------------------------------------------
// Per-step device state and integrator tables
// ---------------------------------------------------------------------------
struct StepDev {
    double t, dt, t0, nu, cfl;
    double force_target;
    double umax;                     // last CFL speed bound (true velocity)
    unsigned long long umax_bits;    // running max of the stage-1 z pass (bits of T, non-negative)
    long long iters;
    int status;                      // 0 ok; 5 numeric
    long long wait_cycles;           // budget of the z pass's first wait on each copy (kWaitCycles by default)
    int sgs_on;                      // learned closure used in this step (energy-budget check passed)
    long long sgs_steps, sgs_fallbacks;
    // Dormand-Prince step control (DP5CN)
    double dp_atol, dp_rtol;         // error tolerances
    double dp_err;                   // error norm of the last attempt
    double dp_h;                     // step size of the last attempt
    int dp_accept;                   // last attempt accepted
    int dp_tries;                    // consecutive rejected attempts
    long long dp_rejects;            // rejected attempts so far
};

enum { INT_IFRK4 = 0, INT_RK4CN = 1, INT_RK5CN = 2, INT_DP5CN = 3 };
// k_xfwd template tag of the tableau-driven epilogue (RK5CN, DP5CN)
enum { INT_TAB = 4 };
constexpr int kStatusDpFail = 7;     // a DP5CN step was rejected kDpMaxTry times in a row
constexpr int kDpMaxTry = 50;        // DP_MAX_TRY (data_types.h:128)

// One stage epilogue of the RK5 family (RK5DPStep, solver.c:217-421): with k
// the projected RHS just computed and K_j the stored earlier stages,
//   kind 0: UT = U + h (sum_{j<nk} c_j K_j + c_cur k)              next stage input
//   kind 1: U  = a U + b (sum c_j K_j + c_cur k)                    RK5CN update
//   kind 2: ACC = a U + b (sum c_j K_j + c_cur k)                   DP5CN trial
//           err_d += |b (sum e_j K_j + e_cur k)|^2 / den_d^2,  den_d = atol + max(|U|, |ACC|) rtol
// with (a, b) = ((2-D)/(2+D), 2h/(2+D)) from the step table; k is stored
// into K_store when store >= 0.
struct RkStage {
    int kind, store, nk, pad;
    double c[6], c_cur;
    double e[6], e_cur;
};
// P5 modes
enum { X_STAGE1 = 0, X_STAGE2 = 1, X_STAGE3 = 2, X_STAGE4 = 3, X_RHS = 8, X_PLAIN = 9 };

// ---------------------------------------------------------------------------
// P1: inverse FFT along kx with curl-on-load. grid (ntile, NKY); block
// TT*P; smem N*TT complex (exchange) + 2*E*TT*P complex (staging). The first
// velocity component is loaded into registers; the other two are copied
// asynchronously into shared memory (each thread its own elements) and read
// back when needed, so at most two E-element arrays are live. The kx-weighted
// inputs of the vorticity are formed from them, so the five transforms below
// read each input once.
// ---------------------------------------------------------------------------
template <typename T, int N, int V = 0>
constexpr size_t xinv_smem() {
    return sizeof(cx<T>) * (size_t)N * tile_x<T, N, V>() * (1 + TileVar<V>::STAGE);
}
template <typename T, int N, int V = 0>
__global__ void __launch_bounds__(tile_x<T, N, V>() * PlansV<N, V>::X::P, TileVar<V>::MINB_XI)
k_xinv(const cx<T>* __restrict__ U, cx<T>* __restrict__ W, const cx<T>* __restrict__ tw) {
    using G = Geo<N>;
    using PL = typename PlansV<N, V>::X;
    constexpr int TT = tile_x<T, N, V>();
    constexpr int E = PL::E, P = PL::P, NT = TT * P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* sbuf = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* stg = sbuf + (size_t)N * TT;   // [2][E][NT]: the staged y and z components
    const int t = threadIdx.x % TT, p = threadIdx.x / TT;
    const int kz = blockIdx.x * TT + t;
    const int ky = (int)blockIdx.y - G::KC;
    const int j = ky < 0 ? ky + N : ky;
    // ensemble member (blockIdx.z): its arrays follow the previous member's
    U += (long long)blockIdx.z * 3 * G::FS;
    W += (long long)blockIdx.z * 6 * G::FS;
    // whole CTA idle when every column of the tile is outside the circle
    const int kz0 = blockIdx.x * TT;
    if (ky * ky + kz0 * kz0 > G::KC2) return;
    const bool colok = (kz <= G::KC) && (ky * ky + kz * kz <= G::KC2);
    const int rem = G::KC2 - ky * ky - kz * kz;
    const long long off = (long long)j * G::NZP + kz;
    const long long xs = (long long)N * G::NZP;
    const T scale = T(1) / (T(N) * T(N) * T(N));
    StridedIdx<TT, PL::R1> sidx{t};
    SyncBlock sync;

    constexpr int kStage = TileVar<V>::STAGE;
    constexpr int kC0 = 3 - kStage;   // first staged component
    // the staged components: asynchronous copies, zero-filled outside the sphere
#pragma unroll
    for (int c = kC0; c <= 2; ++c) {
        const cx<T>* src = U + (long long)c * G::FS + off;
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int kx = kof<N>(p + P * s);
            const bool in = colok && kx * kx <= rem;
            cp_async<sizeof(cx<T>)>(&stg[((c - kC0) * E + s) * NT + threadIdx.x],
                                    in ? src + (long long)(p + P * s) * xs : U, in ? (uint32_t)sizeof(cx<T>) : 0u);
        }
    }
    if (kStage > 0) cp_async_commit();
    auto load = [&](int c, cx<T>(&v)[E]) {
        const cx<T>* src = U + (long long)c * G::FS + off;
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int kx = kof<N>(p + P * s);
            v[s] = (colok && kx * kx <= rem) ? src[(long long)(p + P * s) * xs] * scale : czero<T>();
        }
    };
    auto staged = [&](int c, cx<T>(&v)[E]) {
        cp_async_wait_all();
#pragma unroll
        for (int s = 0; s < E; ++s) v[s] = stg[((c - kC0) * E + s) * NT + threadIdx.x] * scale;
    };
    auto ikx = [&](const cx<T>(&v)[E], cx<T>(&o)[E]) {
#pragma unroll
        for (int s = 0; s < E; ++s) o[s] = mul_i(v[s]) * T(kof<N>(p + P * s));
    };
    auto store = [&](int f, const cx<T>(&v)[E]) {
        if (!colok) return;
        cx<T>* dst = W + (long long)f * G::FS + off;
#pragma unroll
        for (int s = 0; s < E; ++s) dst[(long long)(p + P * s) * xs] = v[s];
    };

    const T fky = T(ky), fkz = T(kz);
    if constexpr (kStage == 1) {
        // x and y components in registers, z staged: three live arrays
        cx<T> X[E], Y[E], B[E];
        load(0, X);
        load(1, Y);
        ikx(Y, B);
        PL::inv(B, sbuf, p, tw, sidx, sync);
        PL::inv(X, sbuf, p, tw, sidx, sync);
        store(0, X);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = B[s] - mul_i(X[s]) * fky;
        store(5, B);
        {
            cx<T> Z[E];
            staged(2, Z);
            ikx(Z, B);
        }
        PL::inv(B, sbuf, p, tw, sidx, sync);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fkz - B[s];
        store(4, B);
        PL::inv(Y, sbuf, p, tw, sidx, sync);
        store(1, Y);
        staged(2, X);   // uz
        PL::inv(X, sbuf, p, tw, sidx, sync);
        store(2, X);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fky - mul_i(Y[s]) * fkz;
        store(3, B);
        return;
    }
    if constexpr (kStage == 0) {
        // every component in registers up front
        cx<T> X[E], Y[E], Z[E], B[E];
        load(0, X);
        load(1, Y);
        load(2, Z);
        ikx(Y, B);
        PL::inv(B, sbuf, p, tw, sidx, sync);
        PL::inv(X, sbuf, p, tw, sidx, sync);
        store(0, X);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = B[s] - mul_i(X[s]) * fky;
        store(5, B);
        ikx(Z, B);
        PL::inv(B, sbuf, p, tw, sidx, sync);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fkz - B[s];
        store(4, B);
        PL::inv(Y, sbuf, p, tw, sidx, sync);
        store(1, Y);
        PL::inv(Z, sbuf, p, tw, sidx, sync);
        store(2, Z);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(Z[s]) * fky - mul_i(Y[s]) * fkz;
        store(3, B);
        return;
    }
    cx<T> X[E], B[E];
    // ux
    load(0, X);
    PL::inv(X, sbuf, p, tw, sidx, sync);
    store(0, X);
    // wz = T(i kx uy) - i ky T(ux)
    {
        cx<T> Y[E];
        staged(1, Y);
        ikx(Y, B);
    }
    PL::inv(B, sbuf, p, tw, sidx, sync);
#pragma unroll
    for (int s = 0; s < E; ++s) B[s] = B[s] - mul_i(X[s]) * fky;
    store(5, B);
    // wy = i kz T(ux) - T(i kx uz)
    {
        cx<T> Z[E];
        staged(2, Z);
        ikx(Z, B);
    }
    PL::inv(B, sbuf, p, tw, sidx, sync);
#pragma unroll
    for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fkz - B[s];
    store(4, B);
    // uy, uz, then wx = i ky T(uz) - i kz T(uy)
    staged(1, X);
    PL::inv(X, sbuf, p, tw, sidx, sync);
    store(1, X);
    staged(2, B);
    PL::inv(B, sbuf, p, tw, sidx, sync);
    store(2, B);
#pragma unroll
    for (int s = 0; s < E; ++s) B[s] = mul_i(B[s]) * fky - mul_i(X[s]) * fkz;
    store(3, B);
}
// ---------------------------------------------------------------------------
// P1, tensor-tile form (FP32, the x plans of variant 3). Persistent CTAs walk
// the (member, ky, kz-tile) items inside the circle ky^2 + kz^2 <= KC^2 (a
// compact list, so that every CTA gets the same number of items). Thread
// 0 copies each velocity component of a tile into one of two slabs [kx][TT]
// with cp.async.bulk.tensor boxes of XB kx rows x TT pencils, only the rows
// |kx| <= kxmax of the tile's widest column (the rest of a slab is stale and
// masked like the rows outside the sphere), completion on the slab's mbarrier.
// Per item: ux and uy are read from their slabs, which then receive this item's
// uz and the next item's ux; uz is read twice (for wy and for itself) and its
// slab then receives the next item's uy. Every copy is issued at least two of
// the item's five transforms before it is read. A slab holds only the rows
// that can lie inside the sphere (SR of N). The six output fields leave through
// an output buffer [N][TT] and bulk tensor stores over a 4D map of W (whole
// tiles: the columns outside the circle, which no later pass reads, receive
// zeros), so no warp waits on a queue of per-thread stores. The transforms and
// their arithmetic are those of k_xinv (results bit-identical). Waits are
// bounded; on a timeout the CTA records kStatusTimeout, waits for its own
// copies and returns.
// ---------------------------------------------------------------------------
// The compact list of the (ky, kz-tile) items whose first column lies inside
// the circle ky^2 + kz0^2 <= KC^2, built on the host in ky-major order: entry
// ((ky + KC) << 8) | tile. Item `it` of member m is entry it - m * nvalid; CTAs
// take items it = blockIdx.x + k gridDim.x, so every CTA gets the same number
// of items to within one (skipping the items outside the circle in a full
// (ky, tile) grid instead left 18 to 22 items per CTA at 512^3).
__device__ __forceinline__ void xtile_item(const int* __restrict__ xitems, int nvalid, int it, int kc, int tt,
                                           int& m, int& ky, int& kz0) {
    m = it / nvalid;
    const int e = __ldg(&xitems[it - m * nvalid]);
    ky = (e >> 8) - kc;
    kz0 = (e & 255) * tt;
}
template <int N> constexpr int xbox_rows() { return N % 32 == 0 ? 32 : 16; }
// pencils per CTA and CTAs per SM: variant 3's x tiles, one CTA per SM (8-pencil
// tiles at two CTAs per SM spill 330 bytes per thread at 512^3 under the 128-register cap)
template <typename T, int N, int V> constexpr int xtma_tile() { return tile_x<T, N, V>(); }
template <typename T, int N, int V> constexpr int xtma_minb() { return 1; }
// rows of an input slab: the XB-row boxes that can hold |kx| <= KC from both ends of
// the kx axis (all N rows when those meet)
template <int N> constexpr int xtma_slab_rows() {
    return 2 * (Geo<N>::KC / xbox_rows<N>() + 1) * xbox_rows<N>() < N
               ? 2 * (Geo<N>::KC / xbox_rows<N>() + 1) * xbox_rows<N>()
               : N;
}
// x rows per output box (bulk tensor store)
template <int N> constexpr int xout_rows() { return N <= 256 ? N : N / 2; }
// exchange buffer and output buffer [N][TT], two input slabs [SR][TT], two mbarriers
template <typename T, int N, int V>
constexpr size_t xinv_tma_smem() {
    return sizeof(cx<T>) * (size_t)xtma_tile<T, N, V>() * (2 * (size_t)N + 2 * (size_t)xtma_slab_rows<N>()) + 16;
}
template <typename T, int N, int V>
constexpr bool xinv_tma_ok() {
    // not at 1024^3 (8-pencil tiles, 64-byte boxes): 5.17 ms per pass against 4.30 ms for k_xinv
    return sizeof(T) == 4 && V == 3 && N % 16 == 0 && N >= 48 && N <= 512 && xinv_tma_smem<T, N, V>() <= 232448 &&
           (2 * xtma_tile<T, N, V>() * sizeof(T)) % 16 == 0 && N % xout_rows<N>() == 0;
}

template <typename T, int N, int V>
__global__ void __launch_bounds__(xtma_tile<T, N, V>() * PlansV<N, V>::X::P, xtma_minb<T, N, V>())
k_xinv_tma(const __grid_constant__ CUtensorMap map, int c0, const __grid_constant__ CUtensorMap wmap, int cw,
           const cx<T>* __restrict__ tw, StepDev* __restrict__ sd, const int* __restrict__ xitems, int nvalid, int cnt) {
    using G = Geo<N>;
    using PL = typename PlansV<N, V>::X;
    constexpr int TT = xtma_tile<T, N, V>();
    constexpr int E = PL::E, P = PL::P;
    constexpr int XB = xbox_rows<N>();
    constexpr uint32_t BOX_BYTES = (uint32_t)XB * TT * sizeof(cx<T>);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int SR = xtma_slab_rows<N>();
    constexpr int XO = xout_rows<N>();
    cx<T>* sbuf = reinterpret_cast<cx<T>*>(smem_raw);       // exchange [N][TT]
    cx<T>* obuf = sbuf + (size_t)N * TT;                     // output [N][TT]
    cx<T>* slab0 = obuf + (size_t)N * TT;                    // [2][SR][TT]
    uint64_t* bars = reinterpret_cast<uint64_t*>(slab0 + 2 * (size_t)SR * TT);
    const int tid = threadIdx.x;
    const int t = tid % TT, p = tid / TT;
    const int items = nvalid * cnt;
    const T scale = T(1) / (T(N) * T(N) * T(N));
    const long long budget = sd[0].wait_cycles > 0 ? sd[0].wait_cycles : kWaitCycles;
    StridedIdx<TT, PL::R1> sidx{t};
    SyncBlock sync;

    // thread 0: component c of item `it` into slab sl
    auto issue = [&](int it, int c, int sl) {
        int m, ky, kz0;
        xtile_item(xitems, nvalid, it, G::KC, TT, m, ky, kz0);
        const int j = ky < 0 ? ky + N : ky;
        const int r2 = G::KC2 - ky * ky - kz0 * kz0;
        int kxm = (int)sqrtf((float)r2);
        while (kxm * kxm > r2) --kxm;
        while ((kxm + 1) * (kxm + 1) <= r2) ++kxm;
        const int nb = kxm / XB + 1;   // boxes covering the rows kx = 0 .. kxm
        cx<T>* dst = slab0 + (size_t)sl * SR * TT;
        const int cc = c0 + 3 * m + c;
        fence_proxy_async_smem();
        if (SR == N && 2 * nb * XB >= N) {
            mbar_arrive_expect_tx(&bars[sl], (uint32_t)(N / XB) * BOX_BYTES);
            for (int b = 0; b < N / XB; ++b) tensor4_g2s(dst + (size_t)b * XB * TT, &map, 2 * kz0, j, b * XB, cc, &bars[sl]);
        } else {
            mbar_arrive_expect_tx(&bars[sl], (uint32_t)(2 * nb) * BOX_BYTES);
            for (int b = 0; b < nb; ++b) {
                const int r_lo = b * XB, r_hi = N - (b + 1) * XB;
                tensor4_g2s(dst + (size_t)r_lo * TT, &map, 2 * kz0, j, r_lo, cc, &bars[sl]);
                tensor4_g2s(dst + (size_t)(r_hi - (N - SR)) * TT, &map, 2 * kz0, j, r_hi, cc, &bars[sl]);
            }
        }
    };

    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    int it = blockIdx.x;
    int sx = 0, sy = 1;       // slabs holding this item's ux and uy
    uint32_t ph = 0u;         // bit sl: parity of the next completion of slab sl
    uint32_t pend = 0u;       // thread 0: slabs with a copy in flight
    if (tid == 0 && it < items) {
        issue(it, 0, sx);
        issue(it, 1, sy);
        pend = 3u;
    }
    // bounded wait of every thread on slab sl; the CTA agrees on the outcome
    auto wait = [&](int sl) -> bool {
        const bool ok = __syncthreads_and(mbar_wait(&bars[sl], (ph >> sl) & 1u, budget) ? 1 : 0) != 0;
        if (ok) {
            ph ^= 1u << sl;
            pend &= ~(1u << sl);
        }
        return ok;
    };
    auto fail = [&](int m) {
        if (tid == 0) {
            atomicExch(&sd[m].status, kStatusTimeout);
            for (int sl = 0; sl < 2; ++sl)
                if (pend & (1u << sl)) (void)mbar_wait(&bars[sl], (ph >> sl) & 1u, kWaitCycles);
            bulk_wait_all();
        }
    };

    while (it < items) {
        int m, ky, kz0;
        xtile_item(xitems, nvalid, it, G::KC, TT, m, ky, kz0);
        const int kz = kz0 + t;
        const int j = ky < 0 ? ky + N : ky;
        const bool colok = (kz <= G::KC) && (ky * ky + kz * kz <= G::KC2);
        const int rem = G::KC2 - ky * ky - kz * kz;
        const int nx = it + (int)gridDim.x;
        auto read = [&](int sl, cx<T>(&v)[E]) {
            const cx<T>* src = slab0 + (size_t)sl * SR * TT + t;
#pragma unroll
            for (int s = 0; s < E; ++s) {
                const int r = p + P * s;
                const int kx = kof<N>(r);
                const bool in = colok && kx * kx <= rem;
                const int sr = !in ? 0 : (r < N / 2 ? r : r - (N - SR));   // slab row of x row r
                v[s] = in ? src[(size_t)sr * TT] * scale : czero<T>();
            }
        };
        auto ikx = [&](cx<T>(&v)[E]) {
#pragma unroll
            for (int s = 0; s < E; ++s) v[s] = mul_i(v[s]) * T(kof<N>(p + P * s));
        };
        // field f of the tile (every x row, the TT columns; zero outside the circle)
        // through the output buffer and bulk tensor stores: the buffer is free once
        // the previous stores have read it
        auto store = [&](int f, const cx<T>(&v)[E]) {
            if (tid == 0) bulk_wait_read_all();
            __syncthreads();
#pragma unroll
            for (int s = 0; s < E; ++s) obuf[(size_t)(p + P * s) * TT + t] = v[s];
            fence_proxy_async_smem();
            __syncthreads();
            if (tid == 0) {
                for (int b = 0; b < N / XO; ++b)
                    tensor4_s2g(&wmap, obuf + (size_t)b * XO * TT, 2 * kz0, j, b * XO, cw + 6 * m + f);
                bulk_commit();
            }
        };
        const T fky = T(ky), fkz = T(kz);
        cx<T> X[E], Y[E], B[E];
        if (!wait(sx) || !wait(sy)) {
            fail(m);
            return;
        }
        read(sx, X);
        read(sy, Y);
        __syncthreads();   // both slabs read: this item's uz, the next item's ux
        if (tid == 0) {
            issue(it, 2, sx);
            pend |= 1u << sx;
            if (nx < items) {
                issue(nx, 0, sy);
                pend |= 1u << sy;
            }
        }
        // ux; wz = T(i kx uy) - i ky T(ux)
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = Y[s];
        ikx(B);
        PL::inv(B, sbuf, p, tw, sidx, sync);
        PL::inv(X, sbuf, p, tw, sidx, sync);
        store(0, X);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = B[s] - mul_i(X[s]) * fky;
        store(5, B);
        // wy = i kz T(ux) - T(i kx uz)
        if (!wait(sx)) {
            fail(m);
            return;
        }
        read(sx, B);
        ikx(B);
        PL::inv(B, sbuf, p, tw, sidx, sync);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fkz - B[s];
        store(4, B);
        // uz (its slab then takes the next item's uy), uy, wx = i ky T(uz) - i kz T(uy)
        read(sx, X);
        __syncthreads();
        if (tid == 0 && nx < items) {
            issue(nx, 1, sx);
            pend |= 1u << sx;
        }
        PL::inv(X, sbuf, p, tw, sidx, sync);
        store(2, X);
        PL::inv(Y, sbuf, p, tw, sidx, sync);
        store(1, Y);
#pragma unroll
        for (int s = 0; s < E; ++s) B[s] = mul_i(X[s]) * fky - mul_i(Y[s]) * fkz;
        store(3, B);
        const int tmp = sx;
        sx = sy;
        sy = tmp;
        it = nx;
    }
    // the bulk stores complete before the CTA exits
    if (tid == 0) bulk_wait_all();
}
// ---------------------------------------------------------------------------
// P2 / P4: FFT along y, in place. grid (ntile, N, nfields).
// Inverse: inputs only where ky^2 + kz^2 <= KC^2, outputs every y.
// Forward: inputs every y, outputs only where ky^2 + kz^2 <= KC^2.
// ---------------------------------------------------------------------------
// CTAs per SM the y pass is compiled for: 1024 threads per SM (64 registers per
// thread), 512 (128 registers) for plans of more than 16 elements per thread
template <typename T, int N, int V, bool INV> constexpr int ypass_minb() {
    constexpr int nt = tile_a<T, N, V, INV>() * YPlan<T, N, INV>::A::P;
    constexpr int per_sm = YPlan<T, N, INV>::A::E > 16 ? 512 : 1024;
    return per_sm / nt > 0 ? per_sm / nt : 1;
}
template <typename T, int N, bool INV, int V = 0>
__global__ void __launch_bounds__(tile_a<T, N, V, INV>() * YPlan<T, N, INV>::A::P, ypass_minb<T, N, V, INV>())
k_ypass(cx<T>* __restrict__ W, const cx<T>* __restrict__ tw) {
    using G = Geo<N>;
    using PL = typename YPlan<T, N, INV>::A;
    constexpr int TT = tile_a<T, N, V, INV>();
    constexpr int E = PL::E, P = PL::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* sbuf = reinterpret_cast<cx<T>*>(smem_raw);
    const int t = threadIdx.x % TT, p = threadIdx.x / TT;
    const int kz = blockIdx.x * TT + t;
    const bool colok = kz <= G::KC;
    const int rem = G::KC2 - kz * kz;
    // blockIdx.z = member * (fields per member) + field: 6 fields inverse, the first 3 forward
    constexpr int NF = INV ? 6 : 3;
    const long long fld = (long long)(blockIdx.z / NF) * 6 + blockIdx.z % NF;
    cx<T>* base = W + fld * G::FS + (long long)blockIdx.y * N * G::NZP + kz;
    StridedIdx<TT, PL::R1> sidx{t};
    SyncBlock sync;
    cx<T> v[E];
#pragma unroll
    for (int s = 0; s < E; ++s) {
        const int jj = p + P * s;
        const int ky = kof<N>(jj);
        bool in = colok;
        if (INV) in = in && (ky * ky <= rem);
        v[s] = in ? base[(long long)jj * G::NZP] : czero<T>();
    }
    if (INV) PL::template inv<true>(v, sbuf, p, tw, sidx, sync);
    else PL::template fwd<true>(v, sbuf, p, tw, sidx, sync);
    if (colok) {
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int jj = p + P * s;
            const int ky = kof<N>(jj);
            if (INV || ky * ky <= rem) base[(long long)jj * G::NZP] = v[s];
        }
    }
}

// ---------------------------------------------------------------------------
// P3: z lines. MODE 0: c2r(6) -> u x w -> r2c(3) (fused hot path);
// MODE 1: c2r(6) -> real out [6][N][N][N]; MODE 2: real in [3][N][N][N] -> r2c(3).
// A CTA takes ZP line pairs; thread groups g = 0..2 each own one complex FFT.
// c2r packs two real lines into one complex transform (fields 2g, 2g+1);
// r2c packs (Nx_a + i Ny_a), (Nx_b + i Ny_b), (Nz_a + i Nz_b) and separates the
// spectra with Z[m] and conj(Z[N-m]).
// ---------------------------------------------------------------------------
template <typename T> struct Bits;
template <> struct Bits<float> {
    __device__ static void amax(unsigned long long* p, float v) {
        atomicMax(reinterpret_cast<unsigned int*>(p), __float_as_uint(v));
    }
};
template <> struct Bits<double> {
    __device__ static void amax(unsigned long long* p, double v) {
        atomicMax(p, (unsigned long long)__double_as_longlong(v));
    }
};

template <int N> constexpr int zpad() { return N + (N >> 4); }

template <typename T, int N, int MODE>
__global__ void __launch_bounds__(3 * Plans<N>::A::P * zpairs<N>())
k_zpass(cx<T>* __restrict__ W, const cx<T>* __restrict__ tw, T* __restrict__ real,
        StepDev* __restrict__ sd, int want_umax) {
    using G = Geo<N>;
    using PL = typename Plans<N>::A;
    constexpr int E = PL::E, P = PL::P, ZP = zpairs<N>();
    constexpr int XS = zpad<N>();
    // ensemble member (blockIdx.y); the real-space modes handle one member only
    W += (long long)blockIdx.y * 6 * G::FS;
    unsigned long long* umax_bits = sd ? &sd[blockIdx.y].umax_bits : nullptr;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* xbuf = reinterpret_cast<cx<T>*>(smem_raw);                       // [ZP][3][XS]
    T* R = reinterpret_cast<T*>(smem_raw + sizeof(cx<T>) * ZP * 3 * XS);     // [ZP][2][6][N]
    const int p = threadIdx.x % P;
    const int g = (threadIdx.x / P) % 3;
    const int lp = threadIdx.x / (3 * P);
    const long long pair = (long long)blockIdx.x * ZP + lp;
    const long long la = 2 * pair;
    cx<T>* sb = xbuf + (lp * 3 + g) * XS;
    T* Rl = R + (long long)lp * 12 * N;   // [2][6][N]
    PaddedIdx sidx;
    SyncBlock sync;
    constexpr long long NL = (long long)N * N;   // lines

    if (MODE == 0 || MODE == 1) {
#pragma unroll 1
        for (int L = 0; L < 2; ++L) {
            const cx<T>* A = W + (long long)(2 * g) * G::FS + (la + L) * G::NZP;
            const cx<T>* B = W + (long long)(2 * g + 1) * G::FS + (la + L) * G::NZP;
            cx<T> v[E];
#pragma unroll
            for (int s = 0; s < E; ++s) {
                const int m = p + P * s;
                cx<T> z = czero<T>();
                if (m == 0) {
                    z = mk(A[0].x, B[0].x);
                } else if (m <= G::KC) {
                    cx<T> a = A[m], b = B[m];
                    z = mk(a.x - b.y, a.y + b.x);
                } else if (m >= N - G::KC) {
                    cx<T> a = A[N - m], b = B[N - m];
                    z = mk(a.x + b.y, b.x - a.y);
                }
                v[s] = z;
            }
            PL::inv(v, sb, p, tw, sidx, sync);
            T* ra = Rl + (L * 6 + 2 * g) * N;
            T* rb = ra + N;
#pragma unroll
            for (int s = 0; s < E; ++s) {
                ra[p + P * s] = v[s].x;
                rb[p + P * s] = v[s].y;
            }
        }
        __syncthreads();
        if (MODE == 1) {
            // real out: [6][N*N lines][N]
            for (int idx = threadIdx.x; idx < ZP * 12 * N; idx += blockDim.x) {
                const int lpp = idx / (12 * N);
                const int rem = idx % (12 * N);
                const int L = rem / (6 * N);
                const int f = (rem / N) % 6;
                const int n = rem % N;
                const long long line = 2 * ((long long)blockIdx.x * ZP + lpp) + L;
                real[(long long)f * NL * N + line * N + n] = R[(long long)lpp * 12 * N + (L * 6 + f) * N + n];
            }
            return;
        }
        // u x w in place over the u slots; CFL bound on the true velocity
        T um = T(0);
        for (int idx = threadIdx.x; idx < ZP * 2 * N; idx += blockDim.x) {
            const int lpp = idx / (2 * N);
            const int L = (idx / N) % 2;
            const int n = idx % N;
            T* r = R + (long long)lpp * 12 * N + L * 6 * N + n;
            const T u0 = r[0], u1 = r[N], u2 = r[2 * N];
            const T w0 = r[3 * N], w1 = r[4 * N], w2 = r[5 * N];
            r[0] = u1 * w2 - u2 * w1;
            r[N] = u2 * w0 - u0 * w2;
            r[2 * N] = u0 * w1 - u1 * w0;
            um = fmax(um, fabs(u0) + fabs(u1) + fabs(u2));
        }
        if (want_umax) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) um = fmax(um, __shfl_xor_sync(0xffffffffu, um, o));
            if ((threadIdx.x & 31) == 0) Bits<T>::amax(umax_bits, um);
        }
        __syncthreads();
    } else {
        // MODE 2: real fields in
        for (int idx = threadIdx.x; idx < ZP * 6 * N; idx += blockDim.x) {
            const int lpp = idx / (6 * N);
            const int rem = idx % (6 * N);
            const int L = rem / (3 * N);
            const int f = (rem / N) % 3;
            const int n = rem % N;
            const long long line = 2 * ((long long)blockIdx.x * ZP + lpp) + L;
            R[(long long)lpp * 12 * N + (L * 6 + f) * N + n] = real[(long long)f * NL * N + line * N + n];
        }
        __syncthreads();
    }

    // forward: group 0 -> line a (Nx + i Ny), 1 -> line b, 2 -> Nz_a + i Nz_b
    {
        const T* ra;
        const T* rb;
        if (g == 0) { ra = Rl; rb = Rl + N; }
        else if (g == 1) { ra = Rl + 6 * N; rb = Rl + 7 * N; }
        else { ra = Rl + 2 * N; rb = Rl + 8 * N; }
        cx<T> v[E];
#pragma unroll
        for (int s = 0; s < E; ++s) v[s] = mk(ra[p + P * s], rb[p + P * s]);
        PL::fwd(v, sb, p, tw, sidx, sync);
#pragma unroll
        for (int s = 0; s < E; ++s) sb[sidx(p + P * s)] = v[s];
        __syncthreads();
        cx<T>* outA;
        cx<T>* outB;
        if (g == 0) { outA = W + la * G::NZP; outB = W + G::FS + la * G::NZP; }
        else if (g == 1) { outA = W + (la + 1) * G::NZP; outB = W + G::FS + (la + 1) * G::NZP; }
        else { outA = W + 2 * G::FS + la * G::NZP; outB = W + 2 * G::FS + (la + 1) * G::NZP; }
        const T half = T(0.5);
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int m = p + P * s;
            if (m <= G::KC) {
                const cx<T> zm = sb[sidx(m)];
                const cx<T> zc = conjg(sb[sidx((N - m) % N)]);
                const cx<T> sum = zm + zc, dif = zm - zc;
                outA[m] = sum * half;
                outB[m] = mk(dif.y * half, -dif.x * half);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// P3, line-per-group form (FP32, P <= 32), persistent and fed by bulk
// asynchronous copies. A group of P = N/E lanes inside one warp owns a z line.
// Each warp walks its own sequence of line groups; lane 0 copies the next
// group's six field lines (cp.async.bulk, completion on an mbarrier) into the
// other half of a two-stage shared-memory buffer while the warp transforms the
// current group: three inverse complex FFTs (ux + i uy, uz + i wx, wy + i wz),
// u x w on the six real fields held in registers, then two forward FFTs:
// Nx + i Ny (separated through the group's exchange buffer) and Nz alone (a
// real input, whose first KC+1 outputs are the spectrum directly). Exchanges
// are warp-synchronous, so warps never wait on each other.
// ---------------------------------------------------------------------------
struct SyncWarp {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
// the GW warps that share one z line: named barrier `id` over their 32 GW threads
struct SyncGroup {
    int id, nthreads;
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
    }
};
constexpr int ZLINE_WARPS = 4;

// A line group is the lanes that transform one z line: P = N/E lanes. With
// P <= 32 a warp holds 32/P lines (GPW); with P = 64 (N = 1024) two warps hold
// one line (GW = 2) and exchange through a named barrier.
// the line kernel's plan: the y-pass plan (at 512^3 two warps per line with 8
// elements per lane, 128 registers and twice the warps per SM, measured 8 %
// slower than one warp with 16 elements)
template <int N> struct ZPlan { using A = typename Plans<N>::A; };
template <int N> constexpr int zline_gw() { return ZPlan<N>::A::P > 32 ? ZPlan<N>::A::P / 32 : 1; }
template <int N> constexpr int zline_gpw() { return ZPlan<N>::A::P <= 32 ? 32 / ZPlan<N>::A::P : 1; }
// the real Nz line as a half-length complex transform (a plan of N/2 points on the
// same lanes with half the elements) where it measured faster: the 512-point lines
// of one warp (1.183 -> 1.168 ms per pass at 512^3). Slower elsewhere: 256 points,
// two lines per warp, 0.123 -> 0.140 ms; 1024 points, two warps per line, 10.86 ->
// 11.57 ms.
template <int N> constexpr bool zline_half_nz() {
    if constexpr (N != 512) {
        return false;
    } else {
        using HP = typename Plans<N / 2>::X;
        return HP::P == ZPlan<N>::A::P && 2 * HP::E == ZPlan<N>::A::E;
    }
}
template <typename T, int N>
constexpr bool zline_ok() {
    constexpr int P = ZPlan<N>::A::P;
    return sizeof(T) == 4 && ZPlan<N>::A::E <= 16 &&
           (P <= 32 ? (32 % P == 0 && ((long long)N * N) % (32 / P) == 0) : P == 64);
}
// With several lines per warp (N <= 256) the exchange buffers live in the
// stage buffer whose lines are already in registers, which cuts shared memory
// per warp by a fifth (3 CTAs per SM instead of 2 at 168 registers); 512- and
// 1024-point lines (16 elements per lane, over 200 registers) keep their own.
template <int N> constexpr bool zline_xbuf_in_stage() { return zline_gpw<N>() > 1; }
template <int N> constexpr int zline_stage_elems() {
    constexpr int a = zline_gpw<N>() * 6 * Geo<N>::NZP, b = zline_gpw<N>() * zpad<N>();
    return ((zline_xbuf_in_stage<N>() && b > a ? b : a) + 15) / 16 * 16;
}
// complex elements of shared memory per line group: two stage buffers (+ the exchange buffers)
template <typename T, int N> constexpr int zline_group_elems() {
    return 2 * zline_stage_elems<N>() +
           (zline_xbuf_in_stage<N>() ? 0 : (zline_gpw<N>() * zpad<N>() + 15) / 16 * 16);
}
// line groups per CTA
template <int N> constexpr int zline_groups() { return ZLINE_WARPS / zline_gw<N>(); }
// shared memory: the groups' buffers, two mbarriers per group, one vote word per warp
template <typename T, int N> constexpr size_t zline_smem() {
    return sizeof(cx<T>) * (size_t)zline_groups<N>() * zline_group_elems<T, N>() + 16 * zline_groups<N>() +
           4 * ZLINE_WARPS;
}

template <typename T, int N>
__global__ void __launch_bounds__(ZLINE_WARPS * 32, zline_xbuf_in_stage<N>() ? 3 : 2)
k_zline(cx<T>* __restrict__ W, const cx<T>* __restrict__ tw, StepDev* __restrict__ sd, int want_umax,
        int nmem) {
    using G = Geo<N>;
    using PL = typename ZPlan<N>::A;
    constexpr int E = PL::E, P = PL::P, GPW = zline_gpw<N>(), GW = zline_gw<N>(), GT = 32 * GW;
    // FP32x2 butterfly additions where a line fills one warp or more (512 points:
    // 4 % faster; 1024 points: 2.6 %); the 256-point lines of two per warp need
    // the registers for three CTAs per SM
    constexpr bool kPK = GPW == 1;
    constexpr int NGRP = zline_groups<N>();
    constexpr int NZP = G::NZP;
    constexpr long long NG = (long long)N * N / GPW;   // work items (line groups) per ensemble member
    constexpr int SE = zline_stage_elems<N>();         // elements per stage buffer
    constexpr uint32_t STAGE_BYTES = GPW * 6 * NZP * sizeof(cx<T>);   // bytes copied per stage
    constexpr uint32_t LINE_BYTES = NZP * sizeof(cx<T>);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int gt = threadIdx.x % GT, grp = threadIdx.x / GT;   // thread within its line group, group
    const int p = gt % P, gi = gt / P;
    cx<T>* wbase = reinterpret_cast<cx<T>*>(smem_raw) + (size_t)grp * zline_group_elems<T, N>();
    cx<T>* stage[2] = {wbase, wbase + SE};
    uint64_t* bars_all = reinterpret_cast<uint64_t*>(smem_raw + sizeof(cx<T>) * (size_t)NGRP * zline_group_elems<T, N>());
    uint64_t* bars = bars_all + 2 * grp;
    int* votes = reinterpret_cast<int*>(bars_all + 2 * NGRP) + grp * GW;   // one word per warp of the group
    PaddedIdx sidx;
    using Sync = typename std::conditional<(GW > 1), SyncGroup, SyncWarp>::type;
    Sync sync{};
    if constexpr (GW > 1) sync = Sync{1 + grp, GT};

    if (gt == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    sync();
    auto issue = [&](long long g, int s) {
        if (gt == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&bars[s], STAGE_BYTES);
            const long long m = g / NG, gl = g % NG;
            for (int l = 0; l < GPW; ++l)
                for (int f = 0; f < 6; ++f)
                    bulk_g2s(stage[s] + (l * 6 + f) * NZP, W + (m * 6 + f) * G::FS + (gl * GPW + l) * NZP,
                             LINE_BYTES, &bars[s]);
        }
    };

    const long long nw = (long long)gridDim.x * NGRP;
    long long g = (long long)blockIdx.x * NGRP + grp;
    const long long NGT = NG * nmem;   // work items over all members
    uint32_t phase = 0;                // bit s = parity to wait for on stage s
    T um = T(0);
    long long cur = -1;                // member whose speed bound um holds
    auto flush_umax = [&]() {
        if (want_umax && cur >= 0) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) um = fmaxf(um, __shfl_xor_sync(0xffffffffu, um, o));
            if (lane == 0) Bits<T>::amax(&sd[cur].umax_bits, um);
        }
        um = T(0);
    };
    int s = 0;
    const long long budget = sd[0].wait_cycles > 0 ? sd[0].wait_cycles : kWaitCycles;
    if (g < NGT) issue(g, 0);
    for (; g < NGT; g += nw, s ^= 1) {
        const bool more = g + nw < NGT;
        if (more) issue(g + nw, s ^ 1);
        // every thread waits (bounded) for the copies; the group agrees on the outcome
        const uint32_t par = (phase >> s) & 1u;
        bool ok = __all_sync(0xffffffffu, mbar_wait(&bars[s], par, budget));
        if constexpr (GW > 1) {
            if (lane == 0) votes[gt >> 5] = ok ? 1 : 0;
            sync();
#pragma unroll
            for (int w = 0; w < GW; ++w) ok = ok && votes[w] != 0;
            sync();   // votes read before they are written again
        }
        phase ^= 1u << s;
        if (!ok) {
            // record the timeout; let the copies of both stages still in flight
            // land (full budget) before the CTA and its shared memory go away
            (void)mbar_wait(&bars[s], par, kWaitCycles);
            if (more) (void)mbar_wait(&bars[s ^ 1], (phase >> (s ^ 1)) & 1u, kWaitCycles);
            if (gt == 0) atomicExch(&sd[g / NG].status, kStatusTimeout);
            return;
        }
        const long long mem = g / NG;
        if (mem != cur) {
            flush_umax();
            cur = mem;
        }
        cx<T>* Wm = W + mem * 6 * G::FS;
        const cx<T>* in = stage[s] + gi * 6 * NZP;
        const long long line = (g % NG) * GPW + gi;
        // exchange buffer of this group (in the stage buffer once its lines are in registers)
        cx<T>* sb = (zline_xbuf_in_stage<N>() ? stage[s] : wbase + 2 * SE) + gi * zpad<N>();

        auto load_pair = [&](int f, cx<T>(&v)[E]) {
            const cx<T>* A = in + f * NZP;
            const cx<T>* B = A + NZP;
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int m = p + P * q;
                cx<T> z = czero<T>();
                if (P * q > G::KC && P * q + P - 1 < N - G::KC) {
                    // every lane's mode of this slot is outside the kept band
                } else if (m == 0) {
                    z = mk(A[0].x, B[0].x);
                } else if (m <= G::KC) {
                    const cx<T> a = A[m], b = B[m];
                    z = mk(a.x - b.y, a.y + b.x);
                } else if (m >= N - G::KC) {
                    const cx<T> a = A[N - m], b = B[N - m];
                    z = mk(a.x + b.y, b.x - a.y);
                }
                v[q] = z;
            }
        };

        cx<T> V1[E], V2[E], V3[E];
        load_pair(0, V1);
        load_pair(2, V2);
        load_pair(4, V3);
        sync();   // every lane has read the staged lines before the buffer is reused
        PL::template inv<kPK>(V1, sb, p, tw, sidx, sync);
        PL::template inv<kPK>(V2, sb, p, tw, sidx, sync);
        PL::template inv<kPK>(V3, sb, p, tw, sidx, sync);
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const T ux = V1[q].x, uy = V1[q].y, uz = V2[q].x;
            const T wx = V2[q].y, wy = V3[q].x, wz = V3[q].y;
            um = fmaxf(um, fabsf(ux) + fabsf(uy) + fabsf(uz));
            V1[q] = mk(uy * wz - uz * wy, uz * wx - ux * wz);
            V2[q] = mk(ux * wy - uy * wx, T(0));
        }
        // Nx + i Ny -> two spectra through the exchange buffer
        PL::template fwd<kPK>(V1, sb, p, tw, sidx, sync);
#pragma unroll
        for (int q = 0; q < E; ++q)   // only the slots read below: m <= KC and N - m
            if (P * q <= G::KC || P * q + P - 1 >= N - G::KC) sb[sidx(p + P * q)] = V1[q];
        sync();
        {
            cx<T>* outA = Wm + line * NZP;
            cx<T>* outB = outA + G::FS;
            const T half = T(0.5);
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int m = p + P * q;
                if (m <= G::KC) {
                    const cx<T> zm = sb[sidx(m)];
                    const cx<T> zc = conjg(sb[sidx((N - m) % N)]);
                    const cx<T> sum = zm + zc, dif = zm - zc;
                    outA[m] = sum * half;
                    outB[m] = mk(dif.y * half, -dif.x * half);
                }
            }
        }
        sync();
        cx<T>* outC = Wm + 2 * G::FS + line * NZP;
        if constexpr (zline_half_nz<N>()) {
            // Nz (real input) by a half-length transform: z[n] = Nz[2n] + i Nz[2n + 1]
            // (the real line through the exchange buffer), Z = DFT_{N/2}(z) with every
            // second twiddle of the N table, then for k <= KC
            //   X[k] = (Z[k] + conj Z[N/2 - k]) / 2 - i W_N^k (Z[k] - conj Z[N/2 - k]) / 2
            using HP = typename Plans<N / 2>::X;
            constexpr int EH = HP::E, M2 = N / 2;
            T* sr = reinterpret_cast<T*>(sb);
#pragma unroll
            for (int q = 0; q < E; ++q) sr[p + P * q] = V2[q].x;
            sync();
            cx<T> Z[EH];
#pragma unroll
            for (int q = 0; q < EH; ++q) Z[q] = reinterpret_cast<const cx<T>*>(sr)[p + P * q];
            sync();
            HP::template fwd<kPK, 2>(Z, sb, p, tw, sidx, sync);
#pragma unroll
            for (int q = 0; q < EH; ++q) sb[sidx(p + P * q)] = Z[q];
            sync();
            const T half = T(0.5);
#pragma unroll
            for (int q = 0; q < EH; ++q) {
                const int k = p + P * q;
                if (P * q <= G::KC && k <= G::KC) {
                    const cx<T> zc = conjg(sb[sidx((M2 - k) % M2)]);
                    const cx<T> e = (Z[q] + zc) * half, d = (Z[q] - zc) * half;
                    const cx<T> wd = cmul(ldg(&tw[k]), d);
                    outC[k] = mk(e.x + wd.y, e.y - wd.x);
                }
            }
        } else {
            // Nz (real input): its spectrum is the transform itself
            PL::template fwd<kPK>(V2, sb, p, tw, sidx, sync);
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int m = p + P * q;
                if (P * q <= G::KC && m <= G::KC) outC[m] = V2[q];
            }
        }
        // the stage buffer is refilled by a bulk copy (async proxy) next iteration:
        // order every lane's exchange accesses to it before that
        fence_proxy_async_smem();
        sync();
    }
    flush_umax();
}
// The stage epilogue reads the state of each of its modes after the FFT. Its
// rows (TT modes of one x row, per array and component: one 16-byte aligned
// segment each) are prefetched into L2 before the FFT, spread over the TT
// threads of a row, so that those loads hit L2. Tile (ky, kz0 .. kz0 + TT).
template <typename T, int N, int INTEG, int MODE, int E, int P, int TT>
__device__ __forceinline__ void xfwd_prefetch_state(const cx<T>* U, const cx<T>* ACC, const cx<T>* K,
                                                    const RkStage& rs, int p, int t, int ky, int kz0, int j) {
    if constexpr (MODE <= X_STAGE4) {
        using G = Geo<N>;
        const long long xs = (long long)N * G::NZP;
        const int rem0 = G::KC2 - ky * ky - kz0 * kz0;
        const uint32_t seg = (uint32_t)((TT < G::NZP - kz0 ? TT : G::NZP - kz0) * sizeof(cx<T>));
        constexpr bool kIF = INTEG == INT_IFRK4;
        constexpr bool needU = !(kIF && MODE == X_STAGE4);
        constexpr bool needA = INTEG != INT_TAB && MODE != X_STAGE1;
        for (int s = t; s < E; s += TT) {
            const int kx = kof<N>(p + P * s);
            if (kx * kx > rem0) continue;
            const long long q = (long long)(p + P * s) * xs + (long long)j * G::NZP + kz0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (needU) bulk_prefetch_l2(U + c * G::FS + q, seg);
                if (needA) bulk_prefetch_l2(ACC + c * G::FS + q, seg);
                if constexpr (INTEG == INT_TAB) {
                    for (int jj = 0; jj < rs.nk && jj < 6; ++jj)
                        if (rs.c[jj] != 0.0 || rs.e[jj] != 0.0)
                            bulk_prefetch_l2(K + (long long)jj * 3 * G::FS + c * G::FS + q, seg);
                }
            }
        }
    }
}
// RK4-family stage epilogue (IF-RK4, RK4CN) of one thread's E modes, the x rows
// p + P s of the column (ky, kz) inside the sphere: the Leray projection of every
// mode first, then, in chunks of up to 8 modes and per component, the chunk's
// state loads before their updates, so that a chunk's loads (per array) are in
// flight at once.
template <typename T, int N, int INTEG, int MODE, int E, int P>
__device__ __forceinline__ void xfwd_rk4_epilogue(cx<T> (&F)[3][E], int p, int ky, int kz, long long off,
                                                  cx<T>* __restrict__ U, cx<T>* __restrict__ UT,
                                                  cx<T>* __restrict__ ACC, const cx<T>* __restrict__ tab,
                                                  const StepDev* __restrict__ sd, const cx<T>* __restrict__ sgs, T h) {
    using G = Geo<N>;
    const long long xs = (long long)N * G::NZP;
    const int rem = G::KC2 - ky * ky - kz * kz;
    constexpr int CH = E > 8 ? 4 : E;
    unsigned valid = 0u;
    int k2s[E];
#pragma unroll
    for (int s = 0; s < E; ++s) {
        const int i = p + P * s;
        const int kx = kof<N>(i);
        k2s[s] = 0;
        if (kx * kx > rem) continue;
        valid |= 1u << s;
        const int k2 = kx * kx + ky * ky + kz * kz;
        cx<T> n0 = F[0][s], n1 = F[1][s], n2 = F[2][s];
        if (sgs && sd->sgs_on) {
            // learned subgrid term -div(tau), single run only (member 0)
            const long long q = (long long)i * xs + off;
            n0 = n0 + sgs[q];
            n1 = n1 + sgs[G::FS + q];
            n2 = n2 + sgs[2 * G::FS + q];
        }
        if (k2 > 0) {
            const T kinv = T(1) / T(k2);
            const cx<T> kdn = n0 * T(kx) + n1 * T(ky) + n2 * T(kz);
            n0 = n0 - kdn * (T(kx) * kinv);
            n1 = n1 - kdn * (T(ky) * kinv);
            n2 = n2 - kdn * (T(kz) * kinv);
        } else {
            n0 = n1 = n2 = czero<T>();
        }
        F[0][s] = n0;
        F[1][s] = n1;
        F[2][s] = n2;
        k2s[s] = k2;
    }
    constexpr bool kIF = INTEG == INT_IFRK4;
    constexpr bool needU = !(kIF && MODE == X_STAGE4);
    constexpr bool needA = kIF ? (MODE != X_STAGE1) : (MODE != X_STAGE1);
#pragma unroll
    for (int s0 = 0; s0 < E; s0 += CH) {
      if (!((valid >> s0) & ((1u << CH) - 1u))) continue;
      cx<T> tb[CH];
#pragma unroll
      for (int s = 0; s < CH; ++s) tb[s] = ldg(&tab[k2s[s0 + s]]);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cx<T> u[CH], a[CH];
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            u[s] = czero<T>();
            a[s] = czero<T>();
            if (!((valid >> (s0 + s)) & 1u)) continue;
            const long long q = c * G::FS + (long long)(p + P * (s0 + s)) * xs + off;
            if (needU) u[s] = U[q];
            if (needA) a[s] = ACC[q];
        }
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            if (!((valid >> (s0 + s)) & 1u)) continue;
            const long long q = c * G::FS + (long long)(p + P * (s0 + s)) * xs + off;
            const cx<T> nn = F[c][s0 + s];
            if constexpr (kIF) {
                const T Eh = tb[s].x, Ef = tb[s].y;
                if (MODE == X_STAGE1) {
                    UT[q] = (u[s] + nn * (h * T(0.5))) * Eh;
                    ACC[q] = (u[s] + nn * (h / T(6))) * Ef;
                } else if (MODE == X_STAGE2) {
                    UT[q] = u[s] * Eh + nn * (h * T(0.5));
                    ACC[q] = a[s] + nn * (h / T(3) * Eh);
                } else if (MODE == X_STAGE3) {
                    UT[q] = u[s] * Ef + nn * (h * Eh);
                    ACC[q] = a[s] + nn * (h / T(3) * Eh);
                } else {
                    U[q] = a[s] + nn * (h / T(6));
                }
            } else {
                if (MODE == X_STAGE1) {
                    UT[q] = u[s] + nn * (h * T(0.5));
                    ACC[q] = nn * (T(1) / T(6));
                } else if (MODE == X_STAGE2) {
                    UT[q] = u[s] + nn * (h * T(0.5));
                    ACC[q] = a[s] + nn * (T(1) / T(3));
                } else if (MODE == X_STAGE3) {
                    UT[q] = u[s] + nn * h;
                    ACC[q] = a[s] + nn * (T(1) / T(3));
                } else {
                    U[q] = u[s] * tb[s].x + (a[s] + nn * (T(1) / T(6))) * tb[s].y;
                }
            }
        }
      }
    }
}
// ---------------------------------------------------------------------------
// P5: forward FFT along x of the 3 product fields, then per mode the Leray
// projection, dealias mask and RK stage update. grid (ntile, NKY).
// tab[k2] holds (E_half, E_full) for IF-RK4 or (a, b) = ((2-D)/(2+D),
// 2h/(2+D)) for the Crank-Nicolson updates, computed in FP64 and rounded to
// T. INTEG = INT_TAB runs the RkStage epilogue of the RK5 family; its DP5CN
// error partial sums go to dpart[member][block][3] in a fixed order.
// ---------------------------------------------------------------------------
template <typename T, int N, int INTEG, int MODE, int V = 0>
__global__ void __launch_bounds__(tile_x<T, N, V, true>() * PlansV<N, V>::X::P, TileVar<V>::MINB)
k_xfwd(const cx<T>* __restrict__ W, cx<T>* __restrict__ U, cx<T>* __restrict__ UT,
       cx<T>* __restrict__ ACC, const cx<T>* __restrict__ tw, const StepDev* __restrict__ sd,
       const cx<T>* __restrict__ tab, const cx<T>* __restrict__ sgs, cx<T>* __restrict__ K,
       double* __restrict__ dpart, const RkStage rs) {
    using G = Geo<N>;
    using PL = typename PlansV<N, V>::X;
    constexpr int TT = tile_x<T, N, V, true>();
    constexpr int E = PL::E, P = PL::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* sbuf = reinterpret_cast<cx<T>*>(smem_raw);
    const int t = threadIdx.x % TT, p = threadIdx.x / TT;
    const int kz = blockIdx.x * TT + t;
    const int ky = (int)blockIdx.y - G::KC;
    const int j = ky < 0 ? ky + N : ky;
    // ensemble member (blockIdx.z)
    {
        const long long mem = blockIdx.z;
        W += mem * 6 * G::FS;
        U += mem * 3 * G::FS;
        UT += mem * 3 * G::FS;
        ACC += mem * 3 * G::FS;
        sd += mem;
        tab += mem * (G::KC2 + 1);
        if (INTEG == INT_TAB) {
            K += mem * 18 * G::FS;
            dpart += (mem * gridDim.y * gridDim.x + (long long)blockIdx.y * gridDim.x + blockIdx.x) * 3;
        }
    }
    const int kz0 = blockIdx.x * TT;
    if (ky * ky + kz0 * kz0 > G::KC2) {
        if (INTEG == INT_TAB && rs.kind == 2 && threadIdx.x < 3) dpart[threadIdx.x] = 0.0;
        return;
    }
    const bool colok = (kz <= G::KC) && (ky * ky + kz * kz <= G::KC2);
    const long long off = (long long)j * G::NZP + kz;
    const long long xs = (long long)N * G::NZP;
    StridedIdx<TT, PL::R1> sidx{t};
    SyncBlock sync;

    cx<T> F[3][E];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const cx<T>* src = W + (long long)c * G::FS + off;
#pragma unroll
        for (int s = 0; s < E; ++s) F[c][s] = colok ? src[(long long)(p + P * s) * xs] : czero<T>();
    }
    xfwd_prefetch_state<T, N, INTEG, MODE, E, P, TT>(U, ACC, K, rs, p, t, ky, kz0, j);
#pragma unroll
    for (int c = 0; c < 3; ++c) PL::fwd(F[c], sbuf, p, tw, sidx, sync);
    if (INTEG != INT_TAB && !colok) return;

    T h = T(0);
    if (MODE <= X_STAGE4) h = T(sd->dt);
    const int rem = G::KC2 - ky * ky - kz * kz;
    if constexpr ((INTEG == INT_IFRK4 || INTEG == INT_RK4CN) && MODE <= X_STAGE4 && TileVar<V>::BATCH) {
        xfwd_rk4_epilogue<T, N, INTEG, MODE, E, P>(F, p, ky, kz, off, U, UT, ACC, tab, sd, sgs, h);
        return;
    }
    double es[3] = {0.0, 0.0, 0.0};   // DP5CN error partial sums
    if constexpr (INTEG == INT_TAB) {
        // RK5 family: the projection of every mode of this thread first; then, in
        // chunks of CH modes and per component, each stored stage's loads for all
        // modes of the chunk before their sums (the stage and coefficient tests
        // are uniform), so that a chunk's loads of one array are in flight at
        // once. Each component's sums run in mode order, as in the per-mode form.
        constexpr int CH = E < 4 ? E : (E >= 16 ? 2 : 4);
        unsigned valid = 0u;
        int k2s[E];
#pragma unroll
        for (int s = 0; s < E; ++s) {
            const int i = p + P * s;
            const int kx = kof<N>(i);
            k2s[s] = 0;
            if (!colok || kx * kx > rem) continue;
            valid |= 1u << s;
            const int k2 = kx * kx + ky * ky + kz * kz;
            k2s[s] = k2;
            cx<T> n0 = F[0][s], n1 = F[1][s], n2 = F[2][s];
            if (sgs && sd->sgs_on) {
                const long long q = (long long)i * xs + off;
                n0 = n0 + sgs[q];
                n1 = n1 + sgs[G::FS + q];
                n2 = n2 + sgs[2 * G::FS + q];
            }
            if (k2 > 0) {
                const T kinv = T(1) / T(k2);
                const cx<T> kdn = n0 * T(kx) + n1 * T(ky) + n2 * T(kz);
                n0 = n0 - kdn * (T(kx) * kinv);
                n1 = n1 - kdn * (T(ky) * kinv);
                n2 = n2 - kdn * (T(kz) * kinv);
            } else {
                n0 = n1 = n2 = czero<T>();
            }
            F[0][s] = n0;
            F[1][s] = n1;
            F[2][s] = n2;
        }
#pragma unroll
        for (int s0 = 0; s0 < E; s0 += CH) {
            if (!((valid >> s0) & ((1u << CH) - 1u))) continue;
            cx<T> ab[CH];
#pragma unroll
            for (int s = 0; s < CH; ++s) ab[s] = ldg(&tab[k2s[s0 + s]]);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                cx<T> acc[CH], ea[CH];
#pragma unroll
                for (int s = 0; s < CH; ++s) {
                    acc[s] = F[c][s0 + s] * T(rs.c_cur);
                    ea[s] = F[c][s0 + s] * T(rs.e_cur);
                }
#pragma unroll
                for (int jj = 0; jj < 6; ++jj) {
                    if (jj < rs.nk && (rs.c[jj] != 0.0 || rs.e[jj] != 0.0)) {
                        cx<T> kv[CH];
#pragma unroll
                        for (int s = 0; s < CH; ++s) {
                            kv[s] = czero<T>();
                            if ((valid >> (s0 + s)) & 1u)
                                kv[s] = K[(long long)jj * 3 * G::FS + c * G::FS + (long long)(p + P * (s0 + s)) * xs + off];
                        }
#pragma unroll
                        for (int s = 0; s < CH; ++s) {
                            acc[s] = acc[s] + kv[s] * T(rs.c[jj]);
                            ea[s] = ea[s] + kv[s] * T(rs.e[jj]);
                        }
                    }
                }
                cx<T> u[CH];
#pragma unroll
                for (int s = 0; s < CH; ++s) {
                    u[s] = czero<T>();
                    if ((valid >> (s0 + s)) & 1u) u[s] = U[c * G::FS + (long long)(p + P * (s0 + s)) * xs + off];
                }
#pragma unroll
                for (int s = 0; s < CH; ++s) {
                    if (!((valid >> (s0 + s)) & 1u)) continue;
                    const long long q = c * G::FS + (long long)(p + P * (s0 + s)) * xs + off;
                    if (rs.store >= 0) K[(long long)rs.store * 3 * G::FS + q] = F[c][s0 + s];
                    if (rs.kind == 0) {
                        UT[q] = u[s] + acc[s] * h;
                    } else if (rs.kind == 1) {
                        U[q] = u[s] * ab[s].x + acc[s] * ab[s].y;
                    } else {
                        const cx<T> un = u[s] * ab[s].x + acc[s] * ab[s].y;
                        ACC[q] = un;
                        const cx<T> df = ea[s] * ab[s].y;
                        const double m0 = sqrt((double)u[s].x * u[s].x + (double)u[s].y * u[s].y);
                        const double m1 = sqrt((double)un.x * un.x + (double)un.y * un.y);
                        const double den = sd->dp_atol + (m0 > m1 ? m0 : m1) * sd->dp_rtol;
                        es[c] += ((double)df.x * df.x + (double)df.y * df.y) / (den * den);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < (INTEG == INT_TAB ? 0 : E); ++s) {
        const int i = p + P * s;
        const int kx = kof<N>(i);
        if (!colok || kx * kx > rem) continue;
        const int k2 = kx * kx + ky * ky + kz * kz;
        cx<T> n0 = F[0][s], n1 = F[1][s], n2 = F[2][s];
        if (MODE <= X_STAGE4 && sgs && sd->sgs_on) {
            // learned subgrid term -div(tau), single run only (member 0)
            const long long q = (long long)i * xs + off;
            n0 = n0 + sgs[q];
            n1 = n1 + sgs[G::FS + q];
            n2 = n2 + sgs[2 * G::FS + q];
        }
        if (MODE != X_PLAIN) {
            if (k2 > 0) {
                const T kinv = T(1) / T(k2);
                const cx<T> kdn = n0 * T(kx) + n1 * T(ky) + n2 * T(kz);
                n0 = n0 - kdn * (T(kx) * kinv);
                n1 = n1 - kdn * (T(ky) * kinv);
                n2 = n2 - kdn * (T(kz) * kinv);
            } else {
                n0 = n1 = n2 = czero<T>();
            }
        }
        const long long idx = (long long)i * xs + off;
        cx<T> nn[3] = {n0, n1, n2};
        if (MODE == X_RHS || MODE == X_PLAIN) {
#pragma unroll
            for (int c = 0; c < 3; ++c) ACC[c * G::FS + idx] = nn[c];
            continue;
        }
        if constexpr (INTEG == INT_TAB) {
            const cx<T> ab = ldg(&tab[k2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const long long q = c * G::FS + idx;
                cx<T> acc = nn[c] * T(rs.c_cur);
                cx<T> ea = nn[c] * T(rs.e_cur);
#pragma unroll
                for (int jj = 0; jj < 6; ++jj) {
                    if (jj < rs.nk && (rs.c[jj] != 0.0 || rs.e[jj] != 0.0)) {
                        const cx<T> kj = K[(long long)jj * 3 * G::FS + q];
                        acc = acc + kj * T(rs.c[jj]);
                        ea = ea + kj * T(rs.e[jj]);
                    }
                }
                if (rs.store >= 0) K[(long long)rs.store * 3 * G::FS + q] = nn[c];
                const cx<T> u = U[q];
                if (rs.kind == 0) {
                    UT[q] = u + acc * h;
                } else if (rs.kind == 1) {
                    U[q] = u * ab.x + acc * ab.y;
                } else {
                    const cx<T> un = u * ab.x + acc * ab.y;
                    ACC[q] = un;
                    const cx<T> df = ea * ab.y;
                    const double m0 = sqrt((double)u.x * u.x + (double)u.y * u.y);
                    const double m1 = sqrt((double)un.x * un.x + (double)un.y * un.y);
                    const double den = sd->dp_atol + (m0 > m1 ? m0 : m1) * sd->dp_rtol;
                    es[c] += ((double)df.x * df.x + (double)df.y * df.y) / (den * den);
                }
            }
            continue;
        }
        if (INTEG == INT_IFRK4) {
            const cx<T> ef = ldg(&tab[k2]);
            const T Eh = ef.x, Ef = ef.y;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const long long q = c * G::FS + idx;
                if (MODE == X_STAGE1) {
                    const cx<T> u = U[q];
                    UT[q] = (u + nn[c] * (h * T(0.5))) * Eh;
                    ACC[q] = (u + nn[c] * (h / T(6))) * Ef;
                } else if (MODE == X_STAGE2) {
                    const cx<T> u = U[q];
                    UT[q] = u * Eh + nn[c] * (h * T(0.5));
                    ACC[q] = ACC[q] + nn[c] * (h / T(3) * Eh);
                } else if (MODE == X_STAGE3) {
                    const cx<T> u = U[q];
                    UT[q] = u * Ef + nn[c] * (h * Eh);
                    ACC[q] = ACC[q] + nn[c] * (h / T(3) * Eh);
                } else {
                    U[q] = ACC[q] + nn[c] * (h / T(6));
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const long long q = c * G::FS + idx;
                if (MODE == X_STAGE1) {
                    UT[q] = U[q] + nn[c] * (h * T(0.5));
                    ACC[q] = nn[c] * (T(1) / T(6));
                } else if (MODE == X_STAGE2) {
                    UT[q] = U[q] + nn[c] * (h * T(0.5));
                    ACC[q] = ACC[q] + nn[c] * (T(1) / T(3));
                } else if (MODE == X_STAGE3) {
                    UT[q] = U[q] + nn[c] * h;
                    ACC[q] = ACC[q] + nn[c] * (T(1) / T(3));
                } else {
                    const cx<T> ab = ldg(&tab[k2]);
                    U[q] = U[q] * ab.x + (ACC[q] + nn[c] * (T(1) / T(6))) * ab.y;
                }
            }
        }
    }
    if constexpr (INTEG == INT_TAB) {
        if (rs.kind == 2) {
            // fixed-order block reduction: warp shuffles (full warps; the
            // block size is a power of two), then the warps' sums in order;
            // blocks of fewer than 32 threads add their threads in order
            __shared__ double red[32][3];
            const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            const bool full = blockDim.x >= 32;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double v = es[c];
                if (full) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                    if (lane == 0) red[wid][c] = v;
                } else {
                    red[threadIdx.x][c] = v;
                }
            }
            __syncthreads();
            if (threadIdx.x < 3) {
                const int n = full ? (int)(blockDim.x >> 5) : (int)blockDim.x;
                double v = 0.0;
                for (int w = 0; w < n; ++w) v += red[w][threadIdx.x];
                dpart[threadIdx.x] = v;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Integrator tables (FP64 exponentials), optionally after a CFL step choice.
// tab[k2], k2 = 0..KC2. IF-RK4: (exp(-nu k2^p h/2), exp(-nu k2^p h));
// RK4CN: ((2-D)/(2+D), 2h/(2+D)), D = h nu k2^p (solver.c:580-603).
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_tables(cx<T>* __restrict__ tab, StepDev* __restrict__ sd, int integ, int vp, int use_cfl) {
    using G = Geo<N>;
    sd += blockIdx.y;   // ensemble member
    tab += (long long)blockIdx.y * (G::KC2 + 1);
    double h = sd->dt;
    if (use_cfl) {
        const unsigned long long b = sd->umax_bits;
        double um = sizeof(T) == 4 ? (double)__uint_as_float((unsigned)b) : __longlong_as_double((long long)b);
        double hn = (um > 0.0) ? sd->cfl * (2.0 * 3.14159265358979323846 / (double)N) / um : h;
        if (!(hn > 0.0) || !isfinite(hn)) hn = h;
        h = hn;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            sd->dt = hn;
            sd->umax = um;
            if (!isfinite(um)) sd->status = 5;
        }
    }
    const int k2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (k2 > G::KC2) return;
    const double kk = (double)k2;
    const double L = sd->nu * (vp == 2 ? kk * kk : kk);
    cx<T> e;
    if (integ == INT_IFRK4) {
        e.x = T(exp(-0.5 * h * L));
        e.y = T(exp(-h * L));
    } else {
        const double D = h * L;
        e.x = T((2.0 - D) / (2.0 + D));
        e.y = T(2.0 * h / (2.0 + D));
    }
    tab[k2] = e;
}

// ---------------------------------------------------------------------------
// End of step: shell-energy forcing (new component) and time bookkeeping
// (solver.c:193). One CTA of 256 threads; deterministic FP64 reduction.
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_step_end(cx<T>* __restrict__ U, StepDev* __restrict__ sd, int force_k, int use_cfl, int dp) {
    using G = Geo<N>;
    U += (long long)blockIdx.x * 3 * G::FS;   // one CTA per ensemble member
    sd += blockIdx.x;
    __shared__ double red[256];
    // a rejected DP5CN attempt leaves the state, the time and the forcing alone.
    // The energy of the shells round(|k|) <= kb is summed every step: it is the
    // forcing's measure, and without forcing (kb = 1) the numeric health check
    // (a NaN or Inf anywhere in the field reaches these shells through the
    // nonlinear term within one step)
    const bool rejected = dp && !sd->dp_accept;
    const int kb = rejected ? 0 : (force_k > 0 ? force_k : 1);
    const int side = 2 * kb + 1;
    const int nbox = side * side * (kb + 1);
    const long long k2max = (long long)kb * (kb + 1);
    double e = 0.0;
    if (kb > 0) {
        for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
            const int kx = q % side - kb, ky = (q / side) % side - kb, kz = q / (side * side);
            const long long k2 = (long long)kx * kx + ky * ky + kz * kz;
            if (k2 == 0 || k2 > k2max || k2 > G::KC2) continue;
            const int i = kx < 0 ? kx + N : kx, j = ky < 0 ? ky + N : ky;
            const long long idx = ((long long)i * N + j) * G::NZP + kz;
            const double m = (kz == 0) ? 1.0 : 2.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const cx<T> v = U[c * G::FS + idx];
                e += m * ((double)v.x * (double)v.x + (double)v.y * (double)v.y);
            }
        }
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double en = red[0] * 8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846 * 0.5 /
                      ((double)N * N * N * (double)N * N * N);
    if (force_k > 0 && kb > 0 && en > 0.0 && sd->force_target > 0.0) {
        const T sc = T(sqrt(sd->force_target / en));
        for (int q = threadIdx.x; q < nbox; q += blockDim.x) {
            const int kx = q % side - kb, ky = (q / side) % side - kb, kz = q / (side * side);
            const long long k2 = (long long)kx * kx + ky * ky + kz * kz;
            if (k2 == 0 || k2 > k2max || k2 > G::KC2) continue;
            const int i = kx < 0 ? kx + N : kx, j = ky < 0 ? ky + N : ky;
            const long long idx = ((long long)i * N + j) * G::NZP + kz;
#pragma unroll
            for (int c = 0; c < 3; ++c) U[c * G::FS + idx] = U[c * G::FS + idx] * sc;
        }
    }
    if (threadIdx.x == 0) {
        if (dp) {
            if (!rejected) {
                sd->iters += 1;
                sd->t += sd->dp_h;
            }
        } else {
            sd->iters += 1;
            if (use_cfl) sd->t += sd->dt;
            else sd->t = sd->t0 + (double)sd->iters * sd->dt;
        }
        if (!isfinite(en)) sd->status = 5;
        sd->umax_bits = 0ull;
    }
}

// ---------------------------------------------------------------------------
// DP5CN step control (SpectralSolve, solver.c:134-154, with D15/D18 fixed):
// err = max_d sqrt(sum_d / (N N (N/2+1))) from the per-block partial sums in
// a fixed order; accept when err <= 1; either way the next attempt uses
// h min(1.5, max(0.01, 0.8 err^(-1/5))). One CTA of 256 threads per member.
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_dp_ctl(const double* __restrict__ dpart, int nparts, StepDev* __restrict__ sd) {
    __shared__ double red[3][256];
    sd += blockIdx.x;
    dpart += (long long)blockIdx.x * nparts * 3;
    double v[3] = {0.0, 0.0, 0.0};
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] += dpart[3 * q + c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) red[c][threadIdx.x] = v[c];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
#pragma unroll
            for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double nm = (double)N * N * (N / 2 + 1);
        double err = sqrt(red[0][0] / nm);
        err = fmax(err, sqrt(red[1][0] / nm));
        err = fmax(err, sqrt(red[2][0] / nm));
        if (!(red[0][0] == red[0][0]) || !(red[1][0] == red[1][0]) || !(red[2][0] == red[2][0])) err = NAN;
        double fac = 0.8 * pow(1.0 / err, 0.2);
        fac = fac < 0.01 ? 0.01 : fac;
        fac = fac > 1.5 ? 1.5 : fac;
        const double h = sd->dt;
        sd->dp_err = err;
        sd->dp_h = h;
        sd->dt = h * fac;
        if (err <= 1.0) {
            sd->dp_accept = 1;
            sd->dp_tries = 0;
        } else {
            sd->dp_accept = 0;
            sd->dp_rejects += 1;
            sd->dp_tries += 1;
            if (sd->dp_tries >= kDpMaxTry || !(sd->dt > 0.0)) sd->status = kStatusDpFail;
        }
    }
}

// accepted DP5CN attempt: the trial solution (ACC) becomes the state (U);
// only the dealiased sphere is copied. grid (x, members)
template <typename T, int N>
__global__ void k_dp_commit(cx<T>* __restrict__ U, const cx<T>* __restrict__ ACC, const StepDev* __restrict__ sd) {
    using G = Geo<N>;
    const long long mem = blockIdx.y;
    if (!sd[mem].dp_accept) return;
    U += mem * 3 * G::FS;
    ACC += mem * 3 * G::FS;
    const long long n = (long long)N * N * G::NZP;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % G::NZP);
        const long long ij = q / G::NZP;
        const int kx = kof<N>((int)(ij / N)), ky = kof<N>((int)(ij % N));
        if (kz > G::KC || kx * kx + ky * ky + kz * kz > G::KC2) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) U[c * G::FS + q] = ACC[c * G::FS + q];
    }
}

// ---------------------------------------------------------------------------
// Diagnostics (ComputeSystemMeasurables, solver.c:1142-1276; D4 fixed).
// A warp walks one (kx, ky) line at a time, lanes over consecutive kz; the
// shell index round(|k|) is non-decreasing along kz, so a segmented warp scan
// merges equal-shell lanes and each segment's last lane adds its sum to the
// warp's private shared-memory histogram. Per-CTA partials (5 totals +
// 2*NSP bins) go to global memory; k_measure_reduce sums them in a fixed
// order. Everything is FP64 and the result is bitwise reproducible.
// ---------------------------------------------------------------------------
constexpr int MEAS_WARPS = 8;
template <int N> constexpr int meas_lines_per_cta() { return 64; }

template <typename T, int N>
__global__ void __launch_bounds__(MEAS_WARPS * 32)
k_measure(const cx<T>* __restrict__ U, double nu, int vp, double* __restrict__ part) {
    using G = Geo<N>;
    constexpr int NSP = G::NSP;
    constexpr int LPC = meas_lines_per_cta<N>();
    __shared__ double hist[MEAS_WARPS][2][NSP];
    __shared__ double tots[MEAS_WARPS][5];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < MEAS_WARPS * 2 * NSP; q += blockDim.x) (&hist[0][0][0])[q] = 0.0;
    __syncthreads();
    double s_en = 0, s_ens = 0, s_pal = 0, s_hel = 0, s_dis = 0;
    const long long nlines = (long long)N * G::NKY;   // (kx index, ky row) pairs
    for (int l = w; l < LPC; l += MEAS_WARPS) {
        const long long line = (long long)blockIdx.x * LPC + l;
        if (line >= nlines) break;
        const int i = (int)(line / G::NKY);
        const int ky = (int)(line % G::NKY) - G::KC;
        const int kx = kof<N>(i);
        const int j = ky < 0 ? ky + N : ky;
        const int r2 = kx * kx + ky * ky;
        if (r2 > G::KC2) continue;
        for (int kz0 = 0; kz0 <= G::KC; kz0 += 32) {
            const int kz = kz0 + lane;
            const int k2 = r2 + kz * kz;
            const bool in = (kz <= G::KC) && (k2 <= G::KC2);
            double eu = 0, ew = 0;
            int bin = 0x7fffffff;
            if (in) {
                // per-mode terms in the state's precision (FP32 products of FP32 modes,
                // 10x cheaper than FP64 on this GPU), every sum in FP64
                using R = T;
                const long long idx = ((long long)i * N + j) * G::NZP + kz;
                const cx<T> a0 = U[idx], a1 = U[G::FS + idx], a2 = U[2 * G::FS + idx];
                const R ux = a0.x, uxi = a0.y, uy = a1.x, uyi = a1.y, uz = a2.x, uzi = a2.y;
                const R fkx = R(kx), fky = R(ky), fkz = R(kz);
                // w = i k x u  ->  re(w) = -(k x u_im), im(w) = k x u_re
                const R wxr = -(fky * uzi - fkz * uyi), wxi = fky * uz - fkz * uy;
                const R wyr = -(fkz * uxi - fkx * uzi), wyi = fkz * ux - fkx * uz;
                const R wzr = -(fkx * uyi - fky * uxi), wzi = fkx * uy - fky * ux;
                const R cxr = -(fky * wzi - fkz * wyi), cxi = fky * wzr - fkz * wyr;
                const R cyr = -(fkz * wxi - fkx * wzi), cyi = fkz * wxr - fkx * wzr;
                const R czr = -(fkx * wyi - fky * wxi), czi = fkx * wyr - fky * wxr;
                eu = double(ux * ux + uxi * uxi + uy * uy + uyi * uyi + uz * uz + uzi * uzi);
                ew = double(wxr * wxr + wxi * wxi + wyr * wyr + wyi * wyi + wzr * wzr + wzi * wzi);
                const double ec = double(cxr * cxr + cxi * cxi + cyr * cyr + cyi * cyi + czr * czr + czi * czi);
                // helicity Re(u . conj(w)); the reference's Re(u . w) (solver.c:1227)
                // is identically zero because u . (k x u) = 0 (defect D12, fixed)
                const double hel = double((ux * wxr + uxi * wxi) + (uy * wyr + uyi * wyi) + (uz * wzr + uzi * wzi));
                const double kk = (double)k2;
                const double pre = nu * (vp == 2 ? kk * kk : kk);
                const double m = (kz == 0) ? 1.0 : 2.0;
                eu *= m;
                ew *= m;
                s_en += eu;
                s_ens += ew;
                s_pal += m * ec;
                s_hel += m * hel;
                s_dis += pre * eu;
                bin = (int)rint(sqrt(kk));   // k2 is never (n+1/2)^2, so rint == round
            }
            // segmented inclusive scan over lanes with equal bins
            double se = eu, sw = ew;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double te = __shfl_up_sync(0xffffffffu, se, o);
                const double tw2 = __shfl_up_sync(0xffffffffu, sw, o);
                const int tb = __shfl_up_sync(0xffffffffu, bin, o);
                if (lane >= o && tb == bin) {
                    se += te;
                    sw += tw2;
                }
            }
            const int nb = __shfl_down_sync(0xffffffffu, bin, 1);
            if (in && (lane == 31 || nb != bin)) {
                hist[w][0][bin] += se;
                hist[w][1][bin] += sw;
            }
        }
    }
    // totals: fixed-order warp tree, then fixed warp order
    double v[5] = {s_en, s_ens, s_pal, s_hel, s_dis};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
        if (lane == 0) tots[w][q] = v[q];
    }
    __syncthreads();
    double* out = part + (long long)blockIdx.x * (5 + 2 * NSP);
    if (threadIdx.x < 5) {
        double a = 0;
        for (int q = 0; q < MEAS_WARPS; ++q) a += tots[q][threadIdx.x];
        out[threadIdx.x] = a;
    }
    for (int b = threadIdx.x; b < 2 * NSP; b += blockDim.x) {
        double a = 0;
        for (int q = 0; q < MEAS_WARPS; ++q) a += hist[q][b / NSP][b % NSP];
        out[5 + b] = a;
    }
}

// Column sums of the partials in CTA order, then the reference scalings
// (defined in ns3d_misc.cu).
__global__ void k_measure_reduce(const double* __restrict__ part, int nparts, int width, int nsp,
                                 double N3sq, double* __restrict__ out);

// ---------------------------------------------------------------------------
// Layout conversion between the reference layout (complex double
// [N][N][N/2+1][3]) and the device layout; modes outside the sphere dropped.
// ---------------------------------------------------------------------------
template <typename T, int N>
__global__ void k_pack(const double2* __restrict__ ref, cx<T>* __restrict__ U) {
    using G = Geo<N>;
    constexpr int NF = N / 2 + 1;
    const long long total = (long long)N * N * G::NZP;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % G::NZP);
        const long long ij = q / G::NZP;
        const int j = (int)(ij % N), i = (int)(ij / N);
        const int kx = kof<N>(i), ky = kof<N>(j);
        const bool in = kz <= G::KC && kx * kx + ky * ky + kz * kz <= G::KC2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cx<T> v = czero<T>();
            if (in) {
                const double2 d = ref[(ij * NF + kz) * 3 + c];
                v = mk(T(d.x), T(d.y));
            }
            U[c * G::FS + q] = v;
        }
    }
}

// Host array -> device state for a page-locked host array: one warp per range
// of 16-byte elements (the 128-byte lines of one (kx, ky) row that hold its
// dealiased modes), four 512-byte loads in flight per warp; the dealiased modes
// among them are written to U, the rest of each line is skipped.
template <typename T, int N>
__global__ void k_pack_lines(const double2* __restrict__ ref, cx<T>* __restrict__ U,
                             const longlong2* __restrict__ ranges, int nranges) {
    using G = Geo<N>;
    constexpr int NF = N / 2 + 1;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nranges) return;
    const longlong2 rg = ranges[w];
    for (long long u0 = rg.x + lane; u0 < rg.y; u0 += 128) {
        double2 d[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (u0 + 32 * k < rg.y) d[k] = ref[u0 + 32 * k];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long u = u0 + 32 * k;
            if (u >= rg.y) break;
            const long long e = u / 3;
            const int c = (int)(u % 3);
            const long long ij = e / NF;
            const int kz = (int)(e % NF);
            const int j = (int)(ij % N), i = (int)(ij / N);
            const int kx = kof<N>(i), ky = kof<N>(j);
            if (kz <= G::KC && kx * kx + ky * ky + kz * kz <= G::KC2)
                U[c * G::FS + ij * G::NZP + kz] = mk(T(d[k].x), T(d[k].y));
        }
    }
}

template <typename T, int N>
__global__ void k_unpack(const cx<T>* __restrict__ U, double2* __restrict__ ref) {
    using G = Geo<N>;
    constexpr int NF = N / 2 + 1;
    const long long total = (long long)N * N * NF;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % NF);
        const long long ij = q / NF;
        const int j = (int)(ij % N), i = (int)(ij / N);
        const int kx = kof<N>(i), ky = kof<N>(j);
        const bool in = kz <= G::KC && kx * kx + ky * ky + kz * kz <= G::KC2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double2 d = make_double2(0.0, 0.0);
            if (in) {
                const cx<T> v = U[c * G::FS + ij * G::NZP + kz];
                d = make_double2((double)v.x, (double)v.y);
            }
            ref[q * 3 + c] = d;
        }
    }
}

// device -> host array (reference layout) over a list of 16-byte unit ranges:
// every unit of the listed ranges gets its mode's value (zero outside the
// sphere); one warp per range. The ranges cover whole 128-byte lines around
// the dealiased modes; the host zeroes every other line.
template <typename T, int N>
__global__ void k_unpack_lines(const cx<T>* __restrict__ U, double2* __restrict__ ref,
                               const longlong2* __restrict__ ranges, int nranges) {
    using G = Geo<N>;
    constexpr int NF = N / 2 + 1;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nranges) return;
    const longlong2 rg = ranges[w];
    for (long long u = rg.x + lane; u < rg.y; u += 32) {
        const long long e = u / 3;
        const int c = (int)(u % 3);
        const long long ij = e / NF;
        const int kz = (int)(e % NF);
        const int j = (int)(ij % N), i = (int)(ij / N);
        const int kx = kof<N>(i), ky = kof<N>(j);
        double2 d = make_double2(0.0, 0.0);
        if (kz <= G::KC && kx * kx + ky * ky + kz * kz <= G::KC2) {
            const cx<T> v = U[c * G::FS + ij * G::NZP + kz];
            d = make_double2((double)v.x, (double)v.y);
        }
        ref[u] = d;
    }
}

// real [6][N][N][N] (u then w) -> reference real layout [N][N][N+2][3] x2
template <typename T, int N>
__global__ void k_real_unpack(const T* __restrict__ R, double* __restrict__ u, double* __restrict__ w) {
    const long long total = (long long)N * N * (N + 2);
    const long long M = (long long)N * N * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % (N + 2));
        const long long ij = q / (N + 2);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double a = 0.0, b = 0.0;
            if (k < N) {
                a = (double)R[c * M + ij * N + k];
                b = (double)R[(3 + c) * M + ij * N + k];
            }
            if (u) u[q * 3 + c] = a;
            if (w) w[q * 3 + c] = b;
        }
    }
}

// ---------------------------------------------------------------------------
// Initial conditions
// ---------------------------------------------------------------------------
// TAYLOR_GREEN (solver.c:1557-1568, KAPPA = 1) and SHAPIRO (solver.c:1579-1595,
// A = 2, K = L = M = 2) in real space, real [3][N][N][N], FP64 evaluation.
// SHAPIRO uses w = A cos(Kx) cos(Ly) sin(Mz), Shapiro's exact Beltrami
// solution; the reference's cos(Mz) (solver.c:1593) is not divergence free.
template <typename T, int N>
__global__ void k_fill_real(T* __restrict__ R, int kind) {
    const long long M = (long long)N * N * N;
    const double dx = 2.0 * 3.14159265358979323846 / (double)N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % N), j = (int)((q / N) % N), i = (int)(q / ((long long)N * N));
        const double x = i * dx, y = j * dx, z = k * dx;
        double a, b, c;
        if (kind == 0) {
            a = sin(x) * cos(y) * cos(z);
            b = -cos(x) * sin(y) * cos(z);
            c = 0.0;
        } else {
            const double A = 2.0, K = 2.0, L = 2.0, Mm = 2.0;
            const double lam = sqrt(K * K + L * L + Mm * Mm);
            a = -A / (K * K + L * L) * (lam * L * cos(K * x) * sin(L * y) * sin(Mm * z) + Mm * K * sin(K * x) * cos(L * y) * cos(Mm * z));
            b = A / (K * K + L * L) * (lam * K * sin(K * x) * cos(L * y) * sin(Mm * z) - Mm * L * cos(K * x) * sin(L * y) * cos(Mm * z));
            c = A * cos(K * x) * cos(L * y) * sin(Mm * z);
        }
        R[q] = T(a);
        R[M + q] = T(b);
        R[2 * M + q] = T(c);
    }
}

// SplitMix64 (Steele, Lea & Flood 2014): finaliser of x + golden gamma.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    unsigned long long z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(unsigned long long key, unsigned long long id, int r) {
    return (double)(splitmix64(key ^ (id * 8ull + (unsigned long long)r)) >> 11) * 0x1.0p-53;
}

// SPECTRUM: seeded random-phase solenoidal field, |u_hat(k)| = |k| exp(-k^2/k0^2)
// (E(k) ~ k^4 exp(-2 (k/k0)^2)), Hermitian on kz = 0; the energy is scaled
// afterwards. Random numbers are keyed by the reference-layout index of the
// canonical mode, so the field does not depend on the device layout.
template <typename T, int N>
__global__ void k_spectrum_ic(cx<T>* __restrict__ U, unsigned long long key, double k0) {
    using G = Geo<N>;
    constexpr int NF = N / 2 + 1;
    const long long total = (long long)N * N * G::NZP;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % G::NZP);
        const long long ij = q / G::NZP;
        const int j = (int)(ij % N), i = (int)(ij / N);
        const int kx = kof<N>(i), ky = kof<N>(j);
        const long long k2 = (long long)kx * kx + (long long)ky * ky + (long long)kz * kz;
        cx<T> o[3] = {czero<T>(), czero<T>(), czero<T>()};
        if (kz <= G::KC && k2 > 0 && k2 <= G::KC2) {
            bool cj = false;
            int ci = i, cjj = j;
            if (kz == 0 && !(kx > 0 || (kx == 0 && ky > 0))) {
                cj = true;
                ci = (N - i) % N;
                cjj = (N - j) % N;
            }
            const unsigned long long id = (unsigned long long)(((long long)ci * N + cjj) * NF + kz);
            double vr[3], vi[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                vr[d] = 2.0 * u01(key, id, 2 * d) - 1.0;
                vi[d] = 2.0 * u01(key, id, 2 * d + 1) - 1.0;
            }
            const double ckx = kof<N>(ci), cky = kof<N>(cjj), ckz = kz;
            const double kk = (double)k2;
            const double kvr = ckx * vr[0] + cky * vr[1] + ckz * vr[2];
            const double kvi = ckx * vi[0] + cky * vi[1] + ckz * vi[2];
            vr[0] -= ckx * kvr / kk; vi[0] -= ckx * kvi / kk;
            vr[1] -= cky * kvr / kk; vi[1] -= cky * kvi / kk;
            vr[2] -= ckz * kvr / kk; vi[2] -= ckz * kvi / kk;
            const double vn = sqrt(vr[0] * vr[0] + vi[0] * vi[0] + vr[1] * vr[1] + vi[1] * vi[1] + vr[2] * vr[2] + vi[2] * vi[2]);
            if (vn > 1e-300) {
                const double amp = sqrt(kk) * exp(-kk / (k0 * k0)) / vn;
#pragma unroll
                for (int d = 0; d < 3; ++d) o[d] = mk(T(amp * vr[d]), T(cj ? -amp * vi[d] : amp * vi[d]));
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) U[d * G::FS + q] = o[d];
    }
}

template <typename T, int N>
__global__ void k_scale(cx<T>* __restrict__ U, double s) {
    using G = Geo<N>;
    const long long total = 3 * G::FS;
    const T sc = T(s);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x)
        U[q] = U[q] * sc;
}

}  // namespace ns3d

namespace ns3d {

// ---------------------------------------------------------------------------
// Learned subgrid closure support (single run, FP32 engines)
// ---------------------------------------------------------------------------
// F_i = -i k_j tau_ij (tau components xx, yy, zz, xy, xz, yz) and the
// per-CTA partials of the energy transfer T = sum_k m Re(u . conj(F)).
template <typename T, int N>
__global__ void k_sgs_div(const cx<T>* __restrict__ TAU, const cx<T>* __restrict__ U, cx<T>* __restrict__ F,
                          double* __restrict__ part) {
    using G = Geo<N>;
    __shared__ double red[256];
    const long long total = (long long)N * N * G::NZP;
    double s = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % G::NZP);
        const long long ij = q / G::NZP;
        const int kx = kof<N>((int)(ij / N)), ky = kof<N>((int)(ij % N));
        cx<T> f[3] = {czero<T>(), czero<T>(), czero<T>()};
        if (kz <= G::KC && kx * kx + ky * ky + kz * kz <= G::KC2) {
            const cx<T> txx = TAU[q], tyy = TAU[G::FS + q], tzz = TAU[2 * G::FS + q];
            const cx<T> txy = TAU[3 * G::FS + q], txz = TAU[4 * G::FS + q], tyz = TAU[5 * G::FS + q];
            const T fx = T(kx), fy = T(ky), fz = T(kz);
            // -i (k . tau)_i
            f[0] = mul_mi(txx * fx + txy * fy + txz * fz);
            f[1] = mul_mi(txy * fx + tyy * fy + tyz * fz);
            f[2] = mul_mi(txz * fx + tyz * fy + tzz * fz);
            const double m = kz == 0 ? 1.0 : 2.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const cx<T> u = U[c * G::FS + q];
                s += m * ((double)u.x * (double)f[c].x + (double)u.y * (double)f[c].y);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) F[c * G::FS + q] = f[c];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// energy-budget check of the closure: keep it for this step only when it
// removes energy on balance (T <= 0) and is finite; otherwise this step is
// the plain coarse solve
template <int Unused = 0>
__global__ void k_sgs_flag(const double* __restrict__ part, int nparts, StepDev* __restrict__ sd,
                           const int* __restrict__ les_status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < nparts; ++i) s += part[i];
    // a closure kernel that gave up on a bounded wait fails the step
    if (les_status && *les_status != 0) sd->status = kStatusTimeout;
    const int ok = isfinite(s) && s <= 0.0 && !(les_status && *les_status != 0);
    sd->sgs_on = ok;
    if (ok) sd->sgs_steps += 1;
    else sd->sgs_fallbacks += 1;
}

// reference real layout [N][N][N+2][3] (double) -> device real fields [3][N^3]
template <typename T, int N>
__global__ void k_real_pack(const double* __restrict__ u, T* __restrict__ R) {
    const long long M = (long long)N * N * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < M; q += (long long)gridDim.x * blockDim.x) {
        const long long ij = q / N;
        const int k = (int)(q % N);
#pragma unroll
        for (int c = 0; c < 3; ++c) R[c * M + q] = T(u[(ij * (N + 2) + k) * 3 + c]);
    }
}

}  // namespace ns3d

// the tensor-core z pass (z-pass form 2) uses Geo, StepDev and Bits above
#include "zgemm.cuh"
