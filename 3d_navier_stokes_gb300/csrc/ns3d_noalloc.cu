// ns3d_noalloc.cu — ns3d_measurables_noalloc: the diagnostics of
// ComputeSystemMeasurables for callers that cannot allocate device memory.
//
// Who needs it: code that runs inside another program's time loop on a GPU
// whose memory that program has already reserved in full (for example an
// in-situ analysis hook of a larger simulation with its own pooling
// allocator), or that runs under a rule forbidding device allocations after
// start-up. Such callers own their input and output buffers but cannot call
// cudaMalloc, so the per-CTA partial sums that the context-based
// ns3d_measurables keeps in a context allocation live here in a file-scope
// static __device__ array of fixed size instead.
//
// What it computes: every mode of the caller's array counts, with the
// reference's multiplicities (1 on the kz = 0 and kz = N/2 planes, 2
// elsewhere, solver.c:1230-1262); shells with round(|k|) >= n_spect (corner
// modes outside the 2/3 sphere, for N whose sqrt(3)N/2 has a fraction >= 1/2)
// are left out of E(k) and Omega(k) but stay in the totals: the reference
// writes one element past its spectrum arrays there (solver.c:1242-1250).
//
// Limits and sharing:
//   * N <= 512 (the partials of a 512^3 grid fill at most 228,608 of the
//     262,144 doubles = 2 MiB of the array); larger N is rejected.
//   * The array exists once per device for as long as the library is loaded,
//     on every GPU that loads it.
//   * Every call uses the same array and leaves its contents behind. Each call
//     writes every slot it later reads, so nothing has to be cleared, but two
//     calls whose kernels overlap on the GPU (different streams, or different
//     host threads) race on the array and corrupt each other's results.
//   * Outside stream capture each call looks up the array's device address
//     for the current context (cudaGetSymbolAddress) and remembers it under
//     that context's unique id. A call made while its stream is being
//     captured uses the remembered address of the current context, so the
//     first call in a context (and the first after a cudaDeviceReset, which
//     makes a new context) must come before any stream capture; otherwise it
//     returns NS3D_ERR_INVALID.
#include <mutex>
#include <stdint.h>
#include <stdio.h>

#include "../../include/ns3d.h"
#include <cuda_runtime.h>

namespace {

constexpr int kMaxN = 512;
constexpr size_t kScratchDoubles = 262144;   // 2 MiB
constexpr int kWarps = 4;
constexpr int kLinesPerCta = 1024;

static __device__ __align__(256) double g_scratch[kScratchDoubles];

// Same algorithm as k_measure (segmented warp scan of equal shells along kz,
// per-warp shared histograms, fixed-order reductions), for a runtime N, over
// every mode of a reference-layout array complex double [N][N][N/2+1][3].
__global__ void __launch_bounds__(kWarps * 32)
k_measure_ref(const double2* __restrict__ u, int N, double nu, int vp, int nsp, double* __restrict__ part) {
    extern __shared__ double sh[];   // [kWarps][2][nsp] then [kWarps][5]
    double* tots = sh + kWarps * 2 * nsp;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int NF = N / 2 + 1;
    for (int q = threadIdx.x; q < kWarps * 2 * nsp; q += blockDim.x) sh[q] = 0.0;
    __syncthreads();
    double s_en = 0, s_ens = 0, s_pal = 0, s_hel = 0, s_dis = 0;
    const long long nlines = (long long)N * N;
    for (int l = w; l < kLinesPerCta; l += kWarps) {
        const long long line = (long long)blockIdx.x * kLinesPerCta + l;
        if (line >= nlines) break;
        const int i = (int)(line / N), j = (int)(line % N);
        const int kx = i <= N / 2 ? i : i - N, ky = j <= N / 2 ? j : j - N;
        const long long r2 = (long long)kx * kx + (long long)ky * ky;
        double* hist = sh + w * 2 * nsp;
        for (int kz0 = 0; kz0 < NF; kz0 += 32) {
            const int kz = kz0 + lane;
            const bool in = kz < NF;
            double eu = 0, ew = 0;
            int bin = 0x7fffffff;
            if (in) {
                const double2* v = u + (line * NF + kz) * 3;
                const double2 a0 = v[0], a1 = v[1], a2 = v[2];
                const double fkx = kx, fky = ky, fkz = kz;
                const double wxr = -(fky * a2.y - fkz * a1.y), wxi = fky * a2.x - fkz * a1.x;
                const double wyr = -(fkz * a0.y - fkx * a2.y), wyi = fkz * a0.x - fkx * a2.x;
                const double wzr = -(fkx * a1.y - fky * a0.y), wzi = fkx * a1.x - fky * a0.x;
                const double cxr = -(fky * wzi - fkz * wyi), cxi = fky * wzr - fkz * wyr;
                const double cyr = -(fkz * wxi - fkx * wzi), cyi = fkz * wxr - fkx * wzr;
                const double czr = -(fkx * wyi - fky * wxi), czi = fkx * wyr - fky * wxr;
                eu = a0.x * a0.x + a0.y * a0.y + a1.x * a1.x + a1.y * a1.y + a2.x * a2.x + a2.y * a2.y;
                ew = wxr * wxr + wxi * wxi + wyr * wyr + wyi * wyi + wzr * wzr + wzi * wzi;
                const double ec = cxr * cxr + cxi * cxi + cyr * cyr + cyi * cyi + czr * czr + czi * czi;
                const double hel = (a0.x * wxr + a0.y * wxi) + (a1.x * wyr + a1.y * wyi) + (a2.x * wzr + a2.y * wzi);
                const double kk = (double)(r2 + (long long)kz * kz);
                const double pre = nu * (vp == 2 ? kk * kk : kk);
                const double m = (kz == 0 || kz == NF - 1) ? 1.0 : 2.0;
                eu *= m;
                ew *= m;
                s_en += eu;
                s_ens += ew;
                s_pal += m * ec;
                s_hel += m * hel;
                s_dis += pre * eu;
                bin = (int)rint(sqrt(kk));
            }
            double se = eu, sw = ew;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double te = __shfl_up_sync(0xffffffffu, se, o);
                const double tw = __shfl_up_sync(0xffffffffu, sw, o);
                const int tb = __shfl_up_sync(0xffffffffu, bin, o);
                if (lane >= o && tb == bin) {
                    se += te;
                    sw += tw;
                }
            }
            const int nb = __shfl_down_sync(0xffffffffu, bin, 1);
            if (in && (lane == 31 || nb != bin) && bin < nsp) {
                hist[bin] += se;
                hist[nsp + bin] += sw;
            }
        }
    }
    double v[5] = {s_en, s_ens, s_pal, s_hel, s_dis};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
        if (lane == 0) tots[w * 5 + q] = v[q];
    }
    __syncthreads();
    const int width = 5 + 2 * nsp;
    double* out = part + (long long)blockIdx.x * width;
    if (threadIdx.x < 5) {
        double a = 0;
        for (int q = 0; q < kWarps; ++q) a += tots[q * 5 + threadIdx.x];
        out[threadIdx.x] = a;
    }
    for (int b = threadIdx.x; b < 2 * nsp; b += blockDim.x) {
        double a = 0;
        for (int q = 0; q < kWarps; ++q) a += sh[q * 2 * nsp + b];
        out[5 + b] = a;
    }
}

// Column sums of the partials in CTA order, scaled as solver.c:1270-1274,
// written straight into the caller's output arrays.
__global__ void k_reduce_out(const double* __restrict__ part, int nparts, int nsp, double N3sq,
                             double* __restrict__ tot, double* __restrict__ Ek, double* __restrict__ Ok) {
    const int width = 5 + 2 * nsp;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= width) return;
    double a = 0.0;
    for (int q = 0; q < nparts; ++q) a += part[(long long)q * width + c];
    const double cf = 8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846;
    const double nf = 0.5 / N3sq;
    if (c < 5) {
        tot[c] = a * (c == 4 ? 2.0 : 1.0) * cf * nf;
    } else if (c < 5 + nsp) {
        if (Ek) Ek[c - 5] = a * cf * nf;
    } else {
        if (Ok) Ok[c - 5 - nsp] = a * cf * nf;
    }
}

std::mutex g_mu;
constexpr int kMaxContexts = 64;
struct ScratchEntry {
    unsigned long long ctx_id;
    double* addr;
};
ScratchEntry g_cache[kMaxContexts];
int g_cached = 0;

typedef int (*ctx_get_current_fn)(void**);
typedef int (*ctx_get_id_fn)(void*, unsigned long long*);

// The driver's unique id of the calling thread's current context (ids are
// never reused within a process), through the runtime's driver entry points.
bool current_context_id(unsigned long long* id) {
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess)
            return false;
        get_current = reinterpret_cast<ctx_get_current_fn>(f1);
        get_id = reinterpret_cast<ctx_get_id_fn>(f2);
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

// The device address of g_scratch in the current context (see the file
// comment for when it is looked up and when a remembered one is used).
ns3d_status scratch_address(cudaStream_t s, double** out) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return NS3D_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        unsigned long long id = 0;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return NS3D_ERR_CUDA;
        if (!current_context_id(&id)) return NS3D_ERR_CUDA;
        int slot = -1;
        for (int q = 0; q < g_cached; ++q)
            if (g_cache[q].ctx_id == id) slot = q;
        if (slot < 0) {
            slot = g_cached < kMaxContexts ? g_cached++ : (int)(id % kMaxContexts);
            g_cache[slot].ctx_id = id;
        }
        g_cache[slot].addr = static_cast<double*>(p);
        *out = static_cast<double*>(p);
        return NS3D_OK;
    }
    unsigned long long id = 0;
    if (!current_context_id(&id)) return NS3D_ERR_CUDA;
    for (int q = 0; q < g_cached; ++q)
        if (g_cache[q].ctx_id == id) {
            *out = g_cache[q].addr;
            return NS3D_OK;
        }
    fprintf(stderr, "ns3d_measurables_noalloc: first call in this context made during stream capture; "
                    "make one call before capturing\n");
    return NS3D_ERR_INVALID;
}

}  // namespace

extern "C" ns3d_status ns3d_measurables_noalloc(int N, double nu, int visc_pow, const double* d_u_hat,
                                                double* d_totals, double* d_Ek, double* d_Ok, void* stream) {
    if (N <= 2 || (N % 2) != 0 || !d_u_hat || !d_totals || (visc_pow != 1 && visc_pow != 2)) return NS3D_ERR_INVALID;
    // the state is read as 16-byte complex pairs, the outputs as doubles
    if ((reinterpret_cast<uintptr_t>(d_u_hat) & 15) != 0 || (reinterpret_cast<uintptr_t>(d_totals) & 7) != 0 ||
        (reinterpret_cast<uintptr_t>(d_Ek) & 7) != 0 || (reinterpret_cast<uintptr_t>(d_Ok) & 7) != 0)
        return NS3D_ERR_INVALID;
    const int nsp = ns3d_n_spect(N);
    const long long nparts = ((long long)N * N + kLinesPerCta - 1) / kLinesPerCta;
    const long long need = nparts * (5 + 2 * (long long)nsp);
    if (N > kMaxN || need > (long long)kScratchDoubles) {
        fprintf(stderr, "ns3d_measurables_noalloc: N=%d needs %lld scratch doubles; the static scratch holds %zu "
                        "(N <= %d). Use ns3d_measurables on a context for larger grids.\n",
                N, need, kScratchDoubles, kMaxN);
        return NS3D_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    const ns3d_status st = scratch_address(s, &scratch);
    if (st != NS3D_OK) return st;
    // each launch's own status: an earlier error of the caller's program is
    // neither reported as ours nor cleared
    const size_t smem = sizeof(double) * ((size_t)kWarps * 2 * nsp + (size_t)kWarps * 5);
    const double2* u = reinterpret_cast<const double2*>(d_u_hat);
    void* a1[] = {(void*)&u, (void*)&N, (void*)&nu, (void*)&visc_pow, (void*)&nsp, (void*)&scratch};
    if (cudaLaunchKernel((const void*)k_measure_ref, dim3((unsigned)nparts), dim3(kWarps * 32), a1, smem, s) !=
        cudaSuccess)
        return NS3D_ERR_CUDA;
    const double N3 = (double)N * N * N;
    const double N3sq = N3 * N3;
    const int width = 5 + 2 * nsp;
    const int np = (int)nparts;
    const double* part = scratch;
    void* a2[] = {(void*)&part, (void*)&np, (void*)&nsp, (void*)&N3sq, (void*)&d_totals, (void*)&d_Ek, (void*)&d_Ok};
    if (cudaLaunchKernel((const void*)k_reduce_out, dim3((width + 127) / 128), dim3(128), a2, 0, s) != cudaSuccess)
        return NS3D_ERR_CUDA;
    return NS3D_OK;
}
