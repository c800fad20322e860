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
// Limits and sharing:
//   * N <= 512 (the partials of a 512^3 grid fill at most 228,608 of the
//     262,144 doubles = 2 MiB of the array); larger N is rejected.
//   * The array exists once per device for as long as the library is loaded,
//     on every GPU that loads it.
//   * Every call uses the same array and leaves its contents behind. Each call
//     writes every slot it later reads, so nothing has to be cleared, but two
//     calls whose kernels overlap on the GPU (different streams, or different
//     host threads) race on the array and corrupt each other's results.
//   * The first call on a device, with that device current, looks up the
//     array's device address (cudaGetSymbolAddress); make that first call
//     before any stream capture begins.
#include <mutex>
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
constexpr int kMaxDevices = 64;
double* g_addr[kMaxDevices] = {};

}  // namespace

extern "C" ns3d_status ns3d_measurables_noalloc(int N, double nu, int visc_pow, const double* d_u_hat,
                                                double* d_totals, double* d_Ek, double* d_Ok, void* stream) {
    if (N <= 2 || (N % 2) != 0 || !d_u_hat || !d_totals || (visc_pow != 1 && visc_pow != 2)) return NS3D_ERR_INVALID;
    const int nsp = ns3d_n_spect(N);
    const long long nparts = ((long long)N * N + kLinesPerCta - 1) / kLinesPerCta;
    const long long need = nparts * (5 + 2 * (long long)nsp);
    if (N > kMaxN || need > (long long)kScratchDoubles) {
        fprintf(stderr, "ns3d_measurables_noalloc: N=%d needs %lld scratch doubles; the static scratch holds %zu "
                        "(N <= %d). Use ns3d_measurables on a context for larger grids.\n",
                N, need, kScratchDoubles, kMaxN);
        return NS3D_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NS3D_ERR_CUDA;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return NS3D_ERR_CUDA;
            g_addr[dev] = static_cast<double*>(p);
        }
        scratch = g_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t smem = sizeof(double) * ((size_t)kWarps * 2 * nsp + (size_t)kWarps * 5);
    k_measure_ref<<<(unsigned)nparts, kWarps * 32, smem, s>>>(reinterpret_cast<const double2*>(d_u_hat), N, nu,
                                                             visc_pow, nsp, scratch);
    const double N3 = (double)N * N * N;
    const int width = 5 + 2 * nsp;
    k_reduce_out<<<(width + 127) / 128, 128, 0, s>>>(scratch, (int)nparts, nsp, N3 * N3, d_totals, d_Ek, d_Ok);
    return cudaGetLastError() == cudaSuccess ? NS3D_OK : NS3D_ERR_CUDA;
}
