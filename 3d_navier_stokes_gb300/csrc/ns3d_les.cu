// ns3d_les.cu — learned subgrid closure (include/ns3d.h, ns3d_les_*).
//
// Training data: the velocity of a fine FP32 run (N_f = F * Nc) is box-filtered
// over F^3 cells into the coarse velocity ubar_i and the exact subgrid stress
// tau_ij = <u_i u_j> - ubar_i ubar_j; pairs are kept in a device dataset.
// Model: 3^3 convolutions 3 -> 32 -> 32 -> 32 -> 6 with GELU and circular
// padding, BF16 weights, FP32 accumulation (cnn.cuh), trained with Adam on
// the mean-squared error of tau in units of s_out = s_in^2, where s_in is the
// RMS of ubar over the dataset. Inference (ns3d_les_attach) adds -div(tau) to
// a coarse run once per step, subject to the energy-budget check in the step
// graph (k_sgs_flag): a step whose closure term would add energy is run as
// the plain coarse solve.
#include <math.h>
#include <string.h>

#include <vector>

#include "cnn.cuh"
#include "cnn_tc.cuh"
#include "ns3d_ctx.h"

namespace ns3d {

// ubar, tau over F^3 boxes of a fine [3][Nf^3] velocity
__global__ void k_box_filter(const float* __restrict__ u, int Nf, int F, float* __restrict__ ubar,
                             float* __restrict__ tau) {
    const int Nc = Nf / F;
    const long long Nc3 = (long long)Nc * Nc * Nc, Nf3 = (long long)Nf * Nf * Nf;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < Nc3; q += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(q / ((long long)Nc * Nc)), cy = (int)((q / Nc) % Nc), cz = (int)(q % Nc);
        double s[3] = {0, 0, 0}, ss[6] = {0, 0, 0, 0, 0, 0};
        for (int a = 0; a < F; ++a)
            for (int b = 0; b < F; ++b)
                for (int c = 0; c < F; ++c) {
                    const long long p = ((long long)(cx * F + a) * Nf + (cy * F + b)) * Nf + (cz * F + c);
                    const double v0 = u[p], v1 = u[Nf3 + p], v2 = u[2 * Nf3 + p];
                    s[0] += v0; s[1] += v1; s[2] += v2;
                    ss[0] += v0 * v0; ss[1] += v1 * v1; ss[2] += v2 * v2;
                    ss[3] += v0 * v1; ss[4] += v0 * v2; ss[5] += v1 * v2;
                }
        const double inv = 1.0 / ((double)F * F * F);
        const double m[3] = {s[0] * inv, s[1] * inv, s[2] * inv};
        for (int c = 0; c < 3; ++c) ubar[c * Nc3 + q] = (float)m[c];
        tau[q] = (float)(ss[0] * inv - m[0] * m[0]);
        tau[Nc3 + q] = (float)(ss[1] * inv - m[1] * m[1]);
        tau[2 * Nc3 + q] = (float)(ss[2] * inv - m[2] * m[2]);
        tau[3 * Nc3 + q] = (float)(ss[3] * inv - m[0] * m[1]);
        tau[4 * Nc3 + q] = (float)(ss[4] * inv - m[0] * m[2]);
        tau[5 * Nc3 + q] = (float)(ss[5] * inv - m[1] * m[2]);
    }
}

// [3][Nc^3] floats -> reference real layout [Nc][Nc][Nc+2][3] doubles
__global__ void k_to_ref_real(const float* __restrict__ r, int N, double* __restrict__ out) {
    const long long total = (long long)N * N * (N + 2), N3 = (long long)N * N * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % (N + 2));
        const long long ij = q / (N + 2);
        for (int c = 0; c < 3; ++c) out[q * 3 + c] = k < N ? (double)r[c * N3 + ij * N + k] : 0.0;
    }
}

__global__ void k_sumsq(const float* __restrict__ x, long long n, double* __restrict__ part) {
    __shared__ double red[256];
    double s = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        s += (double)x[q] * x[q];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

}  // namespace ns3d

namespace {
constexpr int C = 32;   // hidden channels
// offsets of the flat parameter vector
constexpr int oW1 = 0, ob1 = oW1 + C * 3 * 27, oW2 = ob1 + C, ob2 = oW2 + C * C * 27, oW3 = ob2 + C,
              ob3 = oW3 + C * C * 27, oW4 = ob3 + C, ob4 = oW4 + 6 * C * 27, NPARAM = ob4 + 6;
constexpr int NPART = 256;
constexpr int kTrainChunk = 64;   // Adam iterations queued between host checks of the losses
constexpr int kChanParts = 32;    // CTAs per channel of the output-bias gradient sum
// packed tensor-core B operands of the four layers (BF16 elements):
// (KC, NO) = (2, 32), (4, 32), (4, 32), (4, 16); 9 x 3 NO x 8 KC each
constexpr int kTcW1 = 9 * 96 * 2 * 8, kTcW2 = 9 * 96 * 4 * 8, kTcW4 = 9 * 48 * 4 * 8;
constexpr int oT1 = 0, oT2 = oT1 + kTcW1, oT3 = oT2 + kTcW2, oT4 = oT3 + kTcW2, kTcWTotal = oT4 + kTcW4;
// packed B operands of the input-gradient convolutions (transposed, mirrored
// weights): layer 4 (6 -> 32, KC 2), layers 3 and 2 (32 -> 32, KC 4)
constexpr int kTcT4 = 9 * 96 * 2 * 8, kTcT3 = 9 * 96 * 4 * 8;
constexpr int oU4 = 0, oU3 = oU4 + kTcT4, oU2 = oU3 + kTcT3, kTcTTotal = oU2 + kTcT3;

unsigned long long sm64(unsigned long long& s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
}  // namespace

struct ns3d_les : public ns3d::LesHook {
    int Nc = 0, cap = 0, count = 0;
    long long D3 = 0;
    float *data_u = nullptr, *data_t = nullptr;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16* wb = nullptr;
    float *z1 = nullptr, *z2 = nullptr, *z3 = nullptr, *y = nullptr, *gy = nullptr, *gz3 = nullptr,
          *gz2 = nullptr, *gz1 = nullptr, *io_u = nullptr, *io_t = nullptr;
    double* part = nullptr;
    double* part_host = nullptr;
    // tensor-core inference (Nc in {16, 32, 64})
    __nv_bfloat16* wtc = nullptr;                        // packed B operands
    __nv_bfloat16 *act0 = nullptr, *act1 = nullptr, *act2 = nullptr, *act3 = nullptr;   // blocked BF16 activations
    int* dstat = nullptr;                                // device status word
    // tensor-core training (Nc in {16, 32, 64}): transposed weight packs, the
    // weight-gradient operand copies of the activations a0 (wg-A, 8 channels) ..
    // a3 and of the gradients d1 .. d4 (wg-B, three z-shifted copies; d4: 16 channels), the
    // weight-gradient partial sums, a zero bias
    __nv_bfloat16* wtc_t = nullptr;
    __nv_bfloat16 *a0cm = nullptr, *a1cm = nullptr, *a2cm = nullptr, *a3cm = nullptr;
    __nv_bfloat16 *d1cm = nullptr, *d2cm = nullptr, *d3cm = nullptr, *d4cm = nullptr;
    float* wpart = nullptr;
    float* zeros = nullptr;
    // training: the losses of one chunk of Adam iterations (device, pinned host) and
    // the device word that stops the updates after a non-finite loss or a failed wait
    double* losses = nullptr;
    double* losses_host = nullptr;
    int* halt = nullptr;
    float* chanp = nullptr;   // output-bias gradient partial sums [6][kChanParts]
    int wg_grid = 0;
    int train_path = 0;                                  // 0: tensor cores where compiled, 1: FP32 CUDA cores
    int tc_grid[3] = {0, 0, 0};                          // CTAs of the three kernel shapes
    double s_in = 1.0, s_out = 1.0;
    bool scales_set = false;
    long long adam_t = 0;
    unsigned long long rng = 0;
    cudaStream_t stream = nullptr;
    char err[512] = {0};

    unsigned grid() const { return (unsigned)(D3 / 256); }

    void fwd(const float* u, float* out, float in_scale, float out_scale, cudaStream_t s) {
        using namespace ns3d::cnn;
        k_conv3<3, C, false, false, false><<<grid(), 256, 0, s>>>(u, wb + oW1, w + ob1, nullptr, z1, Nc, in_scale, 1.f);
        k_conv3<C, C, true, false, false><<<grid(), 256, 0, s>>>(z1, wb + oW2, w + ob2, nullptr, z2, Nc, 1.f, 1.f);
        k_conv3<C, C, true, false, false><<<grid(), 256, 0, s>>>(z2, wb + oW3, w + ob3, nullptr, z3, Nc, 1.f, 1.f);
        k_conv3<C, 6, true, false, false><<<grid(), 256, 0, s>>>(z3, wb + oW4, w + ob4, nullptr, out, Nc, 1.f,
                                                                  out_scale);
    }

    // loss partial sums (part) and gradients (g) of one sample (u raw velocity, t raw stress)
    void fwd_bwd(const float* u, const float* t, cudaStream_t s) {
        using namespace ns3d::cnn;
        const float is = (float)(1.0 / s_in);
        fwd(u, y, is, 1.f, s);
        k_mse<<<NPART, 256, 0, s>>>(y, t, (float)(1.0 / s_out), gy, 6 * D3, part);
        k_conv3_wgrad<true><<<6 * C, 256, 0, s>>>(gy, z3, g + oW4, g + ob4, C, Nc, 1.f);
        k_conv3<6, C, false, true, true><<<grid(), 256, 0, s>>>(gy, wb + oW4, nullptr, z3, gz3, Nc, 1.f, 1.f);
        k_conv3_wgrad<true><<<C * C, 256, 0, s>>>(gz3, z2, g + oW3, g + ob3, C, Nc, 1.f);
        k_conv3<C, C, false, true, true><<<grid(), 256, 0, s>>>(gz3, wb + oW3, nullptr, z2, gz2, Nc, 1.f, 1.f);
        k_conv3_wgrad<true><<<C * C, 256, 0, s>>>(gz2, z1, g + oW2, g + ob2, C, Nc, 1.f);
        k_conv3<C, C, false, true, true><<<grid(), 256, 0, s>>>(gz2, wb + oW2, nullptr, z1, gz1, Nc, 1.f, 1.f);
        k_conv3_wgrad<false><<<C * 3, 256, 0, s>>>(gz1, u, g + oW1, g + ob1, 3, Nc, is);
    }

    bool tc() const { return ns3d::cnn::tc_grid_ok(Nc) && wtc != nullptr; }
    bool tc_train() const { return tc() && wtc_t != nullptr && train_path == 0; }

    // B operands of the input-gradient convolutions from the current BF16 weights
    void pack_tc_t(cudaStream_t s) {
        if (!wtc_t) return;
        using namespace ns3d::cnn;
        PackJobs jobs{};
        jobs.job[0] = PackJob{wb + oW4, wtc_t + oU4, 6, C, 2, 32, 1};
        jobs.job[1] = PackJob{wb + oW3, wtc_t + oU3, C, C, 4, 32, 1};
        jobs.job[2] = PackJob{wb + oW2, wtc_t + oU2, C, C, 4, 32, 1};
        k_pack_jobs<<<dim3(64, 3), 256, 0, s>>>(jobs);
    }

    // dW of one layer on the tensor cores, reduced into g + off (cin x cout x 27)
    // (and, with boff >= 0, db of the layer into g + boff)
    template <int CI, int NB, int LOGD>
    void wgrad_tc(const __nv_bfloat16* a, const __nv_bfloat16* d, int cin, int cout, int off, int boff,
                  cudaStream_t s) {
        using namespace ns3d::cnn;
        using WG = WgGeo<CI, NB, LOGD>;
        const int grid = wg_grid < WG::D * WG::D ? wg_grid : WG::D * WG::D;
        k_wgrad_tc<CI, NB, LOGD><<<grid, kTcThreads, WG::SMEM, s>>>(reinterpret_cast<const uint4*>(a),
                                                                     reinterpret_cast<const uint4*>(d), wpart, dstat);
        k_wgrad_reduce<<<(WG::PART + 255) / 256, 256, 0, s>>>(wpart, grid, CI, NB, WG::NGRP, cin, cout, g + off,
                                                             boff >= 0 ? g + boff : nullptr);
    }

    // loss and gradients of one sample on the tensor cores (BF16 operands, FP32
    // accumulation): forward with the pre-activations kept, then per layer the
    // bias and weight gradients and the input gradient
    template <int LOGD>
    void fwd_bwd_tc_d(const float* u, const float* t, cudaStream_t s) {
        using namespace ns3d::cnn;
        constexpr int D = 1 << LOGD;
        const float is = (float)(1.0 / s_in);
        const uint4* W = reinterpret_cast<const uint4*>(wtc);
        const uint4* WT = reinterpret_cast<const uint4*>(wtc_t);
        uint4* b0 = reinterpret_cast<uint4*>(act0);
        uint4* b1 = reinterpret_cast<uint4*>(act1);
        uint4* b2 = reinterpret_cast<uint4*>(act2);
        uint4* b3 = reinterpret_cast<uint4*>(act3);
        const unsigned eg = (unsigned)((D3 + 255) / 256);
        k_to_blocked<LOGD><<<eg, 256, 0, s>>>(u, is, b0);
        k_to_wga<LOGD><<<eg, 256, 0, s>>>(u, is, reinterpret_cast<uint4*>(a0cm));
        k_conv3_tc<2, 32, LOGD, 2><<<tc_grid[0], kConvThreads, tc_smem_bytes(2, 32, D), s>>>(
            b0, W + oT1 / 8, w + ob1, b1, C, 1.f, dstat, z1, a1cm);
        k_conv3_tc<4, 32, LOGD, 2><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            b1, W + oT2 / 8, w + ob2, b2, C, 1.f, dstat, z2, a2cm);
        k_conv3_tc<4, 32, LOGD, 2><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            b2, W + oT3 / 8, w + ob3, b3, C, 1.f, dstat, z3, a3cm);
        k_conv3_tc<4, 16, LOGD, 1><<<tc_grid[2], kConvThreads, tc_smem_bytes(4, 16, D), s>>>(
            b3, W + oT4 / 8, w + ob4, y, 6, 1.f, dstat);
        k_mse<<<NPART, 256, 0, s>>>(y, t, (float)(1.0 / s_out), gy, 6 * D3, part);
        // layer 4: d4 = dloss/dy (blocked into b0, which the forward no longer needs)
        k_grad_pack<LOGD><<<eg, 256, 0, s>>>(gy, b0, reinterpret_cast<uint4*>(d4cm));
        k_chan_partial<<<dim3(kChanParts, 6), 256, 0, s>>>(gy, D3, chanp);
        k_chan_final<<<1, 32, 0, s>>>(chanp, kChanParts, 6, g + ob4);
        wgrad_tc<32, 16, LOGD>(a3cm, d4cm, C, 6, oW4, -1, s);
        k_conv3_tc<2, 32, LOGD, 3><<<tc_grid[0], kConvThreads, tc_smem_bytes(2, 32, D), s>>>(
            b0, WT + oU4 / 8, zeros, b3, C, 1.f, dstat, z3, d3cm);
        // layer 3
        wgrad_tc<32, 32, LOGD>(a2cm, d3cm, C, C, oW3, ob3, s);
        k_conv3_tc<4, 32, LOGD, 3><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            b3, WT + oU3 / 8, zeros, b2, C, 1.f, dstat, z2, d2cm);
        // layer 2
        wgrad_tc<32, 32, LOGD>(a1cm, d2cm, C, C, oW2, ob2, s);
        k_conv3_tc<4, 32, LOGD, 3><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            b2, WT + oU2 / 8, zeros, b1, C, 1.f, dstat, z1, d1cm);
        // layer 1
        wgrad_tc<8, 32, LOGD>(a0cm, d1cm, 3, C, oW1, ob1, s);
    }
    void fwd_bwd_tc(const float* u, const float* t, cudaStream_t s) {
        if (Nc == 16) fwd_bwd_tc_d<4>(u, t, s);
        else if (Nc == 32) fwd_bwd_tc_d<5>(u, t, s);
        else fwd_bwd_tc_d<6>(u, t, s);
    }
    // the training path's gradients (tensor cores where compiled and selected), and
    // the sample's loss into the device slot *loss_slot
    void fwd_bwd_train(const float* u, const float* t, double* loss_slot, cudaStream_t s) {
        if (tc_train()) fwd_bwd_tc(u, t, s);
        else fwd_bwd(u, t, s);
        ns3d::cnn::k_loss_store<<<1, 32, 0, s>>>(part, NPART, (double)(6 * D3), loss_slot);
    }
    // the same, synchronously: the loss, or NaN when a bounded wait gave up
    double fwd_bwd_sync(const float* u, const float* t, cudaStream_t s) {
        fwd_bwd_train(u, t, losses, s);
        cudaMemcpyAsync(losses_host, losses, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(part_host + NPART, dstat, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        if (*reinterpret_cast<const int*>(part_host + NPART) != 0) return NAN;
        return losses_host[0];
    }

    // B operands of the tensor-core layers from the current BF16 weights
    void pack_tc(cudaStream_t s) {
        if (!tc()) return;
        using namespace ns3d::cnn;
        PackJobs jobs{};
        jobs.job[0] = PackJob{wb + oW1, wtc + oT1, C, 3, 2, 32, 0};
        jobs.job[1] = PackJob{wb + oW2, wtc + oT2, C, C, 4, 32, 0};
        jobs.job[2] = PackJob{wb + oW3, wtc + oT3, C, C, 4, 32, 0};
        jobs.job[3] = PackJob{wb + oW4, wtc + oT4, 6, C, 4, 16, 0};
        k_pack_jobs<<<dim3(64, 4), 256, 0, s>>>(jobs);
    }

    // tensor-core inference: four implicit-GEMM convolutions on blocked BF16 activations
    template <int LOGD>
    void infer_tc_d(const float* u, float* tau, float in_scale, float out_scale, cudaStream_t s) {
        using namespace ns3d::cnn;
        constexpr int D = 1 << LOGD;
        const uint4* W = reinterpret_cast<const uint4*>(wtc);
        uint4* a0 = reinterpret_cast<uint4*>(act0);
        uint4* a1 = reinterpret_cast<uint4*>(act1);
        uint4* a2 = reinterpret_cast<uint4*>(act2);
        uint4* a3 = reinterpret_cast<uint4*>(act3);
        k_to_blocked<LOGD><<<(unsigned)((D3 + 255) / 256), 256, 0, s>>>(u, in_scale, a0);
        k_conv3_tc<2, 32, LOGD, 0><<<tc_grid[0], kConvThreads, tc_smem_bytes(2, 32, D), s>>>(
            a0, W + oT1 / 8, w + ob1, a1, C, 1.f, dstat);
        k_conv3_tc<4, 32, LOGD, 0><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            a1, W + oT2 / 8, w + ob2, a2, C, 1.f, dstat);
        k_conv3_tc<4, 32, LOGD, 0><<<tc_grid[1], kConvThreads, tc_smem_bytes(4, 32, D), s>>>(
            a2, W + oT3 / 8, w + ob3, a3, C, 1.f, dstat);
        k_conv3_tc<4, 16, LOGD, 1><<<tc_grid[2], kConvThreads, tc_smem_bytes(4, 16, D), s>>>(
            a3, W + oT4 / 8, w + ob4, tau, 6, out_scale, dstat);
    }
    void infer_tc(const float* u, float* tau, float in_scale, float out_scale, cudaStream_t s) {
        if (Nc == 16) infer_tc_d<4>(u, tau, in_scale, out_scale, s);
        else if (Nc == 32) infer_tc_d<5>(u, tau, in_scale, out_scale, s);
        else infer_tc_d<6>(u, tau, in_scale, out_scale, s);
    }

    void forward(const float* u, float* tau, int N, cudaStream_t s) override {
        (void)N;
        if (tc()) infer_tc(u, tau, (float)(1.0 / s_in), (float)s_out, s);
        else fwd(u, tau, (float)(1.0 / s_in), (float)s_out, s);
    }
    int* status_word() override { return dstat; }

    ~ns3d_les() override {
        for (void* q : {(void*)data_u, (void*)data_t, (void*)w, (void*)g, (void*)m, (void*)v, (void*)wb, (void*)z1,
                        (void*)z2, (void*)z3, (void*)y, (void*)gy, (void*)gz3, (void*)gz2, (void*)gz1, (void*)io_u,
                        (void*)io_t, (void*)part, (void*)wtc, (void*)act0, (void*)act1, (void*)act2, (void*)act3,
                        (void*)dstat, (void*)wtc_t, (void*)a0cm, (void*)a1cm, (void*)a2cm, (void*)a3cm, (void*)d1cm,
                        (void*)d2cm, (void*)d3cm, (void*)d4cm, (void*)wpart, (void*)zeros, (void*)losses, (void*)halt, (void*)chanp})
            if (q) cudaFree(q);
        if (part_host) cudaFreeHost(part_host);
        if (losses_host) cudaFreeHost(losses_host);
        if (stream) cudaStreamDestroy(stream);
    }
};

// shared-memory opt-in and persistent grid sizes of the tensor-core kernels
template <int LOGD>
static ns3d_status les_tc_setup_d(ns3d_les* l, int nsm) {
    using namespace ns3d::cnn;
    constexpr int D = 1 << LOGD, ntiles = D * D * D / 128;
    const void* fns[3] = {(const void*)k_conv3_tc<2, 32, LOGD, 0>, (const void*)k_conv3_tc<4, 32, LOGD, 0>,
                          (const void*)k_conv3_tc<4, 16, LOGD, 1>};
    const uint32_t sm[3] = {tc_smem_bytes(2, 32, D), tc_smem_bytes(4, 32, D), tc_smem_bytes(4, 16, D)};
    for (int k = 0; k < 3; ++k) {
        if (cudaFuncSetAttribute(fns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm[k]) != cudaSuccess)
            return NS3D_ERR_CUDA;
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fns[k], kConvThreads, sm[k]) != cudaSuccess || per < 1)
            return NS3D_ERR_CUDA;
        l->tc_grid[k] = per * nsm < ntiles ? per * nsm : ntiles;
    }
    // training: the same layer shapes in the training modes, and the weight-gradient kernels
    const void* tfns[4] = {(const void*)k_conv3_tc<2, 32, LOGD, 2>, (const void*)k_conv3_tc<4, 32, LOGD, 2>,
                           (const void*)k_conv3_tc<2, 32, LOGD, 3>, (const void*)k_conv3_tc<4, 32, LOGD, 3>};
    const uint32_t tsm[4] = {tc_smem_bytes(2, 32, D), tc_smem_bytes(4, 32, D), tc_smem_bytes(2, 32, D),
                             tc_smem_bytes(4, 32, D)};
    for (int k = 0; k < 4; ++k)
        if (cudaFuncSetAttribute(tfns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm[k]) != cudaSuccess)
            return NS3D_ERR_CUDA;
    const void* wfns[3] = {(const void*)k_wgrad_tc<32, 16, LOGD>, (const void*)k_wgrad_tc<32, 32, LOGD>,
                           (const void*)k_wgrad_tc<8, 32, LOGD>};
    const uint32_t wsm[3] = {WgGeo<32, 16, LOGD>::SMEM, WgGeo<32, 32, LOGD>::SMEM, WgGeo<8, 32, LOGD>::SMEM};
    for (int k = 0; k < 3; ++k)
        if (cudaFuncSetAttribute(wfns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm[k]) != cudaSuccess)
            return NS3D_ERR_CUDA;
    l->wg_grid = nsm;
    return NS3D_OK;
}

static ns3d_status les_tc_setup(ns3d_les* l) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return NS3D_ERR_CUDA;
    if (l->Nc == 16) return les_tc_setup_d<4>(l, nsm);
    if (l->Nc == 32) return les_tc_setup_d<5>(l, nsm);
    return les_tc_setup_d<6>(l, nsm);
}

static ns3d_status les_fail(ns3d_les* l, ns3d_status s, const char* msg) {
    if (l) snprintf(l->err, sizeof(l->err), "%s", msg);
    return s;
}

#define LES_CK(call)                                                          \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) return les_fail(l, NS3D_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

extern "C" {

int ns3d_les_num_params(void) { return NPARAM; }

ns3d_status ns3d_les_create(int Nc, int capacity, uint64_t seed, ns3d_les** out) {
    if (!out || Nc < 8 || Nc % 8 != 0 || capacity < 0) return NS3D_ERR_INVALID;
    *out = nullptr;
    ns3d_les* l = new ns3d_les();
    l->Nc = Nc;
    l->cap = capacity;
    l->D3 = (long long)Nc * Nc * Nc;
    l->rng = seed;
    const size_t f = sizeof(float);
    if (cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&l->w, f * NPARAM) != cudaSuccess || cudaMalloc(&l->g, f * NPARAM) != cudaSuccess ||
        cudaMalloc(&l->m, f * NPARAM) != cudaSuccess || cudaMalloc(&l->v, f * NPARAM) != cudaSuccess ||
        cudaMalloc(&l->wb, sizeof(__nv_bfloat16) * NPARAM) != cudaSuccess ||
        cudaMalloc(&l->z1, f * C * l->D3) != cudaSuccess || cudaMalloc(&l->z2, f * C * l->D3) != cudaSuccess ||
        cudaMalloc(&l->z3, f * C * l->D3) != cudaSuccess || cudaMalloc(&l->y, f * 6 * l->D3) != cudaSuccess ||
        cudaMalloc(&l->gy, f * 6 * l->D3) != cudaSuccess || cudaMalloc(&l->gz3, f * C * l->D3) != cudaSuccess ||
        cudaMalloc(&l->gz2, f * C * l->D3) != cudaSuccess || cudaMalloc(&l->gz1, f * C * l->D3) != cudaSuccess ||
        cudaMalloc(&l->io_u, f * 3 * l->D3) != cudaSuccess || cudaMalloc(&l->io_t, f * 6 * l->D3) != cudaSuccess ||
        cudaMalloc(&l->part, sizeof(double) * NPART) != cudaSuccess ||
        cudaMallocHost(&l->part_host, sizeof(double) * (NPART + 1)) != cudaSuccess ||
        cudaMalloc(&l->losses, sizeof(double) * kTrainChunk) != cudaSuccess ||
        cudaMallocHost(&l->losses_host, sizeof(double) * kTrainChunk) != cudaSuccess ||
        cudaMalloc(&l->halt, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&l->chanp, sizeof(float) * 6 * kChanParts) != cudaSuccess ||
        (capacity > 0 && (cudaMalloc(&l->data_u, f * 3 * l->D3 * capacity) != cudaSuccess ||
                          cudaMalloc(&l->data_t, f * 6 * l->D3 * capacity) != cudaSuccess))) {
        delete l;
        cudaGetLastError();
        return NS3D_ERR_NOMEM;
    }
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights from SplitMix64, zero biases,
    // the output layer scaled down so that the untrained closure starts small
    std::vector<float> h(NPARAM, 0.0f);
    unsigned long long s = seed ^ 0x5bd1e995ull;
    auto fill = [&](int off, int n, int fan_in, float gain) {
        const float b = gain / sqrtf((float)fan_in);
        for (int i = 0; i < n; ++i) h[off + i] = b * (2.0f * (float)((sm64(s) >> 11) * 0x1.0p-53) - 1.0f);
    };
    fill(oW1, C * 3 * 27, 3 * 27, 1.0f);
    fill(oW2, C * C * 27, C * 27, 1.0f);
    fill(oW3, C * C * 27, C * 27, 1.0f);
    fill(oW4, 6 * C * 27, C * 27, 0.1f);
    cudaMemcpy(l->w, h.data(), f * NPARAM, cudaMemcpyHostToDevice);
    cudaMemset(l->m, 0, f * NPARAM);
    cudaMemset(l->v, 0, f * NPARAM);
    ns3d::cnn::k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, l->stream>>>(l->w, l->wb, NPARAM);
    if (cudaMalloc(&l->dstat, sizeof(int)) != cudaSuccess || cudaMemset(l->dstat, 0, sizeof(int)) != cudaSuccess) {
        delete l;
        return NS3D_ERR_NOMEM;
    }
    if (ns3d::cnn::tc_grid_ok(Nc)) {
        const size_t a = sizeof(__nv_bfloat16) * C * (size_t)l->D3;
        const size_t dpad = 3 * a;   // the three z-shifted wg-B copies of a gradient
        int nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (cudaMalloc(&l->wtc, sizeof(__nv_bfloat16) * kTcWTotal) != cudaSuccess || cudaMalloc(&l->act0, a / 2) != cudaSuccess ||
            cudaMalloc(&l->act1, a) != cudaSuccess ||
            cudaMalloc(&l->act2, a) != cudaSuccess || cudaMalloc(&l->act3, a) != cudaSuccess ||
            cudaMalloc(&l->wtc_t, sizeof(__nv_bfloat16) * kTcTTotal) != cudaSuccess ||
            cudaMalloc(&l->a0cm, a / 4) != cudaSuccess || cudaMalloc(&l->a1cm, a) != cudaSuccess ||
            cudaMalloc(&l->a2cm, a) != cudaSuccess || cudaMalloc(&l->a3cm, a) != cudaSuccess ||
            cudaMalloc(&l->d1cm, dpad) != cudaSuccess || cudaMalloc(&l->d2cm, dpad) != cudaSuccess ||
            cudaMalloc(&l->d3cm, dpad) != cudaSuccess || cudaMalloc(&l->d4cm, dpad / 2) != cudaSuccess ||
            cudaMalloc(&l->wpart, sizeof(float) * 3 * 128 * 96 * (size_t)(nsm > 0 ? nsm : 1)) != cudaSuccess ||
            cudaMalloc(&l->zeros, sizeof(float) * C) != cudaSuccess || cudaMemset(l->zeros, 0, sizeof(float) * C) != cudaSuccess ||
            les_tc_setup(l) != NS3D_OK) {
            delete l;
            cudaGetLastError();
            return NS3D_ERR_NOMEM;
        }
        l->pack_tc(l->stream);
        l->pack_tc_t(l->stream);
    }
    if (cudaStreamSynchronize(l->stream) != cudaSuccess) {
        delete l;
        return NS3D_ERR_CUDA;
    }
    *out = l;
    return NS3D_OK;
}

ns3d_status ns3d_les_destroy(ns3d_les* l) {
    if (!l) return NS3D_ERR_INVALID;
    delete l;
    return NS3D_OK;
}

const char* ns3d_les_last_error(const ns3d_les* l) { return l ? l->err : "null closure"; }

static ns3d_status les_filter(ns3d_les* l, ns3d_ctx* fine, float* ubar, float* tau) {
    if (!l || !fine) return NS3D_ERR_INVALID;
    const int Nf = fine->p.N;
    if (Nf % l->Nc != 0 || Nf < l->Nc) return les_fail(l, NS3D_ERR_INVALID, "fine grid is not a multiple of Nc");
    ns3d_status st = NS3D_OK;
    const float* u = fine->impl->real_velocity_f32(&st);
    if (st != NS3D_OK) return les_fail(l, st, fine->impl->err());
    // the fine run's stream produced u; the filter runs on it too
    ns3d::k_box_filter<<<(unsigned)((l->D3 + 255) / 256), 256, 0, fine->stream>>>(u, Nf, Nf / l->Nc, ubar, tau);
    LES_CK(cudaStreamSynchronize(fine->stream));
    return NS3D_OK;
}

ns3d_status ns3d_les_add_snapshot(ns3d_les* l, ns3d_ctx* fine) {
    if (!l) return NS3D_ERR_INVALID;
    if (l->count >= l->cap) return les_fail(l, NS3D_ERR_INVALID, "dataset is full");
    ns3d_status st = les_filter(l, fine, l->data_u + 3 * l->D3 * l->count, l->data_t + 6 * l->D3 * l->count);
    if (st == NS3D_OK) l->count++;
    return st;
}

ns3d_status ns3d_les_dataset_size(ns3d_les* l, int* count) {
    if (!l || !count) return NS3D_ERR_INVALID;
    *count = l->count;
    return NS3D_OK;
}

ns3d_status ns3d_les_filtered_velocity_host(ns3d_les* l, ns3d_ctx* fine, double* ubar) {
    if (!l || !ubar) return NS3D_ERR_INVALID;
    ns3d_status st = les_filter(l, fine, l->io_u, l->io_t);
    if (st != NS3D_OK) return st;
    const int N = l->Nc;
    double* d = nullptr;
    const size_t bytes = sizeof(double) * 3 * (size_t)N * N * (N + 2);
    LES_CK(cudaMalloc(&d, bytes));
    ns3d::k_to_ref_real<<<256, 256, 0, l->stream>>>(l->io_u, N, d);
    cudaError_t e = cudaMemcpyAsync(ubar, d, bytes, cudaMemcpyDeviceToHost, l->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(l->stream);
    cudaFree(d);
    return e == cudaSuccess ? NS3D_OK : les_fail(l, NS3D_ERR_CUDA, cudaGetErrorString(e));
}

ns3d_status ns3d_les_set_scales(ns3d_les* l, double s_in, double s_out) {
    if (!l || !(s_in > 0) || !(s_out > 0)) return NS3D_ERR_INVALID;
    l->s_in = s_in;
    l->s_out = s_out;
    l->scales_set = true;
    return NS3D_OK;
}

ns3d_status ns3d_les_get_scales(ns3d_les* l, double* s_in, double* s_out) {
    if (!l) return NS3D_ERR_INVALID;
    if (s_in) *s_in = l->s_in;
    if (s_out) *s_out = l->s_out;
    return NS3D_OK;
}

static ns3d_status les_auto_scales(ns3d_les* l) {
    if (l->scales_set) return NS3D_OK;
    if (l->count == 0) return les_fail(l, NS3D_ERR_INVALID, "empty dataset");
    const long long n = 3 * l->D3 * l->count;
    ns3d::k_sumsq<<<NPART, 256, 0, l->stream>>>(l->data_u, n, l->part);
    LES_CK(cudaMemcpyAsync(l->part_host, l->part, sizeof(double) * NPART, cudaMemcpyDeviceToHost, l->stream));
    LES_CK(cudaStreamSynchronize(l->stream));
    double s = 0;
    for (int i = 0; i < NPART; ++i) s += l->part_host[i];
    l->s_in = sqrt(s / (double)n);
    if (!(l->s_in > 0)) l->s_in = 1.0;
    l->s_out = l->s_in * l->s_in;
    l->scales_set = true;
    return NS3D_OK;
}

ns3d_status ns3d_les_train(ns3d_les* l, int iterations, double lr, double* mean_loss) {
    if (!l || iterations < 0 || !(lr > 0)) return NS3D_ERR_INVALID;
    ns3d_status st = les_auto_scales(l);
    if (st != NS3D_OK) return st;
    LES_CK(cudaMemsetAsync(l->halt, 0, sizeof(int), l->stream));
    double acc = 0.0;
    int nacc = 0;
    const float b1 = 0.9f, b2 = 0.999f;
    // chunks of kTrainChunk iterations queued without host round trips; the samples come
    // from the host generator, each loss goes to its device slot, and the host reads the
    // chunk's losses and status once it is done
    for (int it0 = 0; it0 < iterations; it0 += kTrainChunk) {
        const int n = iterations - it0 < kTrainChunk ? iterations - it0 : kTrainChunk;
        for (int k = 0; k < n; ++k) {
            const int smp = (int)(sm64(l->rng) % (unsigned long long)l->count);
            l->fwd_bwd_train(l->data_u + 3 * l->D3 * smp, l->data_t + 6 * l->D3 * smp, l->losses + k, l->stream);
            const long long t = l->adam_t + 1 + k;
            const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
            ns3d::cnn::k_adam<<<(NPARAM + 255) / 256, 256, 0, l->stream>>>(
                l->w, l->wb, l->g, l->m, l->v, NPARAM, (float)lr, b1, b2, 1e-8f, c1, c2, l->losses + k, l->dstat, l->halt);
            if (l->tc_train()) {   // the next sample's tensor-core layers read the updated weights
                l->pack_tc(l->stream);
                l->pack_tc_t(l->stream);
            }
        }
        LES_CK(cudaMemcpyAsync(l->losses_host, l->losses, sizeof(double) * n, cudaMemcpyDeviceToHost, l->stream));
        LES_CK(cudaMemcpyAsync(l->part_host + NPART, l->dstat, sizeof(int), cudaMemcpyDeviceToHost, l->stream));
        LES_CK(cudaStreamSynchronize(l->stream));
        for (int k = 0; k < n; ++k) {
            if (!isfinite(l->losses_host[k]) || *reinterpret_cast<const int*>(l->part_host + NPART) != 0) {
                l->adam_t += k;   // the updates before the first bad sample were applied
                l->pack_tc(l->stream);
                cudaStreamSynchronize(l->stream);
                if (*reinterpret_cast<const int*>(l->part_host + NPART) != 0)
                    return les_fail(l, NS3D_ERR_TIMEOUT, "a bounded wait in a tensor-core training kernel gave up");
                return les_fail(l, NS3D_ERR_NUMERIC, "training loss is not finite");
            }
            const int it = it0 + k;
            if (it >= iterations - iterations / 10 - 1) {
                acc += l->losses_host[k];
                nacc++;
            }
        }
        l->adam_t += n;
    }
    l->pack_tc(l->stream);
    LES_CK(cudaStreamSynchronize(l->stream));
    if (mean_loss) *mean_loss = nacc ? acc / nacc : 0.0;
    return NS3D_OK;
}

ns3d_status ns3d_les_dataset_loss(ns3d_les* l, double* mean_loss) {
    if (!l || !mean_loss) return NS3D_ERR_INVALID;
    ns3d_status st = les_auto_scales(l);
    if (st != NS3D_OK) return st;
    double acc = 0.0;
    for (int smp = 0; smp < l->count; ++smp) {
        l->fwd(l->data_u + 3 * l->D3 * smp, l->y, (float)(1.0 / l->s_in), 1.f, l->stream);
        ns3d::cnn::k_mse<<<NPART, 256, 0, l->stream>>>(l->y, l->data_t + 6 * l->D3 * smp, (float)(1.0 / l->s_out),
                                                      nullptr, 6 * l->D3, l->part);
        LES_CK(cudaMemcpyAsync(l->part_host, l->part, sizeof(double) * NPART, cudaMemcpyDeviceToHost, l->stream));
        LES_CK(cudaStreamSynchronize(l->stream));
        double s = 0;
        for (int i = 0; i < NPART; ++i) s += l->part_host[i];
        acc += s / (double)(6 * l->D3);
    }
    *mean_loss = l->count ? acc / l->count : 0.0;
    return NS3D_OK;
}

ns3d_status ns3d_les_weights_host(ns3d_les* l, float* w, int set) {
    if (!l || !w) return NS3D_ERR_INVALID;
    if (set) {
        LES_CK(cudaMemcpy(l->w, w, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
        ns3d::cnn::k_to_bf16<<<(NPARAM + 255) / 256, 256, 0, l->stream>>>(l->w, l->wb, NPARAM);
        l->pack_tc(l->stream);
        LES_CK(cudaStreamSynchronize(l->stream));
    } else {
        LES_CK(cudaMemcpy(w, l->w, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    }
    return NS3D_OK;
}

ns3d_status ns3d_les_gradients_host(ns3d_les* l, const float* u, const float* tau, double* loss, float* grads) {
    if (!l || !u || !tau) return NS3D_ERR_INVALID;
    LES_CK(cudaMemcpy(l->io_u, u, sizeof(float) * 3 * l->D3, cudaMemcpyHostToDevice));
    LES_CK(cudaMemcpy(l->io_t, tau, sizeof(float) * 6 * l->D3, cudaMemcpyHostToDevice));
    const double ls = l->fwd_bwd_sync(l->io_u, l->io_t, l->stream);
    if (loss) *loss = ls;
    if (grads) LES_CK(cudaMemcpy(grads, l->g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    return NS3D_OK;
}

ns3d_status ns3d_les_set_train_path(ns3d_les* l, int path) {
    if (!l || (path != 0 && path != 1)) return NS3D_ERR_INVALID;
    l->train_path = path;
    return NS3D_OK;
}

int ns3d_les_train_path(const ns3d_les* l) { return l ? (l->tc_train() ? 0 : 1) : -1; }

ns3d_status ns3d_les_forward_host(ns3d_les* l, const float* u, float* tau) {
    if (!l || !u || !tau) return NS3D_ERR_INVALID;
    LES_CK(cudaMemcpy(l->io_u, u, sizeof(float) * 3 * l->D3, cudaMemcpyHostToDevice));
    l->fwd(l->io_u, l->io_t, (float)(1.0 / l->s_in), (float)l->s_out, l->stream);
    LES_CK(cudaStreamSynchronize(l->stream));
    LES_CK(cudaMemcpy(tau, l->io_t, sizeof(float) * 6 * l->D3, cudaMemcpyDeviceToHost));
    return NS3D_OK;
}

ns3d_status ns3d_les_infer_host(ns3d_les* l, const float* u, float* tau) {
    if (!l || !u || !tau) return NS3D_ERR_INVALID;
    LES_CK(cudaMemcpy(l->io_u, u, sizeof(float) * 3 * l->D3, cudaMemcpyHostToDevice));
    l->forward(l->io_u, l->io_t, l->Nc, l->stream);
    LES_CK(cudaStreamSynchronize(l->stream));
    int st = 0;
    LES_CK(cudaMemcpy(&st, l->dstat, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) return les_fail(l, NS3D_ERR_TIMEOUT, "a bounded wait in the tensor-core convolution gave up");
    LES_CK(cudaMemcpy(tau, l->io_t, sizeof(float) * 6 * l->D3, cudaMemcpyDeviceToHost));
    return NS3D_OK;
}

ns3d_status ns3d_les_profile_infer(ns3d_les* l, int reps, float* ms) {
    if (!l || reps <= 0 || !ms) return NS3D_ERR_INVALID;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    LES_CK(cudaEventCreate(&e0));
    LES_CK(cudaEventCreate(&e1));
    l->forward(l->io_u, l->io_t, l->Nc, l->stream);   // warm-up
    cudaEventRecord(e0, l->stream);
    for (int r = 0; r < reps; ++r) l->forward(l->io_u, l->io_t, l->Nc, l->stream);
    cudaEventRecord(e1, l->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return les_fail(l, NS3D_ERR_CUDA, cudaGetErrorString(e));
    *ms = t / (float)reps;
    return NS3D_OK;
}

ns3d_status ns3d_les_attach(ns3d_ctx* coarse, ns3d_les* l) {
    if (!coarse) return NS3D_ERR_INVALID;
    if (l && coarse->p.N != l->Nc) return NS3D_ERR_INVALID;
    ns3d_status st = coarse->impl->attach_les(l);
    if (st != NS3D_OK) snprintf(coarse->err, sizeof(coarse->err), "%s", coarse->impl->err());
    return st;
}

ns3d_status ns3d_les_counters(ns3d_ctx* coarse, long* closure_steps, long* fallback_steps) {
    if (!coarse) return NS3D_ERR_INVALID;
    return coarse->impl->les_counters(closure_steps, fallback_steps);
}

ns3d_status ns3d_set_state_real_host(ns3d_ctx* c, const double* u) {
    if (!c || !u) return NS3D_ERR_INVALID;
    ns3d_status st = c->impl->set_state_real_host(u);
    if (st != NS3D_OK) snprintf(c->err, sizeof(c->err), "%s", c->impl->err());
    return st;
}

}  // extern "C"
