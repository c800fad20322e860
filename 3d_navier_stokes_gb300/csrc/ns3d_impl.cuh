// ns3d_impl.cuh — host-side engine for one (precision, grid size): device
// memory plan, pass launches, CUDA-graph capture of a whole time step,
// diagnostics, initial conditions and layout conversion.
//
// An engine holds M independent runs ("members") of the same grid size: every
// per-run array is stored member after member, and each pass launch covers a
// contiguous range of members (the member index is blockIdx.z, or part of the
// z pass's work list). A single run is M = 1. Single-run operations (initial
// conditions, diagnostics, host transfers, time) act on the selected member.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ns3d_base.h"
#include "ns3d_kernels.cuh"

namespace ns3d {

#define NS3D_CK(call)                                                        \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            set_err("%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return NS3D_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

// e^{-2 pi i m / n} with the quarter-turn reduction used by the transforms.
void twiddle_table(int n, double* re, double* im);
// 4D FP32 tensor map without swizzle (ns3d_misc.cu)
bool encode_map4_f32(CUtensorMap* map, void* base, const uint64_t dims[4], const uint64_t strides[3],
                     const uint32_t box[4]);

template <typename T, int N, int V = 0>
class Impl final : public Base {
    using G = Geo<N>;
    using PA = typename Plans<N>::A;
    using PY = typename YPlan<T, N, true>::A;    // the inverse y pass's plan
    using PYF = typename YPlan<T, N, false>::A;  // the forward y pass's plan
    using PX = typename PlansV<N, V>::X;
    static constexpr int TA = tile_a<T, N, V>();
    static constexpr int TX = tile_x<T, N, V>();
    static constexpr int ZP = zpairs<N>();
    static constexpr int NTA = (G::NZ1 + TA - 1) / TA;
    static constexpr int TAF = tile_a<T, N, V, false>();   // forward y pass
    static constexpr int NTAF = (G::NZ1 + TAF - 1) / TAF;
    static constexpr int NTX = (G::NZ1 + TX - 1) / TX;
    static constexpr int TXF = tile_x<T, N, V, true>();   // forward x pass
    static constexpr int NTXF = (G::NZ1 + TXF - 1) / TXF;
    static constexpr int LPC = meas_lines_per_cta<N>();
    static constexpr long long NMEAS = ((long long)N * G::NKY + LPC - 1) / LPC;
    static constexpr int MWIDTH = 5 + 2 * G::NSP;

  public:
    Impl(const ns3d_params* ps, int M, cudaStream_t s) : Base(ps[0], s), M_(M), mp_(ps, ps + M) {}

    int members() const override { return M_; }
    ns3d_status select(int m) override {
        if (m < 0 || m >= M_) return NS3D_ERR_INVALID;
        m_ = m;
        return NS3D_OK;
    }
    void enqueue_step() override { launch_step(); }
    ns3d_status status() override { return check_status(); }

    // per-member views of the member-major arrays
    cx<T>* Um(int m) const { return U_ + (size_t)m * 3 * G::FS; }
    cx<T>* UTm(int m) const { return UT_ + (size_t)m * 3 * G::FS; }
    cx<T>* ACCm(int m) const { return ACC_ + (size_t)m * 3 * G::FS; }
    cx<T>* Wm(int m) const { return W_ + (size_t)m * 6 * G::FS; }
    cx<T>* tabm(int m) const { return tab_ + (size_t)m * (G::KC2 + 1); }
    StepDev* sdm(int m) const { return sd_ + m; }

    ~Impl() override {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        for (void* q : {(void*)U_, (void*)UT_, (void*)ACC_, (void*)W_, (void*)tw_, (void*)tab_, (void*)part_,
                        (void*)mout_, (void*)stage_, (void*)real_, (void*)sd_, (void*)TAU_, (void*)F_,
                        (void*)tau_real_, (void*)sgs_part_, (void*)K_, (void*)dpart_, (void*)plan_out_.ranges, (void*)plan_in_.ranges,
                        (void*)zg_b_, (void*)zg_P_, (void*)xt_items_})
            if (q) cudaFree(q);
        if (sd_host_) cudaFreeHost(sd_host_);
        if (mout_host_) cudaFreeHost(mout_host_);
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
    }

    bool rk5() const { return p_.integrator == INT_RK5CN || p_.integrator == INT_DP5CN; }
    bool dp5() const { return p_.integrator == INT_DP5CN; }
    int kernels_per_step() const override {
        const int z2 = zform_ == 2 ? 1 : 0;   // the tensor-core z pass is two kernels
        if (dp5()) return 1 + 7 * (5 + z2) + 3;
        if (rk5()) return 6 * (5 + z2) + (p_.cfl > 0 ? 1 : 0) + 1;
        return 4 * (5 + z2) + (p_.cfl > 0 ? 1 : 0) + 1;
    }

    ns3d_status init() override {
        const size_t fb = sizeof(cx<T>) * (size_t)G::FS * M_;
        NS3D_CK(cudaMalloc(&U_, 3 * fb));
        NS3D_CK(cudaMalloc(&UT_, 3 * fb));
        NS3D_CK(cudaMalloc(&ACC_, 3 * fb));
        NS3D_CK(cudaMalloc(&W_, 6 * fb));
        NS3D_CK(cudaMemsetAsync(U_, 0, 3 * fb, s_));
        NS3D_CK(cudaMemsetAsync(UT_, 0, 3 * fb, s_));
        NS3D_CK(cudaMemsetAsync(ACC_, 0, 3 * fb, s_));
        if (rk5()) {
            // stored stages k_1..k_6 of the RK5 family, and the DP5CN error partial sums
            NS3D_CK(cudaMalloc(&K_, 18 * fb));
            NS3D_CK(cudaMemsetAsync(K_, 0, 18 * fb, s_));
            NS3D_CK(cudaMalloc(&dpart_, sizeof(double) * 3 * (size_t)NTXF * G::NKY * M_));
        }
        NS3D_CK(cudaMalloc(&tw_, sizeof(cx<T>) * N));
        NS3D_CK(cudaMalloc(&tab_, sizeof(cx<T>) * (G::KC2 + 1) * M_));
        NS3D_CK(cudaMalloc(&part_, sizeof(double) * NMEAS * MWIDTH));
        NS3D_CK(cudaMalloc(&mout_, sizeof(double) * MWIDTH));
        NS3D_CK(cudaMallocHost(&mout_host_, sizeof(double) * MWIDTH));
        NS3D_CK(cudaMalloc(&sd_, sizeof(StepDev) * M_));
        NS3D_CK(cudaMallocHost(&sd_host_, sizeof(StepDev) * M_));
        NS3D_CK(cudaEventCreate(&ev0_));
        NS3D_CK(cudaEventCreate(&ev1_));
        // twiddles
        std::vector<double> re(N), im(N);
        twiddle_table(N, re.data(), im.data());
        std::vector<cx<T>> h(N);
        for (int m = 0; m < N; ++m) { h[m].x = T(re[m]); h[m].y = T(im[m]); }
        NS3D_CK(cudaMemcpyAsync(tw_, h.data(), sizeof(cx<T>) * N, cudaMemcpyHostToDevice, s_));
        // step state
        for (int m = 0; m < M_; ++m) {
            StepDev sd{};
            sd.t = mp_[m].t0; sd.dt = mp_[m].dt; sd.t0 = mp_[m].t0; sd.nu = mp_[m].nu; sd.cfl = mp_[m].cfl;
            sd.dp_atol = 1e-7; sd.dp_rtol = 1e-7;   // DP_ABS_TOL, DP_REL_TOL (data_types.h:123-124)
            sd.wait_cycles = kWaitCycles;
            sd_host_[m] = sd;
        }
        NS3D_CK(cudaMemcpyAsync(sd_, sd_host_, sizeof(StepDev) * M_, cudaMemcpyHostToDevice, s_));
        // opt-in shared memory sizes
        NS3D_CK(cudaFuncSetAttribute(k_xinv<T, N, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_xi()));
        NS3D_CK(cudaFuncSetAttribute(k_ypass<T, N, true, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_a()));
        NS3D_CK(cudaFuncSetAttribute(k_ypass<T, N, false, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_af()));
        NS3D_CK(cudaFuncSetAttribute(k_zpass<T, N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_z()));
        if constexpr (zline_ok<T, N>()) {
            NS3D_CK(cudaFuncSetAttribute(k_zline<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_zl()));
            int per_sm = 0, nsm = 0, dev = 0;
            NS3D_CK(cudaGetDevice(&dev));
            NS3D_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            NS3D_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zline<T, N>, ZLINE_WARPS * 32, smem_zl()));
            zline_ctas_ = (per_sm > 0 ? per_sm : 1) * nsm;
        }
        NS3D_CK(cudaFuncSetAttribute(k_zpass<T, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_z()));
        NS3D_CK(cudaFuncSetAttribute(k_zpass<T, N, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_z()));
        if constexpr (zgemm_ok<T, N>()) {
            // z-pass form 2: DFT matrices (built once, on the host), the product workspace
            using Z = ZGeo<N>;
            NS3D_CK(cudaFuncSetAttribute(k_zgemm_inv<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, Z::SMEM_INV));
            NS3D_CK(cudaFuncSetAttribute(k_zgemm_fwd<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, Z::SMEM_FWD));
            std::vector<uint16_t> mats(2 * (size_t)N * Z::KI * 2);
            zgemm_matrices(N, Z::KI, mats.data());
            NS3D_CK(cudaMalloc(&zg_b_, sizeof(uint16_t) * mats.size()));
            NS3D_CK(cudaMemcpyAsync(zg_b_, mats.data(), sizeof(uint16_t) * mats.size(), cudaMemcpyHostToDevice, s_));
            NS3D_CK(cudaMalloc(&zg_P_, sizeof(float) * 3 * (size_t)N * N * N * M_));
            int dev = 0;
            NS3D_CK(cudaGetDevice(&dev));
            NS3D_CK(cudaDeviceGetAttribute(&zg_ctas_, cudaDevAttrMultiProcessorCount, dev));
        }
        if constexpr (xinv_tma_ok<T, N, V>()) {
            // P1 fed by tensor-tile copies: one map over the 3 M velocity components of U and one of UT
            const uint64_t dims[4] = {2ull * G::NZP, (uint64_t)N, (uint64_t)N, 3ull * (uint64_t)M_};
            const uint64_t strides[3] = {sizeof(cx<T>) * (uint64_t)G::NZP, sizeof(cx<T>) * (uint64_t)N * G::NZP,
                                         sizeof(cx<T>) * (uint64_t)G::FS};
            const uint32_t box[4] = {2u * (uint32_t)xtma_tile<T, N, V>(), 1u, (uint32_t)xbox_rows<N>(), 1u};
            // and one over the 6 M fields of W for its bulk tensor stores
            const uint64_t wdims[4] = {2ull * G::NZP, (uint64_t)N, (uint64_t)N, 6ull * (uint64_t)M_};
            const uint32_t wbox[4] = {2u * (uint32_t)xtma_tile<T, N, V>(), 1u, (uint32_t)xout_rows<N>(), 1u};
            if (!encode_map4_f32(&xmap_[0], U_, dims, strides, box) || !encode_map4_f32(&xmap_[1], UT_, dims, strides, box) ||
                !encode_map4_f32(&wmap_, W_, wdims, strides, wbox)) {
                set_err("cuTensorMapEncodeTiled failed for the x-inverse pass");
                return NS3D_ERR_CUDA;
            }
            NS3D_CK(cudaFuncSetAttribute(k_xinv_tma<T, N, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)xinv_tma_smem<T, N, V>()));
            int per_sm = 0, nsm = 0, dev = 0;
            NS3D_CK(cudaGetDevice(&dev));
            NS3D_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            NS3D_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_xinv_tma<T, N, V>,
                                                                  xtma_tile<T, N, V>() * PX::P, xinv_tma_smem<T, N, V>()));
            xt_ctas_ = (per_sm > 0 ? per_sm : 1) * nsm;
            ns3d_status st = build_xitems(xtma_tile<T, N, V>(), &xt_items_, &xt_nvalid_);
            if (st != NS3D_OK) return st;
        }
        set_xfwd_attrs<INT_IFRK4>();
        set_xfwd_attrs<INT_RK4CN>();
        NS3D_CK(cudaFuncSetAttribute(k_xfwd<T, N, INT_TAB, X_STAGE1, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     smem_x()));
        tables(0, 0, M_);
        NS3D_CK(cudaGetLastError());
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }

    // ---------------------------------------------------------------- passes
    static constexpr size_t smem_a() { return sizeof(cx<T>) * (size_t)N * TA; }
    static constexpr size_t smem_af() { return sizeof(cx<T>) * (size_t)N * TAF; }
    static constexpr size_t smem_x() { return sizeof(cx<T>) * (size_t)N * TXF; }   // forward x pass
    static constexpr size_t smem_xi() { return xinv_smem<T, N, V>(); }
    static constexpr size_t smem_z() {
        return sizeof(cx<T>) * (size_t)ZP * 3 * zpad<N>() + sizeof(T) * (size_t)ZP * 12 * N;
    }

    // the compact list of the x tiles of TT pencils whose first column lies inside the
    // circle ky^2 + kz0^2 <= KC^2, ky-major: entry ((ky + KC) << 8) | tile
    ns3d_status build_xitems(int TT, int** dev, int* count) {
        std::vector<int> v;
        const int ntx = (G::NZ1 + TT - 1) / TT;
        for (int ky = -G::KC; ky <= G::KC; ++ky)
            for (int tl = 0; tl < ntx; ++tl)
                if (ky * ky + tl * TT * tl * TT <= G::KC2) v.push_back(((ky + G::KC) << 8) | tl);
        NS3D_CK(cudaMalloc(dev, sizeof(int) * v.size()));
        NS3D_CK(cudaMemcpy(*dev, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice));
        *count = (int)v.size();
        return NS3D_OK;
    }

    template <int INTEG>
    void set_xfwd_attrs() {
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_STAGE1, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_STAGE2, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_STAGE3, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_STAGE4, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_RHS, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
        cudaFuncSetAttribute(k_xfwd<T, N, INTEG, X_PLAIN, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_x());
    }

    // each launcher covers members [m0, m0 + cnt); `in` points at member 0's arrays
    void p1(const cx<T>* in, int m0, int cnt) {
        if constexpr (xinv_tma_ok<T, N, V>()) {
            const int k = in == U_ ? 0 : (in == UT_ ? 1 : -1);
            if (k >= 0) {
                constexpr int XT = xtma_tile<T, N, V>();
                const long long items = (long long)xt_nvalid_ * cnt;
                const unsigned grid = (unsigned)(items < xt_ctas_ ? items : xt_ctas_);
                k_xinv_tma<T, N, V><<<grid, XT * PX::P, xinv_tma_smem<T, N, V>(), s_>>>(
                    xmap_[k], 3 * m0, wmap_, 6 * m0, tw_, sdm(m0), xt_items_, xt_nvalid_, cnt);
                return;
            }
        }
        k_xinv<T, N, V><<<dim3(NTX, G::NKY, cnt), TX * PX::P, smem_xi(), s_>>>(in + (size_t)m0 * 3 * G::FS, Wm(m0), tw_);
    }
    void p2(int m0, int cnt) {
        k_ypass<T, N, true, V><<<dim3(NTA, N, 6 * cnt), TA * PY::P, smem_a(), s_>>>(Wm(m0), tw_);
    }
    static constexpr size_t smem_zl() { return zline_smem<T, N>(); }
    void p3(int want_umax, int m0, int cnt) {
        if constexpr (zgemm_ok<T, N>()) {
            if (zform_ == 2) {
                using Z = ZGeo<N>;
                const long long tiles = (long long)N * N * cnt / 128;
                const unsigned grid = (unsigned)(tiles < zg_ctas_ ? tiles : zg_ctas_);
                float* P = zg_P_ + (size_t)m0 * 3 * N * N * N;
                k_zgemm_inv<N><<<grid, kZgThreads, Z::SMEM_INV, s_>>>(reinterpret_cast<const float*>(Wm(m0)), zg_b_,
                                                                      P, sdm(m0), want_umax, cnt);
                k_zgemm_fwd<N><<<grid, kZgThreads, Z::SMEM_FWD, s_>>>(P, zg_b_ + 2 * Z::BI / 16,
                                                                      reinterpret_cast<float*>(Wm(m0)), sdm(m0), cnt);
                return;
            }
        }
        if constexpr (zline_ok<T, N>()) {
            if (zform_ == 0) {
                // persistent: as many CTAs as fit on the device, never more than there are line groups
                const long long items = (long long)N * N / zline_gpw<N>() * cnt;
                constexpr int ng = zline_groups<N>();
                long long grid = (long long)zline_ctas_;
                if (grid * ng > items) grid = (items + ng - 1) / ng;
                k_zline<T, N><<<(unsigned)grid, ZLINE_WARPS * 32, smem_zl(), s_>>>(Wm(m0), tw_, sdm(m0), want_umax,
                                                                                   cnt);
                return;
            }
        }
        k_zpass<T, N, 0><<<dim3((unsigned)((long long)N * N / 2 / ZP), cnt), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m0), tw_, nullptr, sdm(m0), want_umax);
    }
    void set_zform(int z) override {
        const int zn = (zline_ok<T, N>() && z == 0) ? 0 : (zgemm_ok<T, N>() && z == 2) ? 2 : 1;
        if (zn != zform_ && graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        zform_ = zn;
    }
    int zform() const override { return zform_; }
    int variant() const override { return V; }
    void p4(int m0, int cnt) {
        k_ypass<T, N, false, V><<<dim3(NTAF, N, 3 * cnt), TAF * PYF::P, smem_af(), s_>>>(Wm(m0), tw_);
    }
    template <int INTEG, int MODE>
    void p5x(int m0, int cnt, cx<T>* out) {
        k_xfwd<T, N, INTEG, MODE, V><<<dim3(NTXF, G::NKY, cnt), TXF * PX::P, smem_x(), s_>>>(
            Wm(m0), Um(m0), UTm(m0), out ? out + (size_t)m0 * 3 * G::FS : ACCm(m0), tw_, sdm(m0), tabm(m0),
            (les_ && MODE <= X_STAGE4) ? F_ : nullptr, nullptr, nullptr, RkStage{});
    }
    // RK5-family stage epilogue s (0-based) of members [m0, m0 + cnt)
    void p5tab(int s, int m0, int cnt) {
        k_xfwd<T, N, INT_TAB, X_STAGE1, V><<<dim3(NTXF, G::NKY, cnt), TXF * PX::P, smem_x(), s_>>>(
            Wm(m0), Um(m0), UTm(m0), ACCm(m0), tw_, sdm(m0), tabm(m0), les_ ? F_ : nullptr,
            K_ + (size_t)m0 * 18 * G::FS, dpart_ + (size_t)m0 * 3 * NTXF * G::NKY, rk_stage(s, dp5()));
    }
    template <int MODE>
    void p5(int m0, int cnt, cx<T>* out = nullptr) {
        if (p_.integrator == INT_RK4CN) p5x<INT_RK4CN, MODE>(m0, cnt, out);
        else p5x<INT_IFRK4, MODE>(m0, cnt, out);
    }
    void tables(int use_cfl, int m0, int cnt) {
        const int n = G::KC2 + 1;
        k_tables<T, N><<<dim3((n + 255) / 256, cnt), 256, 0, s_>>>(tabm(m0), sdm(m0), p_.integrator, p_.visc_pow,
                                                                   use_cfl);
    }

    // -div(tau) of the learned closure for the state at the start of the step
    // (single run): real-space u, network, r2c of the six tau components,
    // divergence, energy-budget flag. The term is then held for the 4 stages.
    void launch_sgs() {
        p1(U_, 0, 1); p2(0, 1);
        k_zpass<T, N, 1><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            W_, tw_, real_, nullptr, 0);
        les_->forward(reinterpret_cast<const float*>(real_), reinterpret_cast<float*>(tau_real_), N, s_);
        const long long M3 = (long long)N * N * N;
        for (int h = 0; h < 2; ++h) {
            k_zpass<T, N, 2><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
                W_, tw_, tau_real_ + h * 3 * M3, nullptr, 0);
            p4(0, 1);
            k_xfwd<T, N, INT_IFRK4, X_PLAIN, V><<<dim3(NTXF, G::NKY, 1), TXF * PX::P, smem_x(), s_>>>(
                W_, U_, UT_, TAU_ + (size_t)h * 3 * G::FS, tw_, sd_, tab_, nullptr, nullptr, nullptr, RkStage{});
        }
        k_sgs_div<T, N><<<kSgsParts, 256, 0, s_>>>(TAU_, U_, F_, sgs_part_);
        k_sgs_flag<><<<1, 32, 0, s_>>>(sgs_part_, kSgsParts, sd_, les_->status_word());
    }
    static constexpr int kSgsParts = 512;

    // Dormand & Prince (1980) RK5(4)7M coefficients. The reference's table
    // (solver.c:34-42) holds the same numbers except a32, 1/2 there: the
    // published 9/40 is the value that satisfies a31 + a32 = c3 = 3/10.
    static RkStage rk_stage(int s, bool dp) {
        static const double A[7][6] = {
            {0, 0, 0, 0, 0, 0},
            {1.0 / 5.0, 0, 0, 0, 0, 0},
            {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
            {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
            {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
            {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
            {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
        static const double B[7] = {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0};
        static const double BS[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                                     187.0 / 2100.0, 1.0 / 40.0};
        RkStage r{};
        const int last = dp ? 6 : 5;
        r.nk = s;
        r.store = s < last ? s : -1;
        if (s < last) {
            r.kind = 0;
            for (int j = 0; j < s; ++j) r.c[j] = A[s + 1][j];
            r.c_cur = A[s + 1][s];
        } else {
            r.kind = dp ? 2 : 1;
            for (int j = 0; j < s; ++j) {
                r.c[j] = B[j];
                if (dp) r.e[j] = B[j] - BS[j];
            }
            r.c_cur = B[s];
            if (dp) r.e_cur = B[s] - BS[s];
        }
        return r;
    }

    // one RK5CN step or DP5CN attempt of every member: 6 or 7 nonlinear
    // evaluations, each ending in its tableau epilogue
    void launch_step_rk5() {
        const bool dp = dp5();
        const int cfl = (!dp && p_.cfl > 0) ? 1 : 0;
        const int M = M_;
        const int S = dp ? 7 : 6;
        if (les_) launch_sgs();
        if (dp) tables(0, 0, M);
        for (int s = 0; s < S; ++s) {
            p1(s == 0 ? U_ : UT_, 0, M); p2(0, M); p3(s == 0 ? cfl : 0, 0, M);
            if (s == 0 && cfl) tables(1, 0, M);
            p4(0, M);
            p5tab(s, 0, M);
        }
        if (dp) {
            k_dp_ctl<T, N><<<M, 256, 0, s_>>>(dpart_, NTXF * G::NKY, sd_);
            k_dp_commit<T, N><<<dim3(grid_for((long long)N * N * G::NZP), M), 256, 0, s_>>>(U_, ACC_, sd_);
        }
        k_step_end<T, N><<<M, 256, 0, s_>>>(U_, sd_, p_.forcing == 1 ? p_.force_k : 0, cfl, dp ? 1 : 0);
    }

    // one time step of every member = 4 nonlinear evaluations with fused stage epilogues
    void launch_step() {
        if (rk5()) {
            launch_step_rk5();
            return;
        }
        const int cfl = p_.cfl > 0 ? 1 : 0;
        const int M = M_;
        if (les_) launch_sgs();
        p1(U_, 0, M); p2(0, M); p3(cfl, 0, M);
        if (cfl) tables(1, 0, M);
        p4(0, M); p5<X_STAGE1>(0, M);
        p1(UT_, 0, M); p2(0, M); p3(0, 0, M); p4(0, M); p5<X_STAGE2>(0, M);
        p1(UT_, 0, M); p2(0, M); p3(0, 0, M); p4(0, M); p5<X_STAGE3>(0, M);
        p1(UT_, 0, M); p2(0, M); p3(0, 0, M); p4(0, M); p5<X_STAGE4>(0, M);
        k_step_end<T, N><<<M, 256, 0, s_>>>(U_, sd_, p_.forcing == 1 ? p_.force_k : 0, cfl, 0);
    }

    ns3d_status build_graph() {
        if (graph_exec_) return NS3D_OK;
        cudaGraph_t g = nullptr;
        NS3D_CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
        launch_step();
        cudaError_t e = cudaStreamEndCapture(s_, &g);
        if (e != cudaSuccess) {
            set_err("graph capture: %s", cudaGetErrorString(e));
            return NS3D_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&graph_exec_, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            set_err("graph instantiate: %s", cudaGetErrorString(e));
            graph_exec_ = nullptr;
            return NS3D_ERR_CUDA;
        }
        return NS3D_OK;
    }

    ns3d_status step(int nsteps) override {
        if (nsteps <= 0) return NS3D_OK;
        ns3d_status st = build_graph();
        if (st != NS3D_OK) return st;
        if (dp5()) return step_dp5(nsteps);
        NS3D_CK(cudaEventRecord(ev0_, s_));
        for (int k = 0; k < nsteps; ++k) NS3D_CK(cudaGraphLaunch(graph_exec_, s_));
        NS3D_CK(cudaEventRecord(ev1_, s_));
        return check_status();
    }
    // DP5CN (single run): one graph launch per attempt; launches continue
    // until nsteps attempts were accepted. k_dp_ctl ends the run with
    // kStatusDpFail after kDpMaxTry rejections in a row, so the loop ends.
    ns3d_status step_dp5(int nsteps) {
        ns3d_status st = check_status();
        if (st != NS3D_OK) return st;
        const long long start = sd_host_[0].iters;
        long long done = 0;
        NS3D_CK(cudaEventRecord(ev0_, s_));
        while (done < nsteps) {
            for (long long k = done; k < nsteps; ++k) NS3D_CK(cudaGraphLaunch(graph_exec_, s_));
            NS3D_CK(cudaEventRecord(ev1_, s_));
            st = check_status();
            if (st != NS3D_OK) return st;
            done = sd_host_[0].iters - start;
        }
        return NS3D_OK;
    }

    ns3d_status check_status() {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sd_, sizeof(StepDev) * M_, cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        NS3D_CK(cudaGetLastError());
        for (int m = 0; m < M_; ++m) {
            if (sd_host_[m].status == kStatusTimeout) {
                set_err("member %d: a bounded wait for an asynchronous copy gave up at step %lld", m, sd_host_[m].iters);
                return NS3D_ERR_TIMEOUT;
            }
            if (sd_host_[m].status == kStatusDpFail) {
                set_err("member %d: DP5CN step rejected %d times in a row at step %lld (error norm %g, dt %g)", m,
                        kDpMaxTry, sd_host_[m].iters, sd_host_[m].dp_err, sd_host_[m].dt);
                return NS3D_ERR_NUMERIC;
            }
            if (sd_host_[m].status != 0) {
                set_err("member %d: numeric health check failed at step %lld (NaN/Inf energy or speed)", m,
                        sd_host_[m].iters);
                return NS3D_ERR_NUMERIC;
            }
        }
        return NS3D_OK;
    }

    ns3d_status last_step_ms(float* ms) override {
        NS3D_CK(cudaEventElapsedTime(ms, ev0_, ev1_));
        return NS3D_OK;
    }

    // per-kernel-class timing of `reps` steps launched one kernel at a time
    ns3d_status profile(int reps, const char** names, float* ms, double* bytes, int maxc, int* count) override {
        if (rk5()) {
            set_err("per-kernel profile covers the RK4-family step");
            return NS3D_ERR_UNSUPPORTED;
        }
        const char* kNames[6] = {"k_xinv", "k_ypass_inv",
                                 zform_ == 0 ? "k_zline" : zform_ == 2 ? "k_zgemm" : "k_zpass", "k_ypass_fwd",
                                 "k_xfwd", "k_misc"};
        std::vector<cudaEvent_t> ev(2 * 6 * 4 + 2);
        for (auto& e : ev) NS3D_CK(cudaEventCreate(&e));
        double acc[6] = {0, 0, 0, 0, 0, 0};
        const int cfl = p_.cfl > 0 ? 1 : 0;
        for (int r = 0; r < reps; ++r) {
            int q = 0;
            for (int s = 0; s < 4; ++s) {
                const cx<T>* in = s == 0 ? U_ : UT_;
                const int M = M_;
                NS3D_CK(cudaEventRecord(ev[q++], s_)); p1(in, 0, M);
                NS3D_CK(cudaEventRecord(ev[q++], s_)); p2(0, M);
                NS3D_CK(cudaEventRecord(ev[q++], s_)); p3(s == 0 ? cfl : 0, 0, M);
                if (s == 0 && cfl) tables(1, 0, M);
                NS3D_CK(cudaEventRecord(ev[q++], s_)); p4(0, M);
                NS3D_CK(cudaEventRecord(ev[q++], s_));
                if (s == 0) p5<X_STAGE1>(0, M); else if (s == 1) p5<X_STAGE2>(0, M);
                else if (s == 2) p5<X_STAGE3>(0, M); else p5<X_STAGE4>(0, M);
                NS3D_CK(cudaEventRecord(ev[q++], s_));
            }
            k_step_end<T, N><<<M_, 256, 0, s_>>>(U_, sd_, p_.forcing == 1 ? p_.force_k : 0, cfl, 0);
            NS3D_CK(cudaEventRecord(ev[q++], s_));
            NS3D_CK(cudaStreamSynchronize(s_));
            q = 0;
            for (int s = 0; s < 4; ++s) {
                for (int k = 0; k < 5; ++k) {
                    float t = 0;
                    NS3D_CK(cudaEventElapsedTime(&t, ev[q + k], ev[q + k + 1]));
                    acc[k] += t;
                }
                q += 6;
            }
            float t = 0;
            NS3D_CK(cudaEventElapsedTime(&t, ev[q - 1], ev[q]));
            acc[5] += t;
        }
        for (auto& e : ev) cudaEventDestroy(e);
        // compulsory bytes per launch (loads of non-zero inputs + stores of needed outputs)
        const double w = (double)sizeof(cx<T>);
        const double sph = sphere_modes(), circ = circle_cols(), full = (double)N * N * G::NZ1;
        const double b[6] = {
            w * (3 * sph + 6 * circ),               // P1: u_hat in, 6 fields on the (x, ky^2+kz^2<=KC^2) set
            w * (6 * circ + 6 * full),              // P2
            w * (6 * full + 3 * full),              // P3
            w * (3 * full + 3 * circ),              // P4
            w * (3 * circ + 9.75 * sph),            // P5: 3 fields in + state (mean over the 4 stages)
            0.0};
        int n = 0;
        for (int k = 0; k < 6 && n < maxc; ++k, ++n) {
            names[n] = kNames[k];
            ms[n] = (float)(acc[k] / reps / (k == 5 ? 1 : 4));
            if (bytes) bytes[n] = b[k];
        }
        *count = n;
        return check_status();
    }
    double sphere_modes() const {   // modes with kz >= 0 inside the sphere
        double c = 0;
        for (int kx = -G::KC; kx <= G::KC; ++kx)
            for (int ky = -G::KC; ky <= G::KC; ++ky) {
                const int r = G::KC2 - kx * kx - ky * ky;
                if (r >= 0) c += std::floor(std::sqrt((double)r) + 1e-9) + 1;
            }
        return c;
    }
    double circle_cols() const {   // (x, ky, kz) with ky^2 + kz^2 <= KC^2
        double c = 0;
        for (int ky = -G::KC; ky <= G::KC; ++ky) c += std::floor(std::sqrt((double)(G::KC2 - ky * ky)) + 1e-9) + 1;
        return c * N;
    }

    // --------------------------------------------------------------- rhs
    ns3d_status rhs_host(const double* in, double* out) override {
        ns3d_status st = upload(in, UTm(m_));
        if (st != NS3D_OK) return st;
        p1(UT_, m_, 1); p2(m_, 1); p3(0, m_, 1); p4(m_, 1); p5<X_RHS>(m_, 1, ACC_);
        return download(ACCm(m_), out);
    }

    // ----------------------------------------------------- state transfer
    ns3d_status ensure_stage() {
        if (!stage_) NS3D_CK(cudaMalloc(&stage_, sizeof(double2) * 3 * (size_t)N * N * (N / 2 + 1)));
        return NS3D_OK;
    }
    static constexpr long long kRefBytes = 48LL * N * N * (N / 2 + 1);   // reference Fourier array
    // device address of a page-locked host array (16-byte aligned), else nullptr
    static const void* host_dev_ptr(const void* h) {
        cudaPointerAttributes a, z;
        const unsigned char* last = static_cast<const unsigned char*>(h) + kRefBytes - 1;
        if (cudaPointerGetAttributes(&a, h) != cudaSuccess || cudaPointerGetAttributes(&z, last) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        // the whole array must lie in one page-locked allocation mapped for the device
        if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer || !z.devicePointer ||
            static_cast<const unsigned char*>(z.devicePointer) - static_cast<const unsigned char*>(a.devicePointer) !=
                kRefBytes - 1 ||
            (reinterpret_cast<uintptr_t>(h) & 15))
            return nullptr;
        return a.devicePointer;
    }
    ns3d_status upload(const double* host, cx<T>* dst) {
        if (const void* d = host_dev_ptr(host)) {
            // one warp per row's lines reads the dealiased modes straight from the host
            // array in 512-byte requests; modes outside the sphere are zero in `dst`
            // (cleared at creation, and no kernel writes them) and stay unwritten
            ns3d_status st = line_plan(plan_in_, (int)(reinterpret_cast<uintptr_t>(host) & 127));
            if (st != NS3D_OK) return st;
            k_pack_lines<T, N><<<(unsigned)((plan_in_.nr * 32LL + 255) / 256), 256, 0, s_>>>(
                static_cast<const double2*>(d), dst, plan_in_.ranges, plan_in_.nr);
            NS3D_CK(cudaGetLastError());
            io_h2d_ = plan_in_.gpu_bytes;
            return NS3D_OK;
        }
        ns3d_status st = ensure_stage();
        if (st != NS3D_OK) return st;
        NS3D_CK(cudaMemcpyAsync(stage_, host, kRefBytes, cudaMemcpyHostToDevice, s_));
        k_pack<T, N><<<grid_for((long long)N * N * G::NZP), 256, 0, s_>>>(stage_, dst);
        NS3D_CK(cudaGetLastError());
        io_h2d_ = kRefBytes;
        return NS3D_OK;
    }
    ns3d_status download(const cx<T>* src, double* host) {
        if (const void* d = host_dev_ptr(host)) {
            ns3d_status st = line_plan(plan_out_, (int)(reinterpret_cast<uintptr_t>(host) & 127));
            if (st != NS3D_OK) return st;
            k_unpack_lines<T, N><<<(unsigned)((plan_out_.nr * 32LL + 255) / 256), 256, 0, s_>>>(
                src, static_cast<double2*>(const_cast<void*>(d)), plan_out_.ranges, plan_out_.nr);
            NS3D_CK(cudaGetLastError());
            zero_host_lines(reinterpret_cast<unsigned char*>(host));   // host threads, during the GPU work
            NS3D_CK(cudaStreamSynchronize(s_));
            NS3D_CK(cudaGetLastError());
            io_d2h_ = plan_out_.gpu_bytes;
            return NS3D_OK;
        }
        ns3d_status st = ensure_stage();
        if (st != NS3D_OK) return st;
        k_unpack<T, N><<<grid_for((long long)N * N * (N / 2 + 1)), 256, 0, s_>>>(src, stage_);
        NS3D_CK(cudaMemcpyAsync(host, stage_, kRefBytes, cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        NS3D_CK(cudaGetLastError());
        io_d2h_ = kRefBytes;
        return NS3D_OK;
    }
    static long long isqrt(long long v) {
        long long r = (long long)std::sqrt((double)v);
        while (r * r > v) --r;
        while ((r + 1) * (r + 1) <= v) ++r;
        return r;
    }
    // Split of the reference Fourier array between the GPU and host threads for
    // a host array whose address is `align` mod 128: for every (kx, ky) row
    // with dealiased modes the GPU writes the 128-byte lines that hold them
    // (zeros included where a line extends past them); host threads zero all
    // other bytes. The two sets of lines are disjoint.
    struct LinePlan {
        int align = -1, nr = 0;
        long long gpu_bytes = 0;
        longlong2* ranges = nullptr;                           // [ls, le) in 16-byte units, device
        std::vector<std::pair<long long, long long>> cpu;      // host-owned byte segments
    };
    ns3d_status line_plan(LinePlan& pl, int align) {
        if (pl.align == align) return NS3D_OK;
        constexpr int NF = N / 2 + 1;
        constexpr long long RB = 48LL * NF;
        std::vector<longlong2> ranges;
        pl.cpu.clear();
        long long cursor = 0, gpu = 0;
        for (long long r = 0; r < (long long)N * N; ++r) {
            const int i = (int)(r / N), j = (int)(r % N);
            const int kx = i <= N / 2 ? i : i - N, ky = j <= N / 2 ? j : j - N;
            const long long rem = (long long)G::KC2 - kx * kx - ky * ky;
            if (rem < 0) continue;
            const long long bs = r * RB, be = bs + 48 * (isqrt(rem) + 1);
            long long ls = (align + bs) / 128 * 128 - align, le = (align + be + 127) / 128 * 128 - align;
            if (ls < cursor) ls = cursor;
            if (le > kRefBytes) le = kRefBytes;
            if (ls >= le) continue;
            if (cursor < ls) pl.cpu.push_back({cursor, ls - cursor});
            ranges.push_back(make_longlong2(ls / 16, le / 16));
            gpu += le - ls;
            cursor = le;
        }
        if (cursor < kRefBytes) pl.cpu.push_back({cursor, kRefBytes - cursor});
        if (pl.ranges) cudaFree(pl.ranges);
        pl.ranges = nullptr;
        pl.align = -1;
        NS3D_CK(cudaMalloc(&pl.ranges, sizeof(longlong2) * ranges.size()));
        NS3D_CK(cudaMemcpy(pl.ranges, ranges.data(), sizeof(longlong2) * ranges.size(), cudaMemcpyHostToDevice));
        pl.nr = (int)ranges.size();
        pl.gpu_bytes = gpu;
        pl.align = align;
        return NS3D_OK;
    }
    // zero the host-owned bytes with up to 16 threads, split evenly by bytes
    void zero_host_lines(unsigned char* host) const {
        long long total = 0;
        for (const auto& seg : plan_out_.cpu) total += seg.second;
        unsigned nt = std::thread::hardware_concurrency();
        nt = nt < 1 ? 1 : (nt > 16 ? 16 : nt);
        if (total < (1LL << 22)) nt = 1;
        auto work = [&](long long lo, long long hi) {
            long long pos = 0;
            for (const auto& seg : plan_out_.cpu) {
                const long long a = pos > lo ? pos : lo, b = pos + seg.second < hi ? pos + seg.second : hi;
                if (a < b) memset(host + seg.first + (a - pos), 0, (size_t)(b - a));
                pos += seg.second;
                if (pos >= hi) break;
            }
        };
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nt; ++t) th.emplace_back(work, total * t / nt, total * (t + 1) / nt);
        work(0, total / nt);
        for (auto& x : th) x.join();
    }
    static unsigned grid_for(long long n) {
        long long g = (n + 255) / 256;
        if (g > 152 * 32) g = 152 * 32;
        return (unsigned)(g < 1 ? 1 : g);
    }

    ns3d_status set_state_host(const double* u) override {
        ns3d_status st = upload(u, Um(m_));
        if (st != NS3D_OK) return st;
        return reset_forcing_target();
    }
    ns3d_status get_state_host(double* u) override { return download(Um(m_), u); }

    ns3d_status step_host(const double* in, double* out) override {
        ns3d_status st;
        if (M_ != 1) return NS3D_ERR_INVALID;
        if (in && (st = upload(in, U_)) != NS3D_OK) return st;
        if ((st = build_graph()) != NS3D_OK) return st;
        NS3D_CK(cudaGraphLaunch(graph_exec_, s_));
        if (out) {
            if ((st = download(U_, out)) != NS3D_OK) return st;
        }
        return check_status();
    }

    // -------------------------------------------------------- diagnostics
    ns3d_status measure_dev(const cx<T>* u) {
        k_measure<T, N><<<(unsigned)NMEAS, MEAS_WARPS * 32, 0, s_>>>(u, mp_[m_].nu, p_.visc_pow, part_);
        const double N3 = (double)N * N * N;
        k_measure_reduce<<<(MWIDTH + 127) / 128, 128, 0, s_>>>(part_, (int)NMEAS, MWIDTH, G::NSP, N3 * N3, mout_);
        NS3D_CK(cudaMemcpyAsync(mout_host_, mout_, sizeof(double) * MWIDTH, cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        NS3D_CK(cudaGetLastError());
        return NS3D_OK;
    }
    ns3d_status measurables(ns3d_measures* m, double* Ek, double* Ok) override {
        ns3d_status st = measure_dev(Um(m_));
        if (st != NS3D_OK) return st;
        if (m) {
            m->energy = mout_host_[0];
            m->enstrophy = mout_host_[1];
            m->palinstrophy = mout_host_[2];
            m->helicity = mout_host_[3];
            m->dissipation = mout_host_[4];
        }
        const int ns = n_spect();
        for (int b = 0; b < ns; ++b) {
            if (Ek) Ek[b] = b < G::NSP ? mout_host_[5 + b] : 0.0;
            if (Ok) Ok[b] = b < G::NSP ? mout_host_[5 + G::NSP + b] : 0.0;
        }
        return NS3D_OK;
    }
    int n_spect() const { return (int)std::sqrt(3.0 * ((double)N / 2.0) * ((double)N / 2.0)) + 1; }

    // ------------------------------------------------- initial conditions
    ns3d_status ensure_real() {
        if (!real_) NS3D_CK(cudaMalloc(&real_, sizeof(T) * 6 * (size_t)N * N * N));
        return NS3D_OK;
    }
    ns3d_status ic_real(int kind) override {
        ns3d_status st = ensure_real();
        if (st != NS3D_OK) return st;
        k_fill_real<T, N><<<grid_for((long long)N * N * N), 256, 0, s_>>>(real_, kind);
        k_zpass<T, N, 2><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m_), tw_, real_, nullptr, 0);
        p4(m_, 1);
        p5<X_PLAIN>(m_, 1, U_);
        NS3D_CK(cudaGetLastError());
        return finish_ic();
    }
    ns3d_status ic_spectrum(uint64_t seed, double k0, double energy) override {
        unsigned long long key = host_splitmix64(seed);
        k_spectrum_ic<T, N><<<grid_for((long long)N * N * G::NZP), 256, 0, s_>>>(Um(m_), key, k0);
        ns3d_status st = measure_dev(Um(m_));
        if (st != NS3D_OK) return st;
        const double e = mout_host_[0];
        const double target = 8.0 * M_PI * M_PI * M_PI * energy;
        if (e > 0.0) k_scale<T, N><<<grid_for(3 * G::FS), 256, 0, s_>>>(Um(m_), std::sqrt(target / e));
        NS3D_CK(cudaGetLastError());
        return finish_ic();
    }
    ns3d_status ic_host(const double* u) override {
        ns3d_status st = upload(u, Um(m_));
        if (st != NS3D_OK) return st;
        return finish_ic();
    }
    ns3d_status ic_zero() override {
        NS3D_CK(cudaMemsetAsync(Um(m_), 0, sizeof(cx<T>) * 3 * (size_t)G::FS, s_));
        return finish_ic();
    }
    ns3d_status finish_ic() {
        ns3d_status st = set_time(mp_[m_].t0, mp_[m_].dt, 0);
        if (st != NS3D_OK) return st;
        return reset_forcing_target();
    }
    ns3d_status reset_forcing_target() {
        if (p_.forcing != 1) return NS3D_OK;
        double e = 0;
        ns3d_status st = shell_energy(&e);
        if (st != NS3D_OK) return st;
        return set_forcing_target(e);
    }
    // energy of shells 1 <= round(|k|) <= force_k, FP64, from the spectrum
    ns3d_status shell_energy(double* e) {
        ns3d_status st = measure_dev(Um(m_));
        if (st != NS3D_OK) return st;
        double s = 0;
        for (int b = 1; b <= p_.force_k && b < G::NSP; ++b) s += mout_host_[5 + b];
        *e = s;
        return NS3D_OK;
    }

    // ------------------------------------------------------- real space
    ns3d_status real_space_host(double* u, double* w) override {
        ns3d_status st = ensure_real();
        if (st != NS3D_OK) return st;
        double* du = nullptr;
        size_t rb = sizeof(double) * 3 * (size_t)N * N * (N + 2);
        NS3D_CK(cudaMalloc(&du, 2 * rb));
        p1(U_, m_, 1); p2(m_, 1);
        k_zpass<T, N, 1><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m_), tw_, real_, nullptr, 0);
        k_real_unpack<T, N><<<grid_for((long long)N * N * (N + 2)), 256, 0, s_>>>(real_, du, du + rb / sizeof(double));
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && u) e = cudaMemcpyAsync(u, du, rb, cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess && w) e = cudaMemcpyAsync(w, du + rb / sizeof(double), rb, cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
        cudaFree(du);
        if (e != cudaSuccess) {
            set_err("real_space: %s", cudaGetErrorString(e));
            return NS3D_ERR_CUDA;
        }
        return NS3D_OK;
    }

    ns3d_status max_speed_sum(double* umax) override {
        NS3D_CK(cudaMemsetAsync(&sdm(m_)->umax_bits, 0, sizeof(unsigned long long), s_));
        p1(U_, m_, 1); p2(m_, 1); p3(1, m_, 1);
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        const unsigned long long b = sd_host_->umax_bits;
        if (sizeof(T) == 4) {
            unsigned u32 = (unsigned)b;
            float f;
            std::memcpy(&f, &u32, 4);
            *umax = f;
        } else {
            double d;
            std::memcpy(&d, &b, 8);
            *umax = d;
        }
        NS3D_CK(cudaMemsetAsync(&sdm(m_)->umax_bits, 0, sizeof(unsigned long long), s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }

    // ------------------------------------------------------ bookkeeping
    ns3d_status refresh_tables() {
        tables(0, m_, 1);
        NS3D_CK(cudaGetLastError());
        return NS3D_OK;
    }
    ns3d_status get_time(double* t, double* dt, long* iters) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        if (t) *t = sd_host_->t;
        if (dt) *dt = sd_host_->dt;
        if (iters) *iters = (long)sd_host_->iters;
        return NS3D_OK;
    }
    ns3d_status set_time(double t, double dt, long iters) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        sd_host_->t = t;
        sd_host_->dt = dt;
        sd_host_->iters = iters;
        sd_host_->t0 = t - (p_.cfl > 0 ? 0.0 : (double)iters * dt);
        sd_host_->umax_bits = 0;
        sd_host_->status = 0;
        NS3D_CK(cudaMemcpyAsync(sdm(m_), sd_host_, sizeof(StepDev), cudaMemcpyHostToDevice, s_));
        ns3d_status st = refresh_tables();
        if (st != NS3D_OK) return st;
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }
    // longitudinal velocity-increment statistics of the current state (stats.cuh)
    ns3d_status increment_stats(const int* incr, int nr, int nbins, double* stats, double* ranges,
                                double* counts) override {
        ns3d_status st = ensure_real();
        if (st != NS3D_OK) return st;
        p1(U_, m_, 1); p2(m_, 1);
        k_zpass<T, N, 1><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m_), tw_, real_, nullptr, 0);
        double *part = nullptr, *red = nullptr;
        unsigned long long* cnt = nullptr;
        cudaError_t e = cudaMalloc(&part, sizeof(double) * (kIncrParts * 4 + 8));
        if (e == cudaSuccess) e = cudaMalloc(&cnt, sizeof(unsigned long long) * nbins);
        red = part + kIncrParts * 4;   // [0..3] reduced values, [4] mean, [5..6] lo, hi
        std::vector<unsigned long long> hc(nbins);
        double h[8];
        for (int r = 0; r < nr && e == cudaSuccess; ++r) {
            const int dr = incr[r];
            k_incr_moments<T, N><<<kIncrParts, kIncrThreads, 0, s_>>>(real_, dr, 0, nullptr, part);
            k_incr_reduce<><<<1, 32, 0, s_>>>(part, kIncrParts, 0, red);
            e = cudaMemcpyAsync(h, red, sizeof(double) * 4, cudaMemcpyDeviceToHost, s_);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
            if (e != cudaSuccess) break;
            const double n = h[0], mn = n > 0 ? h[2] : 0.0, mx = n > 0 ? h[3] : 0.0, mean = n > 0 ? h[1] / n : 0.0;
            double m2 = 0, m3 = 0, m4 = 0;
            const double lo = mn - 0.05, hi = mx + 0.05;
            for (int b = 0; b < nbins; ++b) hc[b] = 0;
            if (n > 0) {
                const double lh[3] = {mean, lo, hi};
                e = cudaMemcpyAsync(red + 4, lh, sizeof(double) * 3, cudaMemcpyHostToDevice, s_);
                if (e != cudaSuccess) break;
                k_incr_moments<T, N><<<kIncrParts, kIncrThreads, 0, s_>>>(real_, dr, 1, red + 4, part);
                k_incr_reduce<><<<1, 32, 0, s_>>>(part, kIncrParts, 1, red);
                e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * nbins, s_);
                if (e != cudaSuccess) break;
                k_incr_hist<T, N><<<kIncrParts, kIncrThreads, sizeof(unsigned) * nbins, s_>>>(real_, dr, red + 5, nbins,
                                                                                              cnt);
                e = cudaMemcpyAsync(h, red, sizeof(double) * 4, cudaMemcpyDeviceToHost, s_);
                if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cnt, sizeof(unsigned long long) * nbins,
                                                          cudaMemcpyDeviceToHost, s_);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
                if (e != cudaSuccess) break;
                m2 = h[0]; m3 = h[1]; m4 = h[2];
            }
            // GSL rstat definitions: sample sd (n - 1), skew = m3 / sd^3, excess kurtosis m4 / sd^4 - 3
            const double var = n > 1 ? m2 / (n - 1) : 0.0;
            double* sr = stats + 6 * r;
            sr[0] = mn; sr[1] = mx; sr[2] = mean; sr[3] = sqrt(var);
            sr[4] = var > 0 ? (m3 / n) / pow(var, 1.5) : 0.0;
            sr[5] = var > 0 ? (m4 / n) / (var * var) - 3.0 : 0.0;
            if (ranges)
                for (int b = 0; b <= nbins; ++b) ranges[(long long)r * (nbins + 1) + b] = incr_edge(lo, hi, b, nbins);
            if (counts)
                for (int b = 0; b < nbins; ++b) counts[(long long)r * nbins + b] = (double)hc[b];
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        if (part) cudaFree(part);
        if (cnt) cudaFree(cnt);
        if (e != cudaSuccess) {
            set_err("increment statistics: %s", cudaGetErrorString(e));
            return NS3D_ERR_CUDA;
        }
        return NS3D_OK;
    }
    ns3d_status io_bytes(long long* h2d, long long* d2h) override {
        if (h2d) *h2d = io_h2d_;
        if (d2h) *d2h = io_d2h_;
        return NS3D_OK;
    }
    ns3d_status set_dp_tolerances(double atol, double rtol) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sd_, sizeof(StepDev) * M_, cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        for (int m = 0; m < M_; ++m) {
            sd_host_[m].dp_atol = atol;
            sd_host_[m].dp_rtol = rtol;
        }
        NS3D_CK(cudaMemcpyAsync(sd_, sd_host_, sizeof(StepDev) * M_, cudaMemcpyHostToDevice, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }
    ns3d_status set_wait_budget(long long cycles) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sd_, sizeof(StepDev) * M_, cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        for (int m = 0; m < M_; ++m) sd_host_[m].wait_cycles = cycles > 0 ? cycles : kWaitCycles;
        NS3D_CK(cudaMemcpyAsync(sd_, sd_host_, sizeof(StepDev) * M_, cudaMemcpyHostToDevice, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }
    ns3d_status dp_stats(double* err, long* rejects) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        if (err) *err = sd_host_->dp_err;
        if (rejects) *rejects = (long)sd_host_->dp_rejects;
        return NS3D_OK;
    }
    ns3d_status get_forcing_target(double* e) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        *e = sd_host_->force_target;
        return NS3D_OK;
    }
    ns3d_status set_forcing_target(double e) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        sd_host_->force_target = e;
        NS3D_CK(cudaMemcpyAsync(sdm(m_), sd_host_, sizeof(StepDev), cudaMemcpyHostToDevice, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        return NS3D_OK;
    }

    // device pointers for in-library tools
    void* state_ptr() override { return Um(m_); }

    // ----------------------------------------------- learned closure hooks
    ns3d_status attach_les(LesHook* h) override {
        if (sizeof(T) != 4 || M_ != 1) {
            set_err("the learned closure needs a single FP32 run");
            return NS3D_ERR_INVALID;
        }
        if (h) {
            ns3d_status st = ensure_real();
            if (st != NS3D_OK) return st;
            const size_t fb = sizeof(cx<T>) * (size_t)G::FS;
            if (!TAU_) NS3D_CK(cudaMalloc(&TAU_, 6 * fb));
            if (!F_) NS3D_CK(cudaMalloc(&F_, 3 * fb));
            if (!tau_real_) NS3D_CK(cudaMalloc(&tau_real_, sizeof(T) * 6 * (size_t)N * N * N));
            if (!sgs_part_) NS3D_CK(cudaMalloc(&sgs_part_, sizeof(double) * kSgsParts));
        }
        les_ = h;
        if (graph_exec_) {   // the step graph changes
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        return NS3D_OK;
    }
    ns3d_status les_counters(long* on, long* off) override {
        NS3D_CK(cudaMemcpyAsync(sd_host_, sdm(m_), sizeof(StepDev), cudaMemcpyDeviceToHost, s_));
        NS3D_CK(cudaStreamSynchronize(s_));
        if (on) *on = (long)sd_host_->sgs_steps;
        if (off) *off = (long)sd_host_->sgs_fallbacks;
        return NS3D_OK;
    }
    // real-space velocity of the selected member as [3][N^3] device floats
    const float* real_velocity_f32(ns3d_status* st) override {
        if (sizeof(T) != 4) {
            set_err("real-space velocity export needs an FP32 run");
            *st = NS3D_ERR_INVALID;
            return nullptr;
        }
        *st = ensure_real();
        if (*st != NS3D_OK) return nullptr;
        p1(U_, m_, 1); p2(m_, 1);
        k_zpass<T, N, 1><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m_), tw_, real_, nullptr, 0);
        *st = cudaGetLastError() == cudaSuccess ? NS3D_OK : NS3D_ERR_CUDA;
        return reinterpret_cast<const float*>(real_);
    }
    // r2c + dealias of a host velocity in the reference real layout
    ns3d_status set_state_real_host(const double* u) override {
        ns3d_status st = ensure_real();
        if (st == NS3D_OK) st = ensure_stage();
        if (st != NS3D_OK) return st;
        NS3D_CK(cudaMemcpyAsync(stage_, u, sizeof(double) * 3 * (size_t)N * N * (N + 2), cudaMemcpyHostToDevice, s_));
        k_real_pack<T, N><<<grid_for((long long)N * N * N), 256, 0, s_>>>(reinterpret_cast<const double*>(stage_),
                                                                         real_);
        k_zpass<T, N, 2><<<(unsigned)((long long)N * N / 2 / ZP), 3 * PA::P * ZP, smem_z(), s_>>>(
            Wm(m_), tw_, real_, nullptr, 0);
        p4(m_, 1);
        p5<X_PLAIN>(m_, 1, U_);
        NS3D_CK(cudaGetLastError());
        return reset_forcing_target();
    }

  private:
    cx<T>* U_ = nullptr;
    cx<T>* UT_ = nullptr;
    cx<T>* ACC_ = nullptr;
    cx<T>* W_ = nullptr;
    cx<T>* tw_ = nullptr;
    cx<T>* tab_ = nullptr;
    double* part_ = nullptr;
    double* mout_ = nullptr;
    double* mout_host_ = nullptr;
    double2* stage_ = nullptr;
    T* real_ = nullptr;
    StepDev* sd_ = nullptr;
    StepDev* sd_host_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    int zline_ctas_ = 1;
    int zform_ = zline_ok<T, N>() ? 0 : 1;
    LesHook* les_ = nullptr;       // learned closure (single FP32 run)
    cx<T>* TAU_ = nullptr;         // tau_ij spectra (6 fields)
    cx<T>* F_ = nullptr;           // -div(tau) (3 fields)
    T* tau_real_ = nullptr;        // tau_ij in real space [6][N^3]
    uint4* zg_b_ = nullptr;        // z-pass form 2: DFT matrices (Binv hi, lo, Bfwd hi, lo)
    float* zg_P_ = nullptr;        // z-pass form 2: the three real-space products [member][3][N^3]
    int zg_ctas_ = 0;
    CUtensorMap xmap_[2];          // P1 tensor-tile form: U and UT as [3 M][N kx][N ky][2 NZP] FP32
    CUtensorMap wmap_;             // and W as [6 M][N x][N ky][2 NZP] FP32 (its outputs)
    int xt_ctas_ = 1;
    int* xt_items_ = nullptr;      // P1 tensor-tile form: compact list of the x tiles inside the circle
    int xt_nvalid_ = 0;
    double* sgs_part_ = nullptr;
    cx<T>* K_ = nullptr;           // RK5 family: stored stages [member][6][3]
    double* dpart_ = nullptr;      // DP5CN error partial sums [member][block][3]
    // host-array transfers
    long long io_h2d_ = 0, io_d2h_ = 0;
    LinePlan plan_out_, plan_in_;   // host-array line plans of the download / upload
    int M_ = 1;                    // members
    int m_ = 0;                    // selected member
    std::vector<ns3d_params> mp_;  // per-member parameters
};

}  // namespace ns3d
