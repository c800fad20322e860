// fft_engine.cuh — register-resident mixed-radix Stockham FFT for sm_103a.
//
// One length-N complex transform is spread over P = N/E threads; thread p
// holds the E elements x[p + P*s], s < E, in registers. Each radix-R stage
// does E/R butterflies per thread in registers; between stages the elements
// are exchanged through shared memory (one write, one read per element).
// The first stage's inputs come straight from global memory and the last
// stage's outputs stay in registers in natural order (thread p holds
// X[p + P*s]), so a kernel loads, transforms and stores with coalesced
// accesses and only (stages - 1) shared-memory round trips.
//
// The index scheme is the Stockham autosort formulation used for GPU FFTs by
// Govindaraju et al. (SC 2008): butterfly j of a stage with current sub-size
// Ns reads x[j + r*N/R], twiddles by W_{Ns*R}^{r*(j mod Ns)} and writes
// y[(j/Ns)*Ns*R + (j mod Ns) + r*Ns].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns3d {

template <typename T>
struct __align__(2 * sizeof(T)) cx {
    T x, y;
};

template <typename T> __device__ __forceinline__ cx<T> mk(T a, T b) { cx<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> operator*(cx<T> a, T s) { return mk(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ cx<T> conjg(cx<T> a) { return mk(a.x, -a.y); }
template <typename T> __device__ __forceinline__ cx<T> mul_i(cx<T> a) { return mk(-a.y, a.x); }   // i*a
template <typename T> __device__ __forceinline__ cx<T> mul_mi(cx<T> a) { return mk(a.y, -a.x); }  // -i*a
template <typename T> __device__ __forceinline__ cx<T> czero() { return mk<T>(T(0), T(0)); }

// read-only-path loads of a complex value
__device__ __forceinline__ cx<float> ldg(const cx<float>* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return mk(v.x, v.y);
}
__device__ __forceinline__ cx<double> ldg(const cx<double>* p) {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    return mk(v.x, v.y);
}

// cos/sin of 2*pi*k/16 and 2*pi*k/12 (k < 16 / 12), the internal constants of
// the radix-2..16 codelets.
__device__ constexpr double kC16[16] = {
    1.0, 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173,
    0.0, -0.38268343236508977173, -0.70710678118654752440, -0.92387953251128675613,
    -1.0, -0.92387953251128675613, -0.70710678118654752440, -0.38268343236508977173,
    0.0, 0.38268343236508977173, 0.70710678118654752440, 0.92387953251128675613};
__device__ constexpr double kS16[16] = {
    0.0, 0.38268343236508977173, 0.70710678118654752440, 0.92387953251128675613,
    1.0, 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173,
    0.0, -0.38268343236508977173, -0.70710678118654752440, -0.92387953251128675613,
    -1.0, -0.92387953251128675613, -0.70710678118654752440, -0.38268343236508977173};
__device__ constexpr double kC12[12] = {
    1.0, 0.86602540378443864676, 0.5, 0.0, -0.5, -0.86602540378443864676,
    -1.0, -0.86602540378443864676, -0.5, 0.0, 0.5, 0.86602540378443864676};
__device__ constexpr double kS12[12] = {
    0.0, 0.5, 0.86602540378443864676, 1.0, 0.86602540378443864676, 0.5,
    0.0, -0.5, -0.86602540378443864676, -1.0, -0.86602540378443864676, -0.5};

__device__ __forceinline__ float fmat(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmat(double a, double b, double c) { return fma(a, b, c); }

// Element-wise complex add, subtract and broadcast FMA (c a.x + b.x, c a.y + b.y).
// With PK and FP32 the real and imaginary parts go through one FP32x2
// instruction (sm_100 and later; each lane rounds like the scalar instruction,
// so results are unchanged). Kernels choose PK per plan: it saves issue slots
// in the issue-bound z lines and the y passes, and costs registers elsewhere.
template <bool PK, typename T> __device__ __forceinline__ cx<T> vadd(cx<T> a, cx<T> b) { return a + b; }
template <bool PK, typename T> __device__ __forceinline__ cx<T> vsub(cx<T> a, cx<T> b) { return a - b; }
template <bool PK, typename T> __device__ __forceinline__ cx<T> vfma(T c, cx<T> a, cx<T> b) {
    return mk(fmat(c, a.x, b.x), fmat(c, a.y, b.y));
}
__device__ __forceinline__ float2 f2of(cx<float> a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ cx<float> cxof(float2 a) { return mk(a.x, a.y); }
__device__ __forceinline__ cx<float> vadd2(cx<float> a, cx<float> b) { return cxof(__fadd2_rn(f2of(a), f2of(b))); }
__device__ __forceinline__ cx<float> vsub2(cx<float> a, cx<float> b) {
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    cx<float> d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
    return d;
}
__device__ __forceinline__ cx<float> vfma2(float c, cx<float> a, cx<float> b) {
    return cxof(__ffma2_rn(make_float2(c, c), f2of(a), f2of(b)));
}
template <> __device__ __forceinline__ cx<float> vadd<true, float>(cx<float> a, cx<float> b) { return vadd2(a, b); }
template <> __device__ __forceinline__ cx<float> vsub<true, float>(cx<float> a, cx<float> b) { return vsub2(a, b); }
template <> __device__ __forceinline__ cx<float> vfma<true, float>(float c, cx<float> a, cx<float> b) {
    return vfma2(c, a, b);
}

// lo = e + w o, hi = e - w o for a runtime twiddle w: four FMAs form lo and
// hi = 2e - lo takes two more (6 instructions instead of a complex product
// and four additions; the absolute error stays within a rounding of |e| + |o|)
template <typename T>
__device__ __forceinline__ void bfly_w(cx<T> e, cx<T> o, cx<T> w, cx<T>& lo, cx<T>& hi) {
    lo = mk(fmat(o.x, w.x, fmat(-o.y, w.y, e.x)), fmat(o.y, w.x, fmat(o.x, w.y, e.y)));
    hi = mk(fmat(T(2), e.x, -lo.x), fmat(T(2), e.y, -lo.y));
}

// lo = e + W_R^K o, hi = e - W_R^K o with W_R = exp(-2 pi i / R): additions
// only for the trivial angles, two additions and four FMAs for the odd
// multiples of 45 degrees, four FMAs and the 2e - lo form otherwise.
template <int R, int K, bool PK = false, typename T>
__device__ __forceinline__ void bfly(cx<T> e, cx<T> o, cx<T>& lo, cx<T>& hi) {
    constexpr int k = K % R;
    if constexpr (k == 0) {
        lo = vadd<PK>(e, o);
        hi = vsub<PK>(e, o);
    } else if constexpr (4 * k == R) {
        const cx<T> t = mul_mi(o);
        lo = e + t;
        hi = e - t;
    } else if constexpr (2 * k == R) {
        lo = vsub<PK>(e, o);
        hi = vadd<PK>(e, o);
    } else if constexpr (4 * k == 3 * R) {
        const cx<T> t = mul_i(o);
        lo = e + t;
        hi = e - t;
    } else {
        constexpr bool tri = (R % 3 == 0);
        constexpr int idx = tri ? (k * 12 / R) : (k * 16 / R);
        constexpr double cd = tri ? kC12[idx] : kC16[idx];
        constexpr double sd = tri ? kS12[idx] : kS16[idx];
        const T c = T(cd), s = T(sd);
        // W o = (c o.x + s o.y, c o.y - s o.x)
        if constexpr (!tri && (8 * k) % R == 0 && cd == sd) {          // 1/8, 5/8 turn: (c u, c v)
            const cx<T> uv = mk(o.x + o.y, o.y - o.x);
            lo = vfma<PK>(c, uv, e);
            hi = vfma<PK>(-c, uv, e);
        } else if constexpr (!tri && (8 * k) % R == 0 && cd == -sd) {  // 3/8, 7/8 turn: (-c v, c u)
            const cx<T> vu = mk(o.x - o.y, o.x + o.y);                 // (-v, u)
            lo = vfma<PK>(c, vu, e);
            hi = vfma<PK>(-c, vu, e);
        } else {
            lo = mk(fmat(c, o.x, fmat(s, o.y, e.x)), fmat(c, o.y, fmat(-s, o.x, e.y)));
            hi = mk(fmat(T(2), e.x, -lo.x), fmat(T(2), e.y, -lo.y));
        }
    }
}

// ---------------------------------------------------------------------------
// Forward DFT codelets, in place on a[0..R-1] (natural order in and out).
// Even sizes are split decimation-in-time into two halves.
//   run(a)        : X = DFT(a)
//   run_tw<ONE>(a, w): X = DFT(a[r] w[r]), the stage twiddles folded into the
//                   first butterfly level (w[0] is 1 and unread when ONE)
// ---------------------------------------------------------------------------
template <int R, typename C, bool PK = false> struct Dft;   // C = cx<T>

template <typename C, bool PK> struct Dft<1, C, PK> {
    __device__ __forceinline__ static void run(C*) {}
};
template <typename C, bool PK> struct Dft<2, C, PK> {
    __device__ __forceinline__ static void run(C* a) { bfly<2, 0, PK>(a[0], a[1], a[0], a[1]); }
    template <bool ONE, typename Wt>
    __device__ __forceinline__ static void run_tw(C* a, const Wt* w) {
        const C x0 = ONE ? a[0] : cmul(a[0], w[0]);
        bfly_w(x0, a[1], w[1], a[0], a[1]);
    }
};
// scalar type of an element, and -i h d for a real h
template <typename C> struct RealOf;
template <typename T> struct RealOf<cx<T>> { using type = T; };
template <typename T> __device__ __forceinline__ cx<T> mi_scale(cx<T> d, T h) { return mk(d.y * h, -d.x * h); }

template <typename C, bool PK> struct Dft<3, C, PK> {
    using T = typename RealOf<C>::type;
    __device__ __forceinline__ static void run(C* a) {
        const T h = T(0.86602540378443864676);
        C s = a[1] + a[2], d = a[1] - a[2];
        C m = a[0] - s * T(0.5);
        a[0] = a[0] + s;
        C jd = mi_scale(d, h);   // -i*sin(60)*d
        a[1] = m + jd;
        a[2] = m - jd;
    }
    template <bool ONE, typename Wt>
    __device__ __forceinline__ static void run_tw(C* a, const Wt* w) {
        if (!ONE) a[0] = cmul(a[0], w[0]);
        a[1] = cmul(a[1], w[1]);
        a[2] = cmul(a[2], w[2]);
        run(a);
    }
};
template <typename C, bool PK> struct Dft<4, C, PK> {
    __device__ __forceinline__ static void finish(C* a, C s02, C d02, C s13, C d13) {
        bfly<4, 0, PK>(s02, s13, a[0], a[2]);
        bfly<4, 1, PK>(d02, d13, a[1], a[3]);   // d02 -/+ i d13
    }
    __device__ __forceinline__ static void run(C* a) {
        C s02, d02, s13, d13;
        bfly<2, 0, PK>(a[0], a[2], s02, d02);
        bfly<2, 0, PK>(a[1], a[3], s13, d13);
        finish(a, s02, d02, s13, d13);
    }
    template <bool ONE, typename Wt>
    __device__ __forceinline__ static void run_tw(C* a, const Wt* w) {
        const C x0 = ONE ? a[0] : cmul(a[0], w[0]);
        const C x1 = cmul(a[1], w[1]);
        C s02, d02, s13, d13;
        bfly_w(x0, a[2], w[2], s02, d02);
        bfly_w(x1, a[3], w[3], s13, d13);
        finish(a, s02, d02, s13, d13);
    }
};

template <int R, typename C, bool PK, int K = 0>
__device__ __forceinline__ void combine_half(C* e, C* o, C* a) {
    if constexpr (K < R / 2) {
        bfly<R, K, PK>(e[K], o[K], a[K], a[K + R / 2]);
        combine_half<R, C, PK, K + 1>(e, o, a);
    }
}

template <int R, typename C, bool PK> struct Dft {
    static_assert(R % 2 == 0, "odd codelet sizes other than 3 are not provided");
    __device__ __forceinline__ static void run(C* a) {
        C e[R / 2], o[R / 2];
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            e[i] = a[2 * i];
            o[i] = a[2 * i + 1];
        }
        Dft<R / 2, C, PK>::run(e);
        Dft<R / 2, C, PK>::run(o);
        combine_half<R, C, PK>(e, o, a);
    }
    template <bool ONE, typename Wt>
    __device__ __forceinline__ static void run_tw(C* a, const Wt* w) {
        C e[R / 2], o[R / 2];
        Wt we[R / 2], wo[R / 2];
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            e[i] = a[2 * i];
            o[i] = a[2 * i + 1];
            we[i] = w[2 * i];
            wo[i] = w[2 * i + 1];
        }
        Dft<R / 2, C, PK>::template run_tw<ONE>(e, we);
        Dft<R / 2, C, PK>::template run_tw<false>(o, wo);
        combine_half<R, C, PK>(e, o, a);
    }
};

// stage twiddles of element type C: the table layout and one entry
template <typename C> struct TwOf;
template <typename T> struct TwOf<cx<T>> {
    using tab = cx<T>;
    using type = cx<T>;
    __device__ __forceinline__ static cx<T> at(const cx<T>* tw, int i) { return ldg(&tw[i]); }
    __device__ __forceinline__ static cx<T> one() { return mk(T(1), T(0)); }
};

// ---------------------------------------------------------------------------
// Stage driver.
//   v      : thread's E elements, v[s] = x[p + P*s] on entry, X[p + P*s] on exit
//   sbuf   : exchange buffer; sidx(m) maps sequence index m to its slot
//   tw     : table W_N^m = exp(-2 pi i m / N), m < N (read-only path); with
//            TS > 1 the table of a TS times longer transform, read every TS-th entry
//   sync() : barrier over all threads sharing sbuf
// Plan::inv computes the inverse as conj(DFT(conj(x))).
// ---------------------------------------------------------------------------
template <typename C, bool PK, int TS, int N, int E, int Ns, typename SIdx, typename Sync, int R, int... Rest>
__device__ __forceinline__ void fft_stages(C (&v)[E], C* sbuf, int p, const typename TwOf<C>::tab* __restrict__ tw,
                                           SIdx sidx, Sync sync) {
    constexpr int P = N / E;
    constexpr int Q = E / R;
    constexpr bool last = (sizeof...(Rest) == 0);
    static_assert(E % R == 0, "radix must divide the elements per thread");
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = p + q * P;
        C a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = v[q + r * Q];
        int jm = 0;
        if constexpr (Ns > 1) {
            jm = j % Ns;
            constexpr int step = N / (Ns * R);
            typename TwOf<C>::type w[R];
            w[0] = TwOf<C>::one();
#pragma unroll
            for (int r = 1; r < R; ++r) w[r] = TwOf<C>::at(tw, TS * r * jm * step);
            Dft<R, C, PK>::template run_tw<true>(a, w);
        } else {
            Dft<R, C, PK>::run(a);
        }
        if constexpr (last) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[q + r * Q] = a[r];
        } else {
            const int idxD = (j / Ns) * Ns * R + jm;
#pragma unroll
            for (int r = 0; r < R; ++r) sbuf[sidx(idxD + r * Ns)] = a[r];
        }
    }
    if constexpr (!last) {
        sync();
#pragma unroll
        for (int s = 0; s < E; ++s) v[s] = sbuf[sidx(p + s * P)];
        sync();
        fft_stages<C, PK, TS, N, E, Ns * R, SIdx, Sync, Rest...>(v, sbuf, p, tw, sidx, sync);
    }
}

// A compile-time FFT plan: length N, E elements per thread, radices Rs...
template <int R, int... Rest> struct FirstOf { static constexpr int value = R; };
template <int N_, int E_, int... Rs>
struct Plan {
    static constexpr int N = N_;
    static constexpr int E = E_;
    static constexpr int P = N_ / E_;
    static constexpr int nstages = sizeof...(Rs);
    static constexpr int R1 = FirstOf<Rs...>::value;   // radix of the first stage
    // PK: FP32x2 additions in the butterflies (see vadd); TS: twiddle table of a
    // TS times longer transform
    template <bool PK = false, int TS = 1, typename C, typename SIdx, typename Sync>
    __device__ __forceinline__ static void fwd(C (&v)[E_], C* sbuf, int p, const typename TwOf<C>::tab* __restrict__ tw,
                                               SIdx sidx, Sync sync) {
        fft_stages<C, PK, TS, N_, E_, 1, SIdx, Sync, Rs...>(v, sbuf, p, tw, sidx, sync);
    }
    template <bool PK = false, int TS = 1, typename C, typename SIdx, typename Sync>
    __device__ __forceinline__ static void inv(C (&v)[E_], C* sbuf, int p, const typename TwOf<C>::tab* __restrict__ tw,
                                               SIdx sidx, Sync sync) {
#pragma unroll
        for (int s = 0; s < E_; ++s) v[s] = conjg(v[s]);
        fft_stages<C, PK, TS, N_, E_, 1, SIdx, Sync, Rs...>(v, sbuf, p, tw, sidx, sync);
#pragma unroll
        for (int s = 0; s < E_; ++s) v[s] = conjg(v[s]);
    }
};

}  // namespace ns3d
