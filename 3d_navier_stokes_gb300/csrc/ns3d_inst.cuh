// ns3d_inst.cuh — engines over the compiled grid sizes for one precision and
// tile variant. Each (precision, variant, size range) lives in its own
// translation unit so they compile in parallel. NS3D_SIZES_SMALL / _LARGE /
// _R3 list every N with an FFT plan (powers of two, and 3 x 2^k);
// NS3D_TUNED_SIZES the sizes whose FP32 engines also exist in the alternative
// tile variants the autotuner chooses from.
#pragma once
#include "ns3d_impl.cuh"

#define NS3D_SIZES_SMALL(X) X(8) X(16) X(24) X(32) X(48) X(64) X(96) X(128)
#define NS3D_SIZES_LARGE(X) X(256) X(512) X(1024)
#define NS3D_SIZES_R3(X) X(192) X(384) X(768)
#define NS3D_TUNED_SIZES(X) X(48) X(64) X(96) X(128) X(256) X(512)

#define NS3D_CASE(n) \
    case n:          \
        return new Impl<T, n, V>(ps, M, s);
