// ns3d_inst.cuh — factory over the compiled grid sizes for one precision.
// Each precision lives in its own translation unit so the two compile in
// parallel; NS3D_SIZES lists every N with an FFT plan.
#pragma once
#include "ns3d_impl.cuh"

#define NS3D_SIZES(X) X(8) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(256) X(512) X(1024)

namespace ns3d {
template <typename T>
Base* make_typed(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    switch (N) {
#define NS3D_CASE(n) \
    case n:          \
        return new Impl<T, n>(ps, M, s);
        NS3D_SIZES(NS3D_CASE)
#undef NS3D_CASE
        default:
            return nullptr;
    }
}
}  // namespace ns3d
