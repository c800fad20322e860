// ns3d_inst_f32_v4.cu — FP32-bulk engines in variant 4 (x passes with twice
// the elements per thread and 8-pencil tiles, PlansV<N, 4>) for the sizes
// where that plan exists.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v4(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 4;
    switch (N) {
        NS3D_CASE(64)
        NS3D_CASE(128)
        NS3D_CASE(256)
        NS3D_CASE(512)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
