// ns3d_inst_f32_v3.cu — FP32-bulk engines in variant 3 (x passes with twice
// the elements per thread and 16-pencil tiles, PlansV<N, 3>) for the sizes
// where that plan exists (1024^3 in ns3d_inst_f32_v3_large.cu).
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v3(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 3;
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
