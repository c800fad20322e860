// ns3d_inst_f32_large.cu — FP32-bulk engines, default tile variant, grid
// sizes 256 to 1024.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v0_r3(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v0_large(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_LARGE(NS3D_CASE)
        default:
            return make_f32_v0_r3(N, ps, M, s);
    }
}
}  // namespace ns3d
