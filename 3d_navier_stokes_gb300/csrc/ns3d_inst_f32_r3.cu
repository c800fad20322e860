// ns3d_inst_f32_r3.cu — FP32-bulk engines, default tile variant, the grid
// sizes with a factor 3: 192, 384, 768.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v0_r3(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_R3(NS3D_CASE)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
