// ns3d_inst_f32.cu — FP32-bulk engines (FP64 integrating factors, time and
// reductions), default tile variant, grid sizes up to 128.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v0_large(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f32_v0(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_SMALL(NS3D_CASE)
        default:
            return make_f32_v0_large(N, ps, M, s);
    }
}
}  // namespace ns3d
