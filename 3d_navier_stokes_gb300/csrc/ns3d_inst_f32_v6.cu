// ns3d_inst_f32_v6.cu — FP32-bulk engines in variant 6 (16-pencil y tiles,
// 8-pencil x-inverse and 16-pencil x-forward tiles) for the sizes the
// autotuner chooses among.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v6(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 6;
    switch (N) {
        NS3D_TUNED_SIZES(NS3D_CASE)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
