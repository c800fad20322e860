// ns3d_inst_f32_v5.cu — FP32-bulk engines in variant 5 (default tiles and
// plans, x-forward pass compiled for two CTAs per SM) for the sizes the
// autotuner chooses among.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v5(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 5;
    switch (N) {
        NS3D_TUNED_SIZES(NS3D_CASE)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
