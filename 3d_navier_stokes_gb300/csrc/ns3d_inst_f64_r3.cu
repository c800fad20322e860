// ns3d_inst_f64_r3.cu — FP64 engines for the grid sizes with a factor 3:
// 192, 384, 768.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f64_r3(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = double;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_R3(NS3D_CASE)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
