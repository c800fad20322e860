// ns3d_inst_f64.cu — FP64 engines for every compiled grid size.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f64_v0(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = double;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_SMALL(NS3D_CASE)
        NS3D_SIZES_LARGE(NS3D_CASE)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
