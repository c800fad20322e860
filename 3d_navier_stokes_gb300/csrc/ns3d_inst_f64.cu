// ns3d_inst_f64.cu — FP64 engines for the small grid sizes (256^3 and up in
// ns3d_inst_f64_large.cu, compiled beside this unit).
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f64_v0(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = double;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_SMALL(NS3D_CASE)
        default:
            return make_f64_large(N, ps, M, s);
    }
}
}  // namespace ns3d
