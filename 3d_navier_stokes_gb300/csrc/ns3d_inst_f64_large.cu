// ns3d_inst_f64_large.cu — FP64 engines for 256^3, 512^3 and 1024^3.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f64_r3(int N, const ns3d_params* ps, int M, cudaStream_t s);
Base* make_f64_large(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = double;
    constexpr int V = 0;
    switch (N) {
        NS3D_SIZES_LARGE(NS3D_CASE)
        default:
            return make_f64_r3(N, ps, M, s);
    }
}
}  // namespace ns3d
