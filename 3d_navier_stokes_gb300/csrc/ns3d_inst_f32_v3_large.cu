// ns3d_inst_f32_v3_large.cu — the 1024^3 FP32-bulk engine in variant 3 (x passes
// with 16 elements per thread on 8-pencil tiles), in its own translation unit
// so that it compiles beside the other sizes of the variant.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32_v3_large(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    using T = float;
    constexpr int V = 3;
    switch (N) {
        NS3D_CASE(1024)
        default:
            return nullptr;
    }
}
}  // namespace ns3d
