// ns3d_inst_f32.cu — FP32-bulk engines (FP64 integrating factors, time and
// reductions) for every compiled grid size.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f32(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    return make_typed<float>(N, ps, M, s);
}
}  // namespace ns3d
