// ns3d_inst_f64.cu — FP64 engines for every compiled grid size.
#include "ns3d_inst.cuh"

namespace ns3d {
Base* make_f64(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    return make_typed<double>(N, ps, M, s);
}
}  // namespace ns3d
