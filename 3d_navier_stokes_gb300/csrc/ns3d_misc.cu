// ns3d_misc.cu — non-template kernels: the final reduction of the
// diagnostics and the host-array dealiasing of the C ABI.
#include "ns3d_kernels.cuh"

namespace ns3d {
// Column sums of the measurement partials in CTA order (fixed order, so the
// result is bitwise reproducible), then the reference scalings
// (solver.c:1270-1274).
__global__ void k_measure_reduce(const double* __restrict__ part, int nparts, int width, int nsp,
                                 double N3sq, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= width) return;
    double a = 0.0;
    for (int q = 0; q < nparts; ++q) a += part[(long long)q * width + c];
    const double cf = 8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846;
    const double nf = 0.5 / N3sq;
    if (c < 5) a *= (c == 4 ? 2.0 : 1.0) * cf * nf;
    else a *= cf * nf;
    out[c] = a;
}


__global__ void k_dealias_ref_entry(double2* a, int N, int dim) {
    const int NF = N / 2 + 1;
    const long long total = (long long)N * N * NF;
    const long long kc = N / 3;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int kz = (int)(q % NF);
        const long long ij = q / NF;
        const int j = (int)(ij % N), i = (int)(ij / N);
        const long long kx = i <= N / 2 ? i : i - N, ky = j <= N / 2 ? j : j - N;
        if (kx * kx + ky * ky + (long long)kz * kz > kc * kc)
            for (int c = 0; c < dim; ++c) a[q * dim + c] = make_double2(0.0, 0.0);
    }
}
}  // namespace ns3d
