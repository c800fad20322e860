// ns3d_misc.cu — non-template kernels: the final reduction of the
// diagnostics and the host-array dealiasing of the C ABI; the host-built DFT
// matrices of the tensor-core z pass.
#include <string.h>

#include <vector>

#include "ns3d_kernels.cuh"

namespace ns3d {
void twiddle_table(int n, double* re, double* im);

// BF16 bits of x, round to nearest even (finite x)
static uint16_t bf16_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float bf16_value(uint16_t b) {
    const uint32_t u = (uint32_t)b << 16;
    float x;
    memcpy(&x, &u, 4);
    return x;
}

void zgemm_matrices(int N, int KI, uint16_t* out) {
    const int KC = N / 3, KIN = 2 * (KC + 1);
    std::vector<double> re(N), im(N);
    twiddle_table(N, re.data(), im.data());   // e^{-2 pi i m / N}: re = cos, im = -sin
    // element (row r, column k) of a canonical K-major operand with K columns
    auto at = [](uint16_t* base, int r, int k, int K) -> uint16_t& {
        return base[(size_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7))];
    };
    uint16_t* ih = out;
    uint16_t* il = out + (size_t)N * KI;
    uint16_t* fh = il + (size_t)N * KI;
    uint16_t* fl = fh + (size_t)KI * N;
    auto put = [&](uint16_t* h, uint16_t* l, int r, int k, int K, double v) {
        const uint16_t hb = bf16_bits((float)v);
        at(h, r, k, K) = hb;
        at(l, r, k, K) = bf16_bits((float)(v - (double)bf16_value(hb)));
    };
    for (int z = 0; z < N; ++z)
        for (int k = 0; k < KI; ++k) {
            const int kz = k / 2, part = k % 2;
            double vi = 0.0, vf = 0.0;
            if (k < KIN) {
                const int m = (int)(((long long)kz * z) % N);
                const double c = re[m], sn = -im[m];   // cos, sin of 2 pi kz z / N
                const double mult = kz == 0 ? 1.0 : 2.0;
                // c2r: u = sum m (Re c cos - Im c sin); the kz = 0 imaginary part does not contribute
                vi = part == 0 ? mult * c : (kz == 0 ? 0.0 : -mult * sn);
                // r2c: Re = sum p cos, Im = -sum p sin
                vf = part == 0 ? c : -sn;
            }
            put(ih, il, z, k, KI, vi);
            put(fh, fl, k, z, N, vf);
        }
}

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
