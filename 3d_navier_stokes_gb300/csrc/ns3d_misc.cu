// ns3d_misc.cu — non-template kernels: the final reduction of the
// diagnostics and the host-array dealiasing of the C ABI; the host-built DFT
// matrices of the tensor-core z pass; tensor-map encoding.
#include <string.h>

#include <vector>

#include "ns3d_kernels.cuh"

namespace ns3d {
void twiddle_table(int n, double* re, double* im);

// 4D FP32 tensor map (dims innermost first, byte strides of dims 1..3, box in
// elements), no swizzle, through the driver's cuTensorMapEncodeTiled; false
// when the entry point is missing or the encoding is refused
bool encode_map4_f32(CUtensorMap* map, void* base, const uint64_t dims[4], const uint64_t strides[3],
                     const uint32_t box[4]) {
    using encode_fn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static encode_fn fn = nullptr;
    if (!fn) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !f)
            return false;
        fn = reinterpret_cast<encode_fn>(f);
    }
    const cuuint64_t d[4] = {dims[0], dims[1], dims[2], dims[3]};
    const cuuint64_t st[3] = {strides[0], strides[1], strides[2]};
    const cuuint32_t b[4] = {box[0], box[1], box[2], box[3]};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, d, st, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

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
