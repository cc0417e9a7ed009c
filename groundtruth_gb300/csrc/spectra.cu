// Partial-inductance kernel spectra on the device (GroundTruth: PlaneStack._kernel_pair / _kernel_spectrum,
// peec.py:3276-3306 and 3362-3371, with kernel.strip_kernel / filament_mutual, kernel.py:170-176 and 268-294),
// FP64.
//
// The mutual inductance of two square strips of pitch d at every grid offset (axial a, lateral l, sheet gap dz)
// is the filament formula
//     M = mu0/(4 pi) [G(a + d) - 2 G(a) + G(a - d)],  G(u) = u asinh(u / rho) - sqrt(u^2 + rho^2),
//     rho = max(sqrt(l^2 + dz^2), 1e-12 d),
// except the (NEAR+1)^2 nearest offsets, integrated as tapes (given by the caller).  The kernel is wrapped onto
// the P0 x P1 torus centred at the origin and transformed; being real and even, its spectrum is real: the
// (P0/2+1) x (P1/2+1) quadrant of the real part is returned.
#include <cmath>
#include <vector>
#include "common.cuh"
#include "fft.cuh"
#include "kernels.h"

namespace gt {

namespace {

constexpr double MU0_4PI = 1e-7;

__device__ __forceinline__ double fil_G(double u, double rho) { return u * asinh(u / rho) - sqrt(u * u + rho * rho); }

// Z[P0][P1] (complex, imaginary zero) = the kernel wrapped onto the torus
__global__ void kernel_grid_kernel(int na, int nl, double d, double dz, int P0, int P1, const double* __restrict__ near,
                                   int nnear, c64* __restrict__ Z) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)P0 * P1) return;
    const int r = int(q / P1), c = int(q - (int64_t)r * P1);
    // torus position (r, c) holds offset (oa, ol) with oa = r or r - P0, ol = c or c - P1
    const int oa = r < P0 - (na - 1) ? r : r - P0, ol = c < P1 - (nl - 1) ? c : c - P1;
    double v = 0.0;
    if (oa > -na && oa < na && ol > -nl && ol < nl) {
        const int aa = abs(oa), al = abs(ol);
        if (aa < nnear && al < nnear) {
            v = near[aa * nnear + al];
        } else {
            const double a = oa * d, l = ol * d;
            const double rho = fmax(sqrt(l * l + dz * dz), 1e-12 * d);
            v = MU0_4PI * (fil_G(a + d, rho) - 2.0 * fil_G(a, rho) + fil_G(a - d, rho));
        }
    }
    Z[q] = mk<double>(v, 0.0);
}

// one FFT row (length P) per block, in place in Z (row stride P, or a column with stride `stride`);
// rows: r < nrow; out: when not null, the real parts of entries < nout are written to out[r * nout + i]
__global__ void fft_lines_kernel(c64* __restrict__ Z, int P, int64_t line_step, int64_t elem_step, int nrow,
                                 const c64* __restrict__ tw, double* __restrict__ out, int nout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c64* row = reinterpret_cast<c64*>(smem_raw);
    const int r = blockIdx.x;
    if (r >= nrow) return;
    c64* line = Z + (int64_t)r * line_step;
    for (int i = threadIdx.x; i < P; i += blockDim.x) row[spad(i)] = line[(int64_t)i * elem_step];
    __syncthreads();
    fft_row<double, false>(row, true, P, tw, P / 8, threadIdx.x);
    if (out) {
        for (int i = threadIdx.x; i < nout; i += blockDim.x) out[(int64_t)r * nout + i] = row[spad(i)].re;
    } else {
        for (int i = threadIdx.x; i < P; i += blockDim.x) line[(int64_t)i * elem_step] = row[spad(i)];
    }
}

// device buffers freed on scope exit
struct DevBuf {
    void* p = nullptr;
    explicit DevBuf(size_t bytes) { GT_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16))); }
    ~DevBuf() { if (p) cudaFree(p); }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

void kernel_spectrum(int na, int nl, double d, double dz, int P0, int P1, const double* near_h, int nnear,
                     double* quad_h) {
    cudaStream_t st = 0;
    const int Q0 = P0 / 2 + 1, Q1 = P1 / 2 + 1;
    DevBuf bZ((size_t)P0 * P1 * sizeof(c64)), bN((size_t)nnear * nnear * sizeof(double)),
        bT((size_t)Q1 * Q0 * sizeof(double)), b0((size_t)P0 * sizeof(c64)), b1((size_t)P1 * sizeof(c64));
    c64* Z = bZ.as<c64>();
    double* dn = bN.as<double>();
    double* T = bT.as<double>();
    c64* tw0 = b0.as<c64>();
    c64* tw1 = b1.as<c64>();
    std::vector<c64> t0(P0), t1(P1);
    for (int m = 0; m < P0; ++m) t0[m] = mk<double>(std::cos(-2.0 * M_PI * m / P0), std::sin(-2.0 * M_PI * m / P0));
    for (int m = 0; m < P1; ++m) t1[m] = mk<double>(std::cos(-2.0 * M_PI * m / P1), std::sin(-2.0 * M_PI * m / P1));
    GT_CUDA(cudaMemcpy(dn, near_h, (size_t)nnear * nnear * sizeof(double), cudaMemcpyHostToDevice));
    GT_CUDA(cudaMemcpy(tw0, t0.data(), P0 * sizeof(c64), cudaMemcpyHostToDevice));
    GT_CUDA(cudaMemcpy(tw1, t1.data(), P1 * sizeof(c64), cudaMemcpyHostToDevice));
    const int64_t tot = (int64_t)P0 * P1;
    kernel_grid_kernel<<<ceil_div(tot, 256), 256, 0, st>>>(na, nl, d, dz, P0, P1, dn, nnear, Z);
    GT_LAUNCH_CHECK();
    // rows (length P1), then the columns c <= P1/2 (length P0), keeping rows <= P0/2 of their real parts
    size_t sm1 = (size_t)srow(P1) * sizeof(c64), sm0 = (size_t)srow(P0) * sizeof(c64);
    raise_smem((const void*)fft_lines_kernel, std::max(sm0, sm1));
    fft_lines_kernel<<<P0, P1 / 8, sm1, st>>>(Z, P1, P1, 1, P0, tw1, nullptr, 0);
    GT_LAUNCH_CHECK();
    fft_lines_kernel<<<Q1, P0 / 8, sm0, st>>>(Z, P0, 1, P1, Q1, tw0, T, Q0);
    GT_LAUNCH_CHECK();
    std::vector<double> Th((size_t)Q1 * Q0);
    GT_CUDA(cudaMemcpy(Th.data(), T, Th.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < Q0; ++i)
        for (int j = 0; j < Q1; ++j) quad_h[(int64_t)i * Q1 + j] = Th[(int64_t)j * Q0 + i];
}

}  // namespace gt
