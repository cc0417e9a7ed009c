// Post-solve outputs on the device, from dense FP64 solutions (GroundTruth: Solution.node_field,
// peec.py:1151-1203, copper=False; PlaneStack.moment, peec.py:2668-2700, the plane's part).
#include "kernels.h"

namespace gt {

// (Kx, Ky) at every node of every sheet: each node averages the strips of each direction that touch it and
// carry current, per cell width d.  kx / ky: [col][S][nx][ny].
__global__ void __launch_bounds__(256) node_field_kernel(Geo g, const c64* __restrict__ x, int64_t ld, double d,
                                                         c64* __restrict__ kx, c64* __restrict__ ky) {
    const int S = g.S, nx = g.nx, ny = g.ny;
    const int k = blockIdx.y, col = blockIdx.z;
    const c64* X = x + (int64_t)col * ld + g.off_x + (int64_t)k * (nx - 1) * ny;
    const c64* Y = x + (int64_t)col * ld + g.off_y + (int64_t)k * nx * (ny - 1);
    c64* ox = kx + ((int64_t)col * S + k) * nx * ny;
    c64* oy = ky + ((int64_t)col * S + k) * nx * ny;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)nx * ny; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = int(q / ny), j = int(q - (int64_t)i * ny);
        c64 sx = zero<double>(), sy = zero<double>();
        int cx = 0, cy = 0;
        if (i > 0) { const c64 v = X[(int64_t)(i - 1) * ny + j]; sx += v; cx += (v.re != 0 || v.im != 0); }
        if (i < nx - 1) { const c64 v = X[(int64_t)i * ny + j]; sx += v; cx += (v.re != 0 || v.im != 0); }
        if (j > 0) { const c64 v = Y[(int64_t)i * (ny - 1) + j - 1]; sy += v; cy += (v.re != 0 || v.im != 0); }
        if (j < ny - 1) { const c64 v = Y[(int64_t)i * (ny - 1) + j]; sy += v; cy += (v.re != 0 || v.im != 0); }
        ox[q] = (1.0 / (double)max(cx, 1) / d) * sx;
        oy[q] = (1.0 / (double)max(cy, 1) / d) * sy;
    }
}

void launch_node_field(const Geo& g, const c64* x, int64_t ld, int ncol, double d, c64* kx, c64* ky, cudaStream_t st) {
    const int64_t nxy = (int64_t)g.nx * g.ny;
    node_field_kernel<<<dim3((int)std::min<int64_t>((nxy + 255) / 256, 256), g.S, ncol), 256, 0, st>>>(g, x, ld, d, kx, ky);
    GT_LAUNCH_CHECK();
}

// m = 1/2 sum r x I dl over the plane's strips, capacitances and branches, per column (the signal segments'
// own part is the caller's).  One block per column; m: [col][3].
__global__ void __launch_bounds__(512) moment_kernel(Geo g, const c64* __restrict__ x, int64_t ld,
                                                     const double* __restrict__ zs, double d, c64* __restrict__ m) {
    const int S = g.S, nx = g.nx, ny = g.ny, col = blockIdx.x;
    const c64* xc = x + (int64_t)col * ld;
    const int64_t nX = (int64_t)S * (nx - 1) * ny, nY = (int64_t)S * nx * (ny - 1), nxy = (int64_t)nx * ny;
    c64 a0 = zero<double>(), a1 = zero<double>(), a2 = zero<double>();
    for (int64_t q = threadIdx.x; q < nX; q += blockDim.x) {       // x strips (k, i, j): r = (., j d, z_k)
        const int64_t k = q / ((int64_t)(nx - 1) * ny), j = q % ny;
        const c64 I = xc[g.off_x + q];
        a1 += (zs[k] * d) * I;
        a2 += (-(double)j * d * d) * I;
    }
    for (int64_t q = threadIdx.x; q < nY; q += blockDim.x) {       // y strips (k, i, j): r = (i d, ., z_k)
        const int64_t k = q / ((int64_t)nx * (ny - 1)), i = (q % ((int64_t)nx * (ny - 1))) / (ny - 1);
        const c64 I = xc[g.off_y + q];
        a0 += (-zs[k] * d) * I;
        a2 += ((double)i * d * d) * I;
    }
    for (int64_t q = threadIdx.x; q < (int64_t)g.np * nxy; q += blockDim.x) {   // capacitances, upper -> lower
        const int p = int(q / nxy);
        const int64_t ij = q - (int64_t)p * nxy;
        const double px = (double)(ij / ny) * d, py = (double)(ij % ny) * d;
        const double dz = zs[g.pair_layers[2 * p + 1]] - zs[g.pair_layers[2 * p]];
        const c64 I = xc[g.off_c + q];
        a0 += (py * dz) * I;
        a1 += (-px * dz) * I;
    }
    for (int b = threadIdx.x; b < g.nbr; b += blockDim.x) {         // branches a -> b: r_a x r_b
        const int na = g.branch_nodes[2 * b], nb = g.branch_nodes[2 * b + 1];
        const double ax = (double)((na % nxy) / ny) * d, ay = (double)((na % nxy) % ny) * d, az = zs[na / nxy];
        const double bx = (double)((nb % nxy) / ny) * d, by = (double)((nb % nxy) % ny) * d, bz = zs[nb / nxy];
        const c64 I = xc[g.off_b + b];
        a0 += (ay * bz - az * by) * I;
        a1 += (az * bx - ax * bz) * I;
        a2 += (ax * by - ay * bx) * I;
    }
    __shared__ c64 red[3][512 / 32];
    c64 v[3] = {a0, a1, a2};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
        double re = v[c].re, im = v[c].im;
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (lane == 0) red[c][warp] = mk<double>(re, im);
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        c64 s = zero<double>();
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
        m[(int64_t)col * 3 + threadIdx.x] = 0.5 * s;
    }
}

void launch_moment(const Geo& g, const c64* x, int64_t ld, int ncol, const double* zs, double d, c64* m,
                   cudaStream_t st) {
    moment_kernel<<<ncol, 512, 0, st>>>(g, x, ld, zs, d, m);
    GT_LAUNCH_CHECK();
}

}  // namespace gt
