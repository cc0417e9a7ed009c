// The signal path's coupling to the strips (GroundTruth: PlaneStack.strip_coupling, peec.py:2615-2656, with
// kernel.segment_vector_potential, kernel.py:297-312): psi of every strip, the flux per ampere of signal current
// along it, in FP64 on the device.
//
// For a strip of orientation `axis` on sheet k (centre of its cell at the sheet face nearer the segment) and a
// horizontal signal segment a -> b with a component along the axis, the segment's vector potential
//     A(p) = mu0 / (4 pi) [asinh((L - p.u) / rho) + asinh(p.u / rho)],  rho = max(dist(p, line), r_min)
// is taken at the centre, or averaged over the cell with a 3 x 3 Gauss rule when the centre lies within
// 3 d + 2 w of the segment; psi = d * sum_segments current * (b - a)[axis] / L * A.
#include "kernels.h"

namespace gt {

namespace {

constexpr double MU0_4PI = 1e-7;     // mu0 / (4 pi)
constexpr int SEG_TILE = 256;

struct Seg {
    double a[3], b[3], width, cur;
};

__device__ __forceinline__ double vec_pot(const Seg& s, double L, const double* u, double px, double py, double pz,
                                          double rmin) {
    const double dx = px - s.a[0], dy = py - s.a[1], dz = pz - s.a[2];
    const double pu = dx * u[0] + dy * u[1] + dz * u[2];
    const double rho = sqrt(fmax(dx * dx + dy * dy + dz * dz - pu * pu, rmin * rmin));
    return MU0_4PI * (asinh((L - pu) / rho) + asinh(pu / rho));
}

__device__ __forceinline__ double dist_to_segment(const Seg& s, double px, double py, double pz) {
    const double ab[3] = {s.b[0] - s.a[0], s.b[1] - s.a[1], s.b[2] - s.a[2]};
    const double L2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
    double t = 0.0;
    if (L2 > 0) t = fmin(fmax(((px - s.a[0]) * ab[0] + (py - s.a[1]) * ab[1] + (pz - s.a[2]) * ab[2]) / L2, 0.0), 1.0);
    const double qx = px - (s.a[0] + t * ab[0]), qy = py - (s.a[1] + t * ab[1]), qz = pz - (s.a[2] + t * ab[2]);
    return sqrt(qx * qx + qy * qy + qz * qz);
}

__global__ void __launch_bounds__(256) strip_coupling_kernel(Geo g, const int64_t* __restrict__ c2d, int64_t ns,
                                                             const double* __restrict__ sheet_z,
                                                             const double* __restrict__ sheet_t, double d,
                                                             const double* __restrict__ segs, int nseg,
                                                             double* __restrict__ psi) {
    __shared__ Seg sh[SEG_TILE];
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = c < ns;
    int axis = 0, k = 0;
    double cx = 0, cy = 0;
    if (act) {
        const int64_t pos = c2d[c];
        const int nx = g.nx, ny = g.ny;
        if (pos < g.off_y) {
            const int64_t q = pos - g.off_x, plane = (int64_t)(nx - 1) * ny;
            k = int(q / plane);
            const int64_t ij = q - k * plane;
            const int i = int(ij / ny), j = int(ij - (int64_t)i * ny);
            cx = i * d + 0.5 * d;
            cy = j * d;
        } else {
            axis = 1;
            const int64_t q = pos - g.off_y, plane = (int64_t)nx * (ny - 1);
            k = int(q / plane);
            const int64_t ij = q - k * plane;
            const int i = int(ij / (ny - 1)), j = int(ij - (int64_t)i * (ny - 1));
            cx = i * d;
            cy = j * d + 0.5 * d;
        }
    }
    const double zk = act ? sheet_z[k] : 0.0, half = act ? 0.5 * sheet_t[k] : 0.0;
    // the 3-point Gauss-Legendre rule on [-1/2, 1/2]
    const double gq[3] = {-0.5 * sqrt(0.6), 0.0, 0.5 * sqrt(0.6)};
    const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    double acc = 0.0;
    for (int t0 = 0; t0 < nseg; t0 += SEG_TILE) {
        const int nt = min(SEG_TILE, nseg - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < nt; q += blockDim.x) {
            const double* r = segs + (int64_t)(t0 + q) * 8;
            sh[q] = Seg{{r[0], r[1], r[2]}, {r[3], r[4], r[5]}, r[6], r[7]};
        }
        __syncthreads();
        if (!act) continue;
        for (int q = 0; q < nt; ++q) {
            const Seg& s = sh[q];
            const double ab[3] = {s.b[0] - s.a[0], s.b[1] - s.a[1], s.b[2] - s.a[2]};
            if (ab[0] == 0.0 && ab[1] == 0.0) continue;                  // vertical: not a horizontal segment
            const double L = sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]);
            if (fabs(ab[axis]) < 1e-15 * L) continue;
            const double u[3] = {ab[0] / L, ab[1] / L, ab[2] / L};
            const double cz = zk + (0.5 * (s.a[2] + s.b[2]) > zk ? half : -half);
            const double rmin = fmax(0.5 * s.width, 1e-7);
            double a;
            if (dist_to_segment(s, cx, cy, cz) < 3 * d + 2 * s.width) {
                a = 0.0;
                for (int m = 0; m < 3; ++m)
                    for (int n = 0; n < 3; ++n) {
                        const double da = (axis == 0 ? gq[m] : gq[n]) * d, dl = (axis == 0 ? gq[n] : gq[m]) * d;
                        a += vec_pot(s, L, u, cx + da, cy + dl, cz, rmin) * (gw[m] * gw[n] / 4.0);
                    }
            } else {
                a = vec_pot(s, L, u, cx, cy, cz, rmin);
            }
            acc += (s.cur * ab[axis] / L) * a;
        }
    }
    if (act) psi[c] = d * acc;
}

}  // namespace

void launch_strip_coupling(const Geo& g, const int64_t* c2d, int64_t ns, const double* sheet_z, const double* sheet_t,
                           double d, const double* segs, int nseg, double* psi, cudaStream_t st) {
    if (ns <= 0) return;
    strip_coupling_kernel<<<ceil_div(ns, 256), 256, 0, st>>>(g, c2d, ns, sheet_z, sheet_t, d, segs, nseg, psi);
    GT_LAUNCH_CHECK();
}

}  // namespace gt
