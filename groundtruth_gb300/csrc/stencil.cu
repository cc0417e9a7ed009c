// Grid-stencil kernels of the system product and the preconditioner on the dense layout.
//
// System product rows besides the strips (peec.py:3043-3062):
//   capacitance  z_cap I_c - (V[upper] - V[lower])
//   branch       z_br  I_b - (V[a] - V[b])
//   node (KCL)   Ar^T I: I_x(k,i,j) - I_x(k,i-1,j) + I_y(k,i,j) - I_y(k,i,j-1) + caps + branches
// Preconditioner (peec.py:3064-3083, D^-1 from peec.py:2465-2511):
//   s = r_V - Ar^T D^-1 r_1                  (pc_node, written in factor order)
//   y = S^-1 s                               (factor.cu)
//   out = [D^-1 (r_1 + Ar y); y]             (pc_strip)
// D^-1 acts per strip position through a table of S x S blocks indexed by the position's sheet-presence
// code (diagonal blocks for precond "diag"), per capacitance and per branch through scalars.
#include "kernels.h"

namespace gt {

namespace {

__device__ __forceinline__ int seg_of(const Geo& g, int64_t pos, int64_t nX, int64_t nY) {
    if (pos < g.off_x + nX) return 0;
    if (pos < g.off_y) return -1;
    if (pos < g.off_y + nY) return 1;
    if (pos < g.off_c) return -1;
    if (pos < g.off_b) return 2;
    if (pos < g.off_v) return 3;
    return 4;
}

// D^-1 applied to the strips at one position: strip of sheet k, orientation o, with the vector u over the
// sheets present (code)
template <typename R>
__device__ __forceinline__ cx<R> dinv_strip(const c64* tab, int S, int o, int code, int k, const cx<R>* u) {
    const int NC = 1 << S;
    const c64* T = tab + (((int64_t)o * NC + code) * S + k) * S;
    cx<R> acc = zero<R>();
    for (int l = 0; l < S; ++l)
        if ((code >> l) & 1) acc += cvt<R>(T[l]) * u[l];
    return acc;
}

template <typename R>
__device__ __forceinline__ cx<R> load_or0(const cx<R>* p, bool ok) { return ok ? *p : zero<R>(); }

}  // namespace

template <typename R>
__global__ void tail_kernel(Geo g, const cx<R>* __restrict__ x, const cx<R>* __restrict__ rhs, cx<R>* __restrict__ out,
                            int64_t ld, const int* __restrict__ col_op, const c64* __restrict__ zcap,
                            const c64* __restrict__ zbr, int mode, const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int op = col_op ? col_op[col] : 0;
    const int64_t nX = (int64_t)g.S * (g.nx - 1) * g.ny, nY = (int64_t)g.S * g.nx * (g.ny - 1);
    const cx<R>* xc = x + (int64_t)col * ld;
    for (int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pos < g.n; pos += (int64_t)gridDim.x * blockDim.x) {
        int seg = seg_of(g, pos, nX, nY);
        if (seg == 0 || seg == 1) continue;         // strips: written by the FFT pass
        cx<R> y = zero<R>();
        if (seg >= 2 && g.mask[pos]) {
            const cx<R>* V = xc + g.off_v;
            if (seg == 2) {
                int64_t q = pos - g.off_c;
                int p = int(q / ((int64_t)g.nx * g.ny));
                int64_t ij = q - (int64_t)p * g.nx * g.ny;
                int u = g.pair_layers[2 * p], l = g.pair_layers[2 * p + 1];
                y = cvt<R>(zcap[(int64_t)op * g.np + p]) * xc[pos] - (V[(int64_t)u * g.nx * g.ny + ij] - V[(int64_t)l * g.nx * g.ny + ij]);
            } else if (seg == 3) {
                int b = int(pos - g.off_b);
                y = cvt<R>(zbr[(int64_t)op * g.nbr + b]) * xc[pos] - (V[g.branch_nodes[2 * b]] - V[g.branch_nodes[2 * b + 1]]);
            } else {
                int64_t node = pos - g.off_v;
                int k = int(node / ((int64_t)g.nx * g.ny));
                int64_t ij = node - (int64_t)k * g.nx * g.ny;
                int i = int(ij / g.ny), j = int(ij - (int64_t)i * g.ny);
                const cx<R>* X = xc + g.off_x + (int64_t)k * (g.nx - 1) * g.ny;
                const cx<R>* Y = xc + g.off_y + (int64_t)k * g.nx * (g.ny - 1);
                cx<R> s = zero<R>();
                if (i < g.nx - 1) s += X[(int64_t)i * g.ny + j];
                if (i > 0) s -= X[(int64_t)(i - 1) * g.ny + j];
                if (j < g.ny - 1) s += Y[(int64_t)i * (g.ny - 1) + j];
                if (j > 0) s -= Y[(int64_t)i * (g.ny - 1) + j - 1];
                for (int p = 0; p < g.np; ++p) {
                    int u = g.pair_layers[2 * p], l = g.pair_layers[2 * p + 1];
                    if (u == k) s += xc[g.off_c + (int64_t)p * g.nx * g.ny + ij];
                    if (l == k) s -= xc[g.off_c + (int64_t)p * g.nx * g.ny + ij];
                }
                for (int e = g.node_br_ptr[node]; e < g.node_br_ptr[node + 1]; ++e) {
                    int b = g.node_br_idx[e];
                    if (b > 0) s += xc[g.off_b + b - 1];
                    else s -= xc[g.off_b - b - 1];
                }
                y = s;
            }
            if (mode == 1) y = rhs[(int64_t)col * ld + pos] - y;
        }
        out[(int64_t)col * ld + pos] = y;
    }
}

template <typename R>
void launch_tail(const Geo& g, const cx<R>* x, const cx<R>* rhs, cx<R>* out, int64_t ld, int ncol, const int* col_op,
                 const c64* zcap, const c64* zbr, int mode, const int* col_list, cudaStream_t st) {
    int64_t items = g.n;
    int blocks = (int)std::min<int64_t>((items + 255) / 256, 4096);
    tail_kernel<R><<<dim3(blocks, ncol), 256, 0, st>>>(g, x, rhs, out, ld, col_op, zcap, zbr, mode, col_list);
    GT_LAUNCH_CHECK();
}

// s[perm[node]] = r_V[node] - (Ar^T D^-1 r_1)[node] for every kept node
template <typename R>
__global__ void pc_node_kernel(Geo g, const cx<R>* __restrict__ r, int64_t ld, cx<R>* __restrict__ sd,
                               const int* __restrict__ col_op, const c64* __restrict__ tab, const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int op = col_op ? col_op[col] : 0;
    const c64* T = tab + (int64_t)op * g.ntab;
    const cx<R>* rc = r + (int64_t)col * ld;
    const int S = g.S, nx = g.nx, ny = g.ny;
    const int64_t nxy = (int64_t)nx * ny;
    for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < S * nxy; node += (int64_t)gridDim.x * blockDim.x) {
        if (!g.mask[g.off_v + node]) continue;
        int k = int(node / nxy);
        int64_t ij = node - k * nxy;
        int i = int(ij / ny), j = int(ij - (int64_t)i * ny);
        cx<R> u[8];
        cx<R> kcl = zero<R>();
        // x strips (k,i,j) [a end] and (k,i-1,j) [b end]
        for (int side = 0; side < 2; ++side) {
            int ii = i - side;
            if (ii < 0 || ii >= nx - 1) continue;
            int code = g.code_x[(int64_t)ii * ny + j];
            if (!((code >> k) & 1)) continue;
            for (int l = 0; l < S; ++l)
                u[l] = ((code >> l) & 1) ? rc[g.off_x + ((int64_t)l * (nx - 1) + ii) * ny + j] : zero<R>();
            cx<R> t = dinv_strip<R>(T, S, 0, code, k, u);
            if (side == 0) kcl += t; else kcl -= t;
        }
        for (int side = 0; side < 2; ++side) {
            int jj = j - side;
            if (jj < 0 || jj >= ny - 1) continue;
            int code = g.code_y[(int64_t)i * (ny - 1) + jj];
            if (!((code >> k) & 1)) continue;
            for (int l = 0; l < S; ++l)
                u[l] = ((code >> l) & 1) ? rc[g.off_y + ((int64_t)l * nx + i) * (ny - 1) + jj] : zero<R>();
            cx<R> t = dinv_strip<R>(T, S, 1, code, k, u);
            if (side == 0) kcl += t; else kcl -= t;
        }
        for (int p = 0; p < g.np; ++p) {
            int up = g.pair_layers[2 * p], lo = g.pair_layers[2 * p + 1];
            if (up != k && lo != k) continue;
            int64_t pos = g.off_c + p * nxy + ij;
            if (!g.mask[pos]) continue;
            cx<R> t = cvt<R>(T[g.tab_cap0 + p]) * rc[pos];
            if (up == k) kcl += t; else kcl -= t;
        }
        for (int e = g.node_br_ptr[node]; e < g.node_br_ptr[node + 1]; ++e) {
            int b = g.node_br_idx[e];
            int bb = (b > 0 ? b : -b) - 1;
            cx<R> t = cvt<R>(T[g.tab_br0 + bb]) * rc[g.off_b + bb];
            if (b > 0) kcl += t; else kcl -= t;
        }
        sd[(int64_t)col * S * nxy + node] = rc[g.off_v + node] - kcl;
    }
}

template <typename R>
void launch_pc_node(const Geo& g, const cx<R>* r, int64_t ld, cx<R>* sd, int ncol, const int* col_op, const c64* tab,
                    const int* col_list, cudaStream_t st) {
    int64_t items = (int64_t)g.S * g.nx * g.ny;
    int blocks = (int)std::min<int64_t>((items + 255) / 256, 4096);
    pc_node_kernel<R><<<dim3(blocks, ncol), 256, 0, st>>>(g, r, ld, sd, col_op, tab, col_list);
    GT_LAUNCH_CHECK();
}

// out = [D^-1 (r_1 + Ar y); y] over the whole dense vector (padding written zero)
template <typename R>
__global__ void pc_strip_kernel(Geo g, const cx<R>* __restrict__ r, int64_t ldr, const cx<R>* __restrict__ sd,
                                cx<R>* __restrict__ out, int64_t ldo, const int* __restrict__ col_op,
                                const c64* __restrict__ tab, const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int op = col_op ? col_op[col] : 0;
    const c64* T = tab + (int64_t)op * g.ntab;
    const cx<R>* rc = r + (int64_t)col * ldr;
    const cx<R>* yc = sd + (int64_t)col * g.S * g.nx * g.ny;
    const int S = g.S, nx = g.nx, ny = g.ny;
    const int64_t nxy = (int64_t)nx * ny;
    const int64_t nX = (int64_t)S * (nx - 1) * ny, nY = (int64_t)S * nx * (ny - 1);
    auto yv = [&](int64_t node) -> cx<R> { return yc[node]; };     // zero at nodes that are not kept
    for (int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pos < g.n; pos += (int64_t)gridDim.x * blockDim.x) {
        int seg = seg_of(g, pos, nX, nY);
        cx<R> o = zero<R>();
        if (seg >= 0 && g.mask[pos]) {
            if (seg == 0 || seg == 1) {
                int64_t q = pos - (seg == 0 ? g.off_x : g.off_y);
                int n0 = seg == 0 ? nx - 1 : nx, n1 = seg == 0 ? ny : ny - 1;
                int k = int(q / ((int64_t)n0 * n1));
                int64_t ij = q - (int64_t)k * n0 * n1;
                int i = int(ij / n1), j = int(ij - (int64_t)i * n1);
                int code = (seg == 0 ? g.code_x : g.code_y)[ij];
                int di = seg == 0, dj = seg == 1;
                int64_t segoff = seg == 0 ? g.off_x : g.off_y;
                cx<R> u[8];
                for (int l = 0; l < S; ++l) {
                    if ((code >> l) & 1) {
                        int64_t na = (int64_t)l * nxy + (int64_t)i * ny + j;
                        int64_t nb = na + (int64_t)di * ny + dj;
                        u[l] = rc[segoff + (int64_t)l * n0 * n1 + ij] + (yv(na) - yv(nb));
                    } else {
                        u[l] = zero<R>();
                    }
                }
                o = dinv_strip<R>(T, S, seg, code, k, u);
            } else if (seg == 2) {
                int64_t q = pos - g.off_c;
                int p = int(q / nxy);
                int64_t ij = q - (int64_t)p * nxy;
                int up = g.pair_layers[2 * p], lo = g.pair_layers[2 * p + 1];
                o = cvt<R>(T[g.tab_cap0 + p]) * (rc[pos] + (yv(up * nxy + ij) - yv(lo * nxy + ij)));
            } else if (seg == 3) {
                int b = int(pos - g.off_b);
                o = cvt<R>(T[g.tab_br0 + b]) * (rc[pos] + (yv(g.branch_nodes[2 * b]) - yv(g.branch_nodes[2 * b + 1])));
            } else {
                o = yv(pos - g.off_v);
            }
        }
        out[(int64_t)col * ldo + pos] = o;
    }
}

template <typename R>
void launch_pc_strip(const Geo& g, const cx<R>* r, int64_t ldr, const cx<R>* sd, cx<R>* out, int64_t ldo, int ncol,
                     const int* col_op, const c64* tab, const int* col_list, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((g.n + 255) / 256, 4096);
    pc_strip_kernel<R><<<dim3(blocks, ncol), 256, 0, st>>>(g, r, ldr, sd, out, ldo, col_op, tab, col_list);
    GT_LAUNCH_CHECK();
}

__global__ void scatter_kernel(const int64_t* __restrict__ c2d, int64_t ncomp, const c64* __restrict__ in, int64_t ldin,
                               c64* __restrict__ out, int64_t ldout) {
    const int col = blockIdx.y;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncomp; i += (int64_t)gridDim.x * blockDim.x)
        out[(int64_t)col * ldout + c2d[i]] = in[(int64_t)col * ldin + i];
}

__global__ void gather_kernel(const int64_t* __restrict__ c2d, int64_t ncomp, const c64* __restrict__ in, int64_t ldin,
                              c64* __restrict__ out, int64_t ldout) {
    const int col = blockIdx.y;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncomp; i += (int64_t)gridDim.x * blockDim.x)
        out[(int64_t)col * ldout + i] = in[(int64_t)col * ldin + c2d[i]];
}

void launch_scatter(const int64_t* c2d, int64_t ncomp, const c64* in, int64_t ldin, c64* out, int64_t ldout, int ncol,
                    cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((ncomp + 255) / 256, 2048);
    scatter_kernel<<<dim3(std::max(blocks, 1), ncol), 256, 0, st>>>(c2d, ncomp, in, ldin, out, ldout);
    GT_LAUNCH_CHECK();
}

void launch_gather(const int64_t* c2d, int64_t ncomp, const c64* in, int64_t ldin, c64* out, int64_t ldout, int ncol,
                   cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((ncomp + 255) / 256, 2048);
    gather_kernel<<<dim3(std::max(blocks, 1), ncol), 256, 0, st>>>(c2d, ncomp, in, ldin, out, ldout);
    GT_LAUNCH_CHECK();
}

template void launch_tail<float>(const Geo&, const c32*, const c32*, c32*, int64_t, int, const int*, const c64*, const c64*, int, const int*, cudaStream_t);
template void launch_tail<double>(const Geo&, const c64*, const c64*, c64*, int64_t, int, const int*, const c64*, const c64*, int, const int*, cudaStream_t);
template void launch_pc_node<float>(const Geo&, const c32*, int64_t, c32*, int, const int*, const c64*, const int*, cudaStream_t);
template void launch_pc_node<double>(const Geo&, const c64*, int64_t, c64*, int, const int*, const c64*, const int*, cudaStream_t);
template void launch_pc_strip<float>(const Geo&, const c32*, int64_t, const c32*, c32*, int64_t, int, const int*, const c64*, const int*, cudaStream_t);
template void launch_pc_strip<double>(const Geo&, const c64*, int64_t, const c64*, c64*, int64_t, int, const int*, const c64*, const int*, cudaStream_t);

}  // namespace gt
