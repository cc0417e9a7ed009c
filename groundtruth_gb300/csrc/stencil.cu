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

// grid rows per block of the stencil kernels (fewer, fuller blocks)
constexpr int RPB = 8;
constexpr int RPB_NODE = 2;     // pc_node's threads carry more work per row

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

}  // namespace

// blockIdx.y selects the part: 0 nodes (sheet k, row i), 1 capacitances (pair p, row i), 2 branches and the
// padding between segments.  The strips are written by the FFT pass.
template <typename R>
__global__ void __launch_bounds__(256) tail_kernel(Geo g, const cx<R>* __restrict__ x, const cx<R>* __restrict__ rhs,
                                                   cx<R>* __restrict__ out, int64_t ld, const int* __restrict__ col_op,
                                                   const c64* __restrict__ zcap, const c64* __restrict__ zbr, int mode,
                                                   const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const int op = col_op ? col_op[col] : 0;
    const int S = g.S, nx = g.nx, ny = g.ny, nxy = nx * ny;
    const cx<R>* xc = x + (int64_t)col * ld;
    const cx<R>* V = xc + g.off_v;
    const cx<R>* bc = rhs ? rhs + (int64_t)col * ld : nullptr;
    cx<R>* oc = out + (int64_t)col * ld;
    const int part = blockIdx.y;
    auto put = [&](int64_t pos, cx<R> y) { oc[pos] = mode == 1 ? bc[pos] - y : y; };
    if (part == 0) for (int bx = blockIdx.x * RPB; bx < blockIdx.x * RPB + RPB; ++bx) {
        // node (KCL) rows: I_x(k,i,j) - I_x(k,i-1,j) + I_y(k,i,j) - I_y(k,i,j-1) + caps + branches, the strips of
        // every sheet on layer k (a split layer's two faces)
        const int k = bx / nx, i = bx - k * nx;
        if (k >= g.NL) break;
        for (int j = threadIdx.x; j < ny; j += blockDim.x) {
            const int ij = i * ny + j, node = k * nxy + ij;
            const int64_t pos = g.off_v + node;
            if (!g.mask[pos]) {
                oc[pos] = zero<R>();
                continue;
            }
            cx<R> s = zero<R>();
            for (int sh = g.NL == S ? k : 0; sh < (g.NL == S ? k + 1 : S); ++sh) {
                if (g.sheet_layer[sh] != k) continue;
                const cx<R>* X = xc + g.off_x + (int64_t)sh * (nx - 1) * ny;
                const cx<R>* Y = xc + g.off_y + (int64_t)sh * nx * (ny - 1);
                if (i < nx - 1) s += X[i * ny + j];
                if (i > 0) s -= X[(i - 1) * ny + j];
                if (j < ny - 1) s += Y[i * (ny - 1) + j];
                if (j > 0) s -= Y[i * (ny - 1) + j - 1];
            }
            for (int p = 0; p < g.np; ++p) {
                const int u = g.pair_layers[2 * p], l = g.pair_layers[2 * p + 1];
                if (u == k) s += xc[g.off_c + (int64_t)p * nxy + ij];
                if (l == k) s -= xc[g.off_c + (int64_t)p * nxy + ij];
            }
            for (int e = g.node_br_ptr[node]; e < g.node_br_ptr[node + 1]; ++e) {
                const int b = g.node_br_idx[e];
                if (b > 0) s += xc[g.off_b + b - 1];
                else s -= xc[g.off_b - b - 1];
            }
            put(pos, s);
        }
    } else if (part == 1) for (int bx = blockIdx.x * RPB; bx < blockIdx.x * RPB + RPB; ++bx) {
        // capacitance rows: z_cap I_c - (V[upper] - V[lower])
        const int p = bx / nx, i = bx - p * nx;
        if (p >= g.np) break;
        const int u = g.pair_layers[2 * p], l = g.pair_layers[2 * p + 1];
        const cx<R> zc = cvt<R>(zcap[(int64_t)op * g.np + p]);
        for (int j = threadIdx.x; j < ny; j += blockDim.x) {
            const int ij = i * ny + j;
            const int64_t pos = g.off_c + (int64_t)p * nxy + ij;
            if (!g.mask[pos]) {
                oc[pos] = zero<R>();
                continue;
            }
            // a partly covered cell: its capacitance is the share's, its impedance z_cap / share
            const cx<R> z = g.cap_fill ? R(1.0 / g.cap_fill[(int64_t)p * nxy + ij]) * zc : zc;
            put(pos, z * xc[pos] - (V[u * nxy + ij] - V[l * nxy + ij]));
        }
    } else {
        // branch rows z_br I_b - (V[a] - V[b]); padding zero
        const int64_t nX = (int64_t)S * (nx - 1) * ny, nY = (int64_t)S * nx * (ny - 1);
        const int64_t gap[5][2] = {{g.off_x + nX, g.off_y}, {g.off_y + nY, g.off_c},
                                   {g.off_c + (int64_t)g.np * nxy, g.off_b}, {g.off_b + g.nbr, g.off_v},
                                   {g.off_v + (int64_t)g.NL * nxy, g.n}};
        const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
        for (int b = tid; b < g.nbr; b += nth) {
            const int64_t pos = g.off_b + b;
            if (!g.mask[pos]) {
                oc[pos] = zero<R>();
                continue;
            }
            put(pos, cvt<R>(zbr[(int64_t)op * g.nbr + b]) * xc[pos] - (V[g.branch_nodes[2 * b]] - V[g.branch_nodes[2 * b + 1]]));
        }
        for (int q = 0; q < 5; ++q)
            for (int64_t pos = gap[q][0] + tid; pos < gap[q][1]; pos += nth) oc[pos] = zero<R>();
    }
}

template <typename R>
void launch_tail(const Geo& g, const cx<R>* x, const cx<R>* rhs, cx<R>* out, int64_t ld, int ncol, const int* col_op,
                 const c64* zcap, const c64* zbr, int mode, const int* col_list, cudaStream_t st) {
    const dim3 grid(std::max(ceil_div((int64_t)g.nx * std::max(g.np, g.S), RPB), 1), 3, ncol);
    tail_kernel<R><<<grid, 256, 0, st>>>(g, x, rhs, out, ld, col_op, zcap, zbr, mode, col_list);
    GT_LAUNCH_CHECK();
}

// D^-1 of the strips at one grid position applied to the S-vector u (sheets present: code); out[k] for the
// sheets k present.  B: the position's S x S block (by its sheet code from the orientation's table, or the
// position's own where its strips are not all full width).
constexpr int SHEETS_MAX = 8;
template <typename R, int MAXS>
__device__ __forceinline__ void dinv_apply(const cx<R>* __restrict__ B, int S, int code, const cx<R>* u, cx<R>* out) {
#pragma unroll
    for (int k = 0; k < MAXS; ++k) {
        out[k] = zero<R>();
        if (k >= S || !((code >> k) & 1)) continue;
#pragma unroll
        for (int l = 0; l < MAXS; ++l)
            if (l < S && ((code >> l) & 1)) out[k] += B[k * S + l] * u[l];
    }
}

// s = r_V - Ar^T D^-1 r_1 at every kept node, written in factor order (sf[col][nfac], through perm).  One block per grid row i and
// column; a thread takes the S nodes of one position (i, j): the strips on either side of it are loaded once
// for all sheets.
template <typename R, int MAXS>
__global__ void __launch_bounds__(256) pc_node_kernel(Geo g, const cx<R>* __restrict__ r, int64_t ld, cx<R>* __restrict__ sd,
                                                      const int* __restrict__ col_op, const cx<R>* __restrict__ tab,
                                                      const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int op = col_op ? col_op[col] : 0;
    const int S = g.S, nx = g.nx, ny = g.ny, nxy = nx * ny, NC = 1 << S;
    const cx<R>* T = tab + (int64_t)op * g.ntab;
    const cx<R>* rc = r + (int64_t)col * ld;
    const cx<R>* X = rc + g.off_x;
    const cx<R>* Y = rc + g.off_y;
    cx<R>* sc = sd + (int64_t)col * g.nfac;
    for (int i = blockIdx.x * RPB_NODE; i < min(nx, blockIdx.x * RPB_NODE + RPB_NODE); ++i)
    for (int j = threadIdx.x; j < ny; j += blockDim.x) {
        const int ij = i * ny + j;
        cx<R> kcl[MAXS], u[4][MAXS], t[MAXS];
        int code[4], pq[4];
#pragma unroll
        for (int k = 0; k < MAXS; ++k) kcl[k] = zero<R>();
        // x strips (., i, j) [their a end] and (., i-1, j) [b end]; y strips (., i, j) and (., i, j-1):
        // all codes, then all strip loads, then the products
#pragma unroll
        for (int side = 0; side < 4; ++side) {
            const bool xo = side < 2;
            const int ii = xo ? i - side : i, jj = xo ? j : j - (side - 2);
            const bool ok = xo ? (ii >= 0 && ii < nx - 1) : (jj >= 0 && jj < ny - 1);
            pq[side] = xo ? ii * ny + jj : ii * (ny - 1) + jj;
            code[side] = ok ? (xo ? g.code_x[pq[side]] : g.code_y[pq[side]]) : 0;
        }
#pragma unroll
        for (int side = 0; side < 4; ++side) {
            const bool xo = side < 2;
            const int lstride = xo ? (nx - 1) * ny : nx * (ny - 1);
            const cx<R>* base = xo ? X : Y;
#pragma unroll
            for (int l = 0; l < MAXS; ++l)
                u[side][l] = (l < S && ((code[side] >> l) & 1)) ? base[(int64_t)l * lstride + pq[side]] : zero<R>();
        }
#pragma unroll
        for (int side = 0; side < 4; ++side) {
            if (!code[side]) continue;
            const int* ovr = side < 2 ? g.ovr_x : g.ovr_y;
            const int ob = ovr ? ovr[pq[side]] : -1;
            dinv_apply<R, MAXS>(ob >= 0 ? T + g.tab_ovr0 + (int64_t)ob * S * S
                                        : T + ((int64_t)(side < 2 ? 0 : 1) * NC + code[side]) * S * S,
                                S, code[side], u[side], t);
            const bool plus = (side & 1) == 0;
            if (g.NL == S) {
#pragma unroll
                for (int k = 0; k < MAXS; ++k)
                    if (k < S) kcl[k] = plus ? kcl[k] + t[k] : kcl[k] - t[k];
            } else {
#pragma unroll
                for (int k = 0; k < MAXS; ++k) {
                    if (k >= S) continue;
                    const int L = g.sheet_layer[k];      // a face sheet's strips join its layer's nodes
#pragma unroll
                    for (int m = 0; m < MAXS; ++m)
                        if (m == L) kcl[m] = plus ? kcl[m] + t[k] : kcl[m] - t[k];
                }
            }
        }
        for (int p = 0; p < g.np; ++p) {
            const int up = g.pair_layers[2 * p], lo = g.pair_layers[2 * p + 1];
            const int64_t pos = g.off_c + (int64_t)p * nxy + ij;
            if (!g.mask[pos]) continue;
            cx<R> v = T[g.tab_cap0 + p] * rc[pos];
            if (g.cap_fill) v = R(g.cap_fill[(int64_t)p * nxy + ij]) * v;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) {
                if (k == up) kcl[k] += v;
                if (k == lo) kcl[k] -= v;
            }
        }
#pragma unroll
        for (int k = 0; k < MAXS; ++k) {
            if (k >= g.NL) break;
            const int node = k * nxy + ij;
            if (!g.mask[g.off_v + node]) continue;
            cx<R> acc = kcl[k];
            for (int e = g.node_br_ptr[node]; e < g.node_br_ptr[node + 1]; ++e) {
                const int bq = g.node_br_idx[e];
                const int bb = (bq > 0 ? bq : -bq) - 1;
                const cx<R> v = T[g.tab_br0 + bb] * rc[g.off_b + bb];
                acc = bq > 0 ? acc + v : acc - v;
            }
            sc[g.perm[node]] = rc[g.off_v + node] - acc;
        }
    }
}

template <typename R>
void launch_pc_node(const Geo& g, const cx<R>* r, int64_t ld, cx<R>* sd, int ncol, const int* col_op, const cx<R>* tab,
                    const int* col_list, cudaStream_t st) {
    if (g.S > SHEETS_MAX) throw CudaError{cudaErrorInvalidValue, "more sheets than the stencil kernels take"};
    const dim3 grid(ceil_div(g.nx, RPB_NODE), ncol);
    if (g.S <= 2) pc_node_kernel<R, 2><<<grid, 256, 0, st>>>(g, r, ld, sd, col_op, tab, col_list);
    else if (g.S <= 4) pc_node_kernel<R, 4><<<grid, 256, 0, st>>>(g, r, ld, sd, col_op, tab, col_list);
    else pc_node_kernel<R, 8><<<grid, 256, 0, st>>>(g, r, ld, sd, col_op, tab, col_list);
    GT_LAUNCH_CHECK();
}

// out = [D^-1 (r_1 + Ar y); y] over the whole dense vector (padding written zero).  blockIdx.y selects the
// part: 0 x strips (block per row i), 1 y strips (row i), 2 capacitances (pair p, row i), 3 nodes (sheet k,
// row i), 4 branches and the padding between segments.  A strip thread takes all sheets of its position.
template <typename R, int MAXS>
__global__ void __launch_bounds__(256) pc_strip_kernel(Geo g, const cx<R>* __restrict__ r, int64_t ldr,
                                                       const cx<R>* __restrict__ sd, cx<R>* __restrict__ out, int64_t ldo,
                                                       const int* __restrict__ col_op, const cx<R>* __restrict__ tab,
                                                       const int* __restrict__ col_list) {
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const int op = col_op ? col_op[col] : 0;
    const int S = g.S, nx = g.nx, ny = g.ny, nxy = nx * ny, NC = 1 << S;
    const cx<R>* T = tab + (int64_t)op * g.ntab;
    const cx<R>* rc = r + (int64_t)col * ldr;
    const cx<R>* yc = sd + (int64_t)col * g.NL * nxy;    // zero at nodes that are not kept
    cx<R>* oc = out + (int64_t)col * ldo;
    const int part = blockIdx.y;
    if (part <= 1) for (int bx = blockIdx.x * RPB; bx < blockIdx.x * RPB + RPB; ++bx) {
        const bool xo = part == 0;
        const int i = bx;
        if (i >= (xo ? nx - 1 : nx)) break;
        const int n1 = xo ? ny : ny - 1, lstride = (xo ? nx - 1 : nx) * n1;
        const int64_t seg = xo ? g.off_x : g.off_y;
        const uint8_t* codes = xo ? g.code_x : g.code_y;
        const int dn = xo ? ny : 1;                          // node b = node a + dn
        for (int j = threadIdx.x; j < n1; j += blockDim.x) {
            const int pq = i * n1 + j, na = i * ny + j;
            const int code = codes[pq];
            cx<R> u[MAXS], t[MAXS];
#pragma unroll
            for (int l = 0; l < MAXS; ++l)
                u[l] = (l < S && ((code >> l) & 1))
                           ? rc[seg + (int64_t)l * lstride + pq] +
                                 (yc[g.sheet_layer[l] * nxy + na] - yc[g.sheet_layer[l] * nxy + na + dn])
                           : zero<R>();
            const int* ovr = xo ? g.ovr_x : g.ovr_y;
            const int ob = ovr ? ovr[pq] : -1;
            dinv_apply<R, MAXS>(ob >= 0 ? T + g.tab_ovr0 + (int64_t)ob * S * S
                                        : T + ((int64_t)(xo ? 0 : 1) * NC + code) * S * S,
                                S, code, u, t);
#pragma unroll
            for (int k = 0; k < MAXS; ++k)
                if (k < S) oc[seg + (int64_t)k * lstride + pq] = t[k];      // zero where the strip is absent
        }
    } else if (part == 2) for (int bx = blockIdx.x * RPB; bx < blockIdx.x * RPB + RPB; ++bx) {
        const int p = bx / nx, i = bx - p * nx;
        if (p >= g.np) break;
        const int up = g.pair_layers[2 * p], lo = g.pair_layers[2 * p + 1];
        const cx<R> zc = T[g.tab_cap0 + p];
        for (int j = threadIdx.x; j < ny; j += blockDim.x) {
            const int ij = i * ny + j;
            const int64_t pos = g.off_c + (int64_t)p * nxy + ij;
            const cx<R> y = g.cap_fill ? R(g.cap_fill[(int64_t)p * nxy + ij]) * zc : zc;
            oc[pos] = g.mask[pos] ? y * (rc[pos] + (yc[up * nxy + ij] - yc[lo * nxy + ij])) : zero<R>();
        }
    } else if (part == 3) for (int bx = blockIdx.x * RPB; bx < blockIdx.x * RPB + RPB; ++bx) {
        const int k = bx / nx, i = bx - k * nx;
        if (k >= g.NL) break;
        for (int j = threadIdx.x; j < ny; j += blockDim.x) {
            const int node = k * nxy + i * ny + j;
            oc[g.off_v + node] = yc[node];
        }
    } else {
        // branches, then the padding: [off_x + nX, off_y), [off_y + nY, off_c), [off_c + np nxy, off_b),
        // [off_b + nbr, off_v), [off_v + S nxy, n)
        const int64_t nX = (int64_t)S * (nx - 1) * ny, nY = (int64_t)S * nx * (ny - 1);
        const int64_t gap[5][2] = {{g.off_x + nX, g.off_y}, {g.off_y + nY, g.off_c},
                                   {g.off_c + (int64_t)g.np * nxy, g.off_b}, {g.off_b + g.nbr, g.off_v},
                                   {g.off_v + (int64_t)g.NL * nxy, g.n}};
        const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
        for (int b = tid; b < g.nbr; b += nth) {
            const int64_t pos = g.off_b + b;
            oc[pos] = g.mask[pos] ? T[g.tab_br0 + b] * (rc[pos] + (yc[g.branch_nodes[2 * b]] - yc[g.branch_nodes[2 * b + 1]]))
                                  : zero<R>();
        }
        for (int q = 0; q < 5; ++q)
            for (int64_t pos = gap[q][0] + tid; pos < gap[q][1]; pos += nth) oc[pos] = zero<R>();
    }
}

template <typename R>
void launch_pc_strip(const Geo& g, const cx<R>* r, int64_t ldr, const cx<R>* sd, cx<R>* out, int64_t ldo, int ncol,
                     const int* col_op, const cx<R>* tab, const int* col_list, cudaStream_t st) {
    if (g.S > SHEETS_MAX) throw CudaError{cudaErrorInvalidValue, "more sheets than the stencil kernels take"};
    const dim3 grid(std::max(ceil_div((int64_t)g.nx * std::max(g.np, g.S), RPB), 1), 5, ncol);
    if (g.S <= 2) pc_strip_kernel<R, 2><<<grid, 256, 0, st>>>(g, r, ldr, sd, out, ldo, col_op, tab, col_list);
    else if (g.S <= 4) pc_strip_kernel<R, 4><<<grid, 256, 0, st>>>(g, r, ldr, sd, out, ldo, col_op, tab, col_list);
    else pc_strip_kernel<R, 8><<<grid, 256, 0, st>>>(g, r, ldr, sd, out, ldo, col_op, tab, col_list);
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
template void launch_pc_node<float>(const Geo&, const c32*, int64_t, c32*, int, const int*, const c32*, const int*, cudaStream_t);
template void launch_pc_node<double>(const Geo&, const c64*, int64_t, c64*, int, const int*, const c64*, const int*, cudaStream_t);
template void launch_pc_strip<float>(const Geo&, const c32*, int64_t, const c32*, c32*, int64_t, int, const int*, const c32*, const int*, cudaStream_t);
template void launch_pc_strip<double>(const Geo&, const c64*, int64_t, const c64*, c64*, int64_t, int, const int*, const c64*, const int*, cudaStream_t);

}  // namespace gt
