// The Schur complement S = Ar^T D^-1 Ar of the preconditioner (peec.py:2379), its factorisation and its
// solves, on the device.  The reference factorises S with SuperLU (peec.py:2423, MMD ordering) and applies
// it with SuperLU's triangular solves every iteration (peec.py:3071, on the CPU also in gpu.py:566-573);
// here S (complex symmetric) is factorised as L D L^T by the multifrontal method along a nested-dissection
// elimination tree, one batched launch per tree level for all fronts of the level and all frequencies:
//
//   assemble   S values = sum of coef * admittance table entries (a fixed sparse map, per frequency)
//   front      F = own columns of S + children's update matrices (extend-add)
//   eliminate  the own columns of F by rank-1 updates; L and D go to the front's panel (nf x nown,
//              column-major, D on its diagonal), the trailing block is the front's update matrix
//
// FP64 throughout (a floating plane coupled only by plane-pair capacitance makes S nearly singular in one
// mode whose pivot is ~1e-10 of the strips' admittance); the panels are also rounded to FP32 for the
// inner iterations' solves.  The solves run level by level: leaves up for L z = s (each front gathers its
// children's update vectors, eliminates its own rows and passes its boundary rows up), z /= D, root down
// for L^T y = z (each front reads its ancestors' finished y).
#include "kernels.h"

namespace gt {

// Complex multiply-accumulate as four explicit FMAs (acc += a u; cfms: acc -= a u): written out, the
// product and the sum round as separate operations (six instructions instead of four on the FP64 pipe).
__device__ __forceinline__ void cfma(c32& acc, c32 a, c32 u) {
    acc.re = __fmaf_rn(a.re, u.re, acc.re);
    acc.re = __fmaf_rn(-a.im, u.im, acc.re);
    acc.im = __fmaf_rn(a.re, u.im, acc.im);
    acc.im = __fmaf_rn(a.im, u.re, acc.im);
}
__device__ __forceinline__ void cfma(c64& acc, c64 a, c64 u) {
    acc.re = __fma_rn(a.re, u.re, acc.re);
    acc.re = __fma_rn(-a.im, u.im, acc.re);
    acc.im = __fma_rn(a.re, u.im, acc.im);
    acc.im = __fma_rn(a.im, u.re, acc.im);
}
__device__ __forceinline__ void cfms(c64& acc, c64 a, c64 u) {
    acc.re = __fma_rn(-a.re, u.re, acc.re);
    acc.re = __fma_rn(a.im, u.im, acc.re);
    acc.im = __fma_rn(-a.re, u.im, acc.im);
    acc.im = __fma_rn(-a.im, u.re, acc.im);
}

__global__ void assemble_s_kernel(const int64_t* __restrict__ ptr, const int* __restrict__ tab_idx,
                                  const double* __restrict__ coef, int64_t nsv, const c64* __restrict__ table, int ntab,
                                  c64* __restrict__ svals) {
    const int op = blockIdx.y;
    const c64* T = table + (int64_t)op * ntab;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nsv; e += (int64_t)gridDim.x * blockDim.x) {
        c64 acc = zero<double>();
        for (int64_t q = ptr[e]; q < ptr[e + 1]; ++q) acc += coef[q] * T[tab_idx[q]];
        svals[(int64_t)op * nsv + e] = acc;
    }
}

void launch_assemble_s(const int64_t* ptr, const int* tab_idx, const double* coef, int64_t nsv, const c64* table,
                       int ntab, c64* svals, int nops, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((nsv + 255) / 256, 2048);
    assemble_s_kernel<<<dim3(std::max(blocks, 1), nops), 256, 0, st>>>(ptr, tab_idx, coef, nsv, table, ntab, svals);
    GT_LAUNCH_CHECK();
}

// Front entry (r, c), r >= c: own columns in the panel, the trailing block in the update matrix.
struct FrontView {
    c64* panel;
    c64* upd;
    int nf, nown, nbnd;
    __device__ __forceinline__ c64& at(int r, int c) const {
        return c < nown ? panel[(int64_t)c * nf + r] : upd[(int64_t)(c - nown) * nbnd + (r - nown)];
    }
};

// A front's entries before elimination: the own columns of S and the children's update matrices, one child
// at a time (their boundaries overlap).  The panels start zeroed (one memset before the first level); the
// update matrix's slot is shared with matrices of other levels (its last owner's was assembled into its
// parent at an earlier level) and is cleared here.
__device__ void assemble_front(const Fronts& F, int f, int op, const c64* __restrict__ svals, const FrontView& Fv,
                               const c64* __restrict__ upd) {
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int64_t q = tid; q < (int64_t)Fv.nbnd * Fv.nbnd; q += nth) Fv.upd[q] = zero<double>();
    __syncthreads();
    const c64* sv = svals + (int64_t)op * F.nsv;
    for (int64_t e = F.ent_ptr[f] + tid; e < F.ent_ptr[f + 1]; e += nth) Fv.at(F.ent_row[e], F.ent_col[e]) += sv[F.ent_s[e]];
    __syncthreads();
    for (int64_t ci = F.child_ptr[f]; ci < F.child_ptr[f + 1]; ++ci) {
        const int c = (int)F.child_idx[ci];
        const int nb = (int)F.nbnd[c];
        const int64_t* map = F.cmap_idx + F.cmap_ptr[ci];
        const c64* U = upd + (int64_t)op * F.upd_total + F.upd_off[c];
        for (int64_t q = tid; q < (int64_t)nb * nb; q += nth) {
            int j = int(q / nb), i = int(q - (int64_t)j * nb);
            if (i >= j) Fv.at((int)map[i], (int)map[j]) += U[q];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ FrontView front_view(const Fronts& F, int f, int op, c64* panel, c64* upd) {
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f];
    return FrontView{panel + (int64_t)op * F.panel_total + F.panel_off[f], upd + (int64_t)op * F.upd_total + F.upd_off[f],
                     nown + nbnd, nown, nbnd};
}

__device__ __forceinline__ c64 pivot_inverse(c64 d, int* status) {
    const double dd = d.re * d.re + d.im * d.im;
    if (!(dd > 1e-300) || !isfinite(dd)) {
        atomicOr(status, 1);
        d = mk<double>(1e-150, 0.0);
    }
    return cdiv(mk<double>(1.0, 0.0), d);
}

// Small fronts: one CTA per (front, operator) assembles the front and eliminates its own columns by rank-1
// updates in place.
__global__ void factor_level_kernel(Fronts F, const int64_t* __restrict__ front_list, const c64* __restrict__ svals,
                                    c64* __restrict__ panel, c64* __restrict__ upd, int* __restrict__ status) {
    const int f = (int)front_list[blockIdx.x];
    const int op = blockIdx.y;
    const FrontView Fv = front_view(F, f, op, panel, upd);
    const int nf = Fv.nf, nown = Fv.nown;
    assemble_front(F, f, op, svals, Fv, upd);
    const int tid = threadIdx.x, nth = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
    for (int k = 0; k < nown; ++k) {
        const c64 d = Fv.panel[(int64_t)k * nf + k];
        const double dd = d.re * d.re + d.im * d.im;
        if ((!(dd > 1e-300) || !isfinite(dd)) && tid == 0) atomicOr(status, 1);
        const c64 dinv = (!(dd > 1e-300) || !isfinite(dd)) ? cdiv(mk<double>(1.0, 0.0), mk<double>(1e-150, 0.0))
                                                            : cdiv(mk<double>(1.0, 0.0), d);
        const c64* colk = Fv.panel + (int64_t)k * nf;
        for (int j = k + 1 + warp; j < nf; j += nwarp) {
            const c64 ljd = colk[j] * dinv;
            for (int i = j + lane; i < nf; i += 32) {
                c64& v = Fv.at(i, j);
                cfms(v, colk[i], ljd);
            }
        }
        __syncthreads();
        for (int i = k + 1 + tid; i < nf; i += nth) Fv.panel[(int64_t)k * nf + i] = Fv.panel[(int64_t)k * nf + i] * dinv;
        __syncthreads();
    }
}

void launch_factor_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const c64* svals,
                         c64* panel, c64* upd, int nops, int* status, cudaStream_t st) {
    int threads = max_nf >= 256 ? 512 : 256;
    factor_level_kernel<<<dim3(nf_level, nops), threads, 0, st>>>(F, front_list, svals, panel, upd, status);
    GT_LAUNCH_CHECK();
}

// Large fronts: blocked elimination, FB own columns per step, every step over many CTAs (the top of the tree
// has a few fronts per operator, and an SM's FP64 rate is 1/152 of the GPU's):
//   diag   one warp per (front, operator) factors the FB x FB diagonal block in shared memory (lane = row)
//   rows   L21 = A21 L11^-T D^-1 for the rows below it, one thread per row, 128 rows per CTA
//   trail  A22 -= L21 D L21^T over 64 x 64 tiles of the trailing lower triangle, one tile per CTA
// The arithmetic is the rank-1 kernel's, the updates of a block summed before they are subtracted.
constexpr int FB = 32, FT = 64, ROWS_CTA = 128;

__global__ void assemble_fronts_kernel(Fronts F, const int64_t* __restrict__ front_list, const c64* __restrict__ svals,
                                       c64* __restrict__ panel, c64* __restrict__ upd) {
    const int f = (int)front_list[blockIdx.x];
    const int op = blockIdx.y;
    assemble_front(F, f, op, svals, front_view(F, f, op, panel, upd), upd);
}

__global__ void __launch_bounds__(32) tiled_diag_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                        c64* __restrict__ panel, c64* __restrict__ upd,
                                                        int* __restrict__ status) {
    __shared__ c64 a[FB][FB + 1];
    const int f = (int)front_list[blockIdx.x];
    const FrontView Fv = front_view(F, f, blockIdx.y, panel, upd);
    const int nb = min(FB, Fv.nown - kb);
    if (nb <= 0) return;
    const int i = threadIdx.x;
    for (int j = 0; j < nb; ++j)
        a[i][j] = (i < nb && j <= i) ? Fv.panel[(int64_t)(kb + j) * Fv.nf + kb + i] : zero<double>();
    __syncwarp();
    for (int k = 0; k < nb; ++k) {
        const c64 dinv = pivot_inverse(a[k][k], status);
        const c64 lik = a[i][k];
        for (int j = k + 1; j <= i && i < nb; ++j) a[i][j] -= lik * (a[j][k] * dinv);
        __syncwarp();
        if (i > k && i < nb) a[i][k] = lik * dinv;
        __syncwarp();
    }
    if (i < nb)
        for (int j = 0; j <= i; ++j) Fv.panel[(int64_t)(kb + j) * Fv.nf + kb + i] = a[i][j];
}

__global__ void __launch_bounds__(ROWS_CTA) tiled_rows_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                              c64* __restrict__ panel, c64* __restrict__ upd) {
    __shared__ c64 l11[FB][FB];
    __shared__ c64 dv[FB];
    const int f = (int)front_list[blockIdx.y];
    const FrontView Fv = front_view(F, f, blockIdx.z, panel, upd);
    const int nb = min(FB, Fv.nown - kb);
    if (nb <= 0) return;
    const int i = kb + nb + blockIdx.x * ROWS_CTA + threadIdx.x;
    if (kb + nb + blockIdx.x * ROWS_CTA >= Fv.nf) return;             // the whole CTA is past the front
    for (int q = threadIdx.x; q < FB * FB; q += ROWS_CTA) {
        const int r = q / FB, c = q - r * FB;
        l11[r][c] = (r < nb && c < r) ? Fv.panel[(int64_t)(kb + c) * Fv.nf + kb + r] : zero<double>();
        if (r == c) dv[r] = r < nb ? Fv.panel[(int64_t)(kb + r) * Fv.nf + kb + r] : mk<double>(1.0, 0.0);
    }
    __syncthreads();
    if (i >= Fv.nf) return;
    c64 w[FB];                                                          // w = l D: the row's updates to come
#pragma unroll
    for (int k = 0; k < FB; ++k) {
        if (k < nb) {
            c64 t = Fv.panel[(int64_t)(kb + k) * Fv.nf + i];
#pragma unroll
            for (int m = 0; m < k; ++m) cfms(t, w[m], l11[k][m]);
            w[k] = t;
        }
    }
#pragma unroll
    for (int k = 0; k < FB; ++k)
        if (k < nb) Fv.panel[(int64_t)(kb + k) * Fv.nf + i] = cdiv(w[k], dv[k]);
}

// tile t of the lower triangle of a T x T tile grid: (bi, bj), bj <= bi
__device__ __forceinline__ void lower_tile(int t, int& bi, int& bj) {
    int b = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((int64_t)b * (b + 1) / 2 > t) --b;
    while ((int64_t)(b + 1) * (b + 2) / 2 <= t) ++b;
    bi = b;
    bj = t - b * (b + 1) / 2;
}

constexpr size_t TRAIL_SMEM = 2 * (size_t)FB * FT * sizeof(c64);

__global__ void __launch_bounds__(256) tiled_trail_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                          c64* __restrict__ panel, c64* __restrict__ upd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c64* As = reinterpret_cast<c64*>(smem_raw);          // [m][FT]: L(i0 + r, kb + m)
    c64* Bs = As + FB * FT;                              // [m][FT]: L(j0 + c, kb + m) d_m
    const int f = (int)front_list[blockIdx.y];
    const FrontView Fv = front_view(F, f, blockIdx.z, panel, upd);
    const int nb = min(FB, Fv.nown - kb);
    if (nb <= 0) return;
    const int t0 = kb + nb, n2 = Fv.nf - t0;
    const int T = (n2 + FT - 1) / FT;
    if ((int64_t)blockIdx.x >= (int64_t)T * (T + 1) / 2) return;
    int bi, bj;
    lower_tile(blockIdx.x, bi, bj);
    const int i0 = t0 + bi * FT, j0 = t0 + bj * FT;
    for (int q = threadIdx.x; q < FB * FT; q += 256) {
        const int m = q / FT, r = q - m * FT;
        c64 a = zero<double>(), b = zero<double>();
        if (m < nb) {
            const c64* col = Fv.panel + (int64_t)(kb + m) * Fv.nf;
            if (i0 + r < Fv.nf) a = col[i0 + r];
            if (j0 + r < Fv.nf) b = col[j0 + r] * col[kb + m];
        }
        As[q] = a;
        Bs[q] = b;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    c64 acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = zero<double>();
    for (int m = 0; m < nb; ++m) {
        c64 a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = As[m * FT + tx + 16 * r];
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = Bs[m * FT + ty + 16 * c];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) cfma(acc[r][c], a[r], b[c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int j = j0 + ty + 16 * c;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = i0 + tx + 16 * r;
            if (i < Fv.nf && j <= i) Fv.at(i, j) -= acc[r][c];
        }
    }
}

void launch_factor_tiled(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                         const c64* svals, c64* panel, c64* upd, int nops, int* status, cudaStream_t st) {
    assemble_fronts_kernel<<<dim3(nf_level, nops), 512, 0, st>>>(F, front_list, svals, panel, upd);
    GT_LAUNCH_CHECK();
    raise_smem((const void*)tiled_trail_kernel, TRAIL_SMEM);
    for (int kb = 0; kb < max_nown; kb += FB) {
        tiled_diag_kernel<<<dim3(nf_level, nops), 32, 0, st>>>(F, front_list, kb, panel, upd, status);
        GT_LAUNCH_CHECK();
        const int below = max_nf - kb - 1;              // rows below the block (at least this front's nb of them)
        if (below <= 0) continue;
        tiled_rows_kernel<<<dim3(ceil_div(below, ROWS_CTA), nf_level, nops), ROWS_CTA, 0, st>>>(F, front_list, kb, panel,
                                                                                                 upd);
        GT_LAUNCH_CHECK();
        const int T = ceil_div(below, FT);
        tiled_trail_kernel<<<dim3((unsigned)((int64_t)T * (T + 1) / 2), nf_level, nops), 256, TRAIL_SMEM, st>>>(
            F, front_list, kb, panel, upd);
        GT_LAUNCH_CHECK();
    }
}

// Selective inversion: the inverse X of each front's own block (unit lower triangular; D on the diagonal
// kept as is), FP64.  Rows are independent: X[i, k] = -(L[i, k] + sum_{k < m < i} X[i, m] L[m, k]) for k
// descending.  X[i, k] is written to the unused upper triangle, transposed (position (k, i)), so the factor's
// lower triangle stays intact while other rows read it; panel_convert moves X into place.  One thread per
// row, rows of large fronts over several blocks, no barriers.
constexpr int INV_ROWS = 128;
__global__ void __launch_bounds__(INV_ROWS) invert_own_kernel(Fronts F, c64* __restrict__ panel, int nchunk, int tiled_nf) {
    const int f = blockIdx.x / nchunk, chunk = blockIdx.x - f * nchunk, op = blockIdx.y;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    if (chunk * INV_ROWS >= nown || nf >= tiled_nf) return;      // large fronts: the blocked inversion
    const int i = chunk * INV_ROWS + threadIdx.x;
    c64* L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int kmax = min(nown, chunk * INV_ROWS + INV_ROWS) - 2;   // the block's largest row - 1
    c64* Xi = L + (int64_t)min(i, nown - 1) * nf;                   // X[i, m] at Xi[m], m < i
    for (int k = kmax; k >= 0; --k) {
        if (k >= i || i >= nown) continue;
        c64 acc = L[(int64_t)k * nf + i];
        const c64* Lk = L + (int64_t)k * nf;
        for (int m = k + 1; m < i; ++m) cfma(acc, Xi[m], Lk[m]);
        Xi[k] = mk<double>(-acc.re, -acc.im);
    }
}

void launch_invert_own(const Fronts& F, c64* panel, int max_nown, int nops, int tiled_nf, cudaStream_t st) {
    const int nchunk = std::max(1, ceil_div(max_nown, INV_ROWS));
    invert_own_kernel<<<dim3(F.nfront * nchunk, nops), INV_ROWS, 0, st>>>(F, panel, nchunk, tiled_nf);
    GT_LAUNCH_CHECK();
}

// Boundary rows of each front replaced by M = -L_bnd Linv_own (in place, FP64; after invert_own_kernel,
// Linv read from the upper triangle).  Every boundary row is independent: M[j, k] = -(L[j, k] + sum_{m > k} L[j, m] Linv[m, k]) for k ascending reads only entries
// m > k of its own row, which are still the factor's.  One thread per row (rows of a warp consecutive, so
// the row loads coalesce and the Linv loads broadcast); the rows of large fronts spread over many blocks.
constexpr int BND_ROWS = 128;
__global__ void __launch_bounds__(BND_ROWS) bnd_inv_kernel(Fronts F, c64* __restrict__ panel, int nchunk, int tiled_nf) {
    const int f = blockIdx.x / nchunk, chunk = blockIdx.x - f * nchunk, op = blockIdx.y;
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int j = nown + chunk * BND_ROWS + threadIdx.x;
    if (chunk * BND_ROWS >= nbnd || nf >= tiled_nf) return;
    c64* L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const bool act = j < nf;
    const int jr = act ? j : nf - 1;
    for (int k = 0; k < nown; ++k) {
        c64 acc = L[(int64_t)k * nf + jr];
        // Linv[m, k] (m > k) is held transposed at position (k, m): L[m * nf + k]
        int m = k + 1;
        for (; m + 4 <= nown; m += 4) {
            const c64 a0 = L[(int64_t)m * nf + jr], a1 = L[(int64_t)(m + 1) * nf + jr];
            const c64 a2 = L[(int64_t)(m + 2) * nf + jr], a3 = L[(int64_t)(m + 3) * nf + jr];
            cfma(acc, a0, L[(int64_t)m * nf + k]);
            cfma(acc, a1, L[(int64_t)(m + 1) * nf + k]);
            cfma(acc, a2, L[(int64_t)(m + 2) * nf + k]);
            cfma(acc, a3, L[(int64_t)(m + 3) * nf + k]);
        }
        for (; m < nown; ++m) cfma(acc, L[(int64_t)m * nf + jr], L[(int64_t)m * nf + k]);
        if (act) L[(int64_t)k * nf + j] = mk<double>(-acc.re, -acc.im);
    }
}

void launch_bnd_inv(const Fronts& F, c64* panel, int max_nbnd, int nops, int tiled_nf, cudaStream_t st) {
    const int nchunk = std::max(1, ceil_div(max_nbnd, BND_ROWS));
    bnd_inv_kernel<<<dim3(F.nfront * nchunk, nops), BND_ROWS, 0, st>>>(F, panel, nchunk, tiled_nf);
    GT_LAUNCH_CHECK();
}

// Selective inversion of large fronts, blocked.  The inverted panel [Linv_own; -L_bnd Linv_own] is the first
// nown columns of the inverse of the unit lower triangular T = [L_own 0; L_bnd I], so it is computed in place
// as the forward substitution T Y = [I; 0], FB rows of T per step (kb = FB k, nb = the step's rows):
//   inv_rows   Y[kb.., c] = L_kk^-1 Y[kb.., c] for columns c < kb (their right-hand sides accumulated so far)
//   inv_diag   L_kk -> its inverse, in place, by one warp (a lane per row; D stays on the diagonal)
//   inv_trail  Y[i, c] -= L[i, kb..] Y[kb.., c] for the rows i below the block: first the columns c < kb,
//              then the block's own columns, whose Y takes the place of the L it is made from (each tile
//              reads its rows of L before it writes; the c < kb pass has read them all by then).
// The panel's upper triangle stays zero; the diagonal keeps D for panel_convert.
__global__ void __launch_bounds__(ROWS_CTA) inv_rows_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                            c64* __restrict__ panel) {
    __shared__ c64 l11[FB][FB];
    const int f = (int)front_list[blockIdx.y];
    const int op = blockIdx.z;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int nb = min(FB, nown - kb);
    if (nb <= 0 || blockIdx.x * ROWS_CTA >= kb) return;
    c64* P = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    for (int q = threadIdx.x; q < FB * FB; q += ROWS_CTA) {
        const int r = q / FB, c = q - r * FB;
        l11[r][c] = (r < nb && c < r) ? P[(int64_t)(kb + c) * nf + kb + r] : zero<double>();
    }
    __syncthreads();
    const int c = blockIdx.x * ROWS_CTA + threadIdx.x;
    if (c >= kb) return;
    c64* col = P + (int64_t)c * nf + kb;
    c64 y[FB];
#pragma unroll
    for (int r = 0; r < FB; ++r) {
        if (r < nb) {
            c64 t = col[r];
#pragma unroll
            for (int m = 0; m < r; ++m) cfms(t, l11[r][m], y[m]);
            y[r] = t;
        }
    }
#pragma unroll
    for (int r = 0; r < FB; ++r)
        if (r < nb) col[r] = y[r];
}

__global__ void __launch_bounds__(32) inv_diag_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                      c64* __restrict__ panel) {
    __shared__ c64 a[FB][FB + 1];
    const int f = (int)front_list[blockIdx.x];
    const int op = blockIdx.y;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int nb = min(FB, nown - kb);
    if (nb <= 0) return;
    c64* P = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int i = threadIdx.x;
    for (int j = 0; j < FB; ++j) a[i][j] = (i < nb && j < i) ? P[(int64_t)(kb + j) * nf + kb + i] : zero<double>();
    __syncwarp();
    if (i >= nb) return;
    // X[i, k] = -(L[i, k] + sum_{k < m < i} X[i, m] L[m, k]), k descending: lane i needs only its own row of X
    c64 x[FB];
#pragma unroll
    for (int k = FB - 1; k >= 0; --k) {
        if (k < i) {
            c64 acc = a[i][k];
#pragma unroll
            for (int m = k + 1; m < FB; ++m)
                if (m < i) cfma(acc, x[m], a[m][k]);
            x[k] = mk<double>(-acc.re, -acc.im);
        }
    }
#pragma unroll
    for (int k = 0; k < FB; ++k)
        if (k < i) P[(int64_t)(kb + k) * nf + kb + i] = x[k];
}

// rows i >= kb + nb of the front; mode 0: columns c < kb (tile grid rt x ct), mode 1: the block's columns
__global__ void __launch_bounds__(256) inv_trail_kernel(Fronts F, const int64_t* __restrict__ front_list, int kb,
                                                        c64* __restrict__ panel, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c64* As = reinterpret_cast<c64*>(smem_raw);          // [m][FT]: L(i0 + r, kb + m)
    c64* Bs = As + FB * FT;                              // [m][FT]: Y(kb + m, c0 + c)
    const int f = (int)front_list[blockIdx.y];
    const int op = blockIdx.z;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int nb = min(FB, nown - kb);
    if (nb <= 0) return;
    const int t0 = kb + nb, n2 = nf - t0;
    if (n2 <= 0) return;
    const int rt = (n2 + FT - 1) / FT;
    const int ncols = mode == 0 ? kb : nb;
    if (ncols <= 0) return;
    const int ct = (ncols + FT - 1) / FT;
    if ((int)blockIdx.x >= rt * ct) return;
    const int bi = blockIdx.x % rt, bj = blockIdx.x / rt;
    const int i0 = t0 + bi * FT, c0 = (mode == 0 ? 0 : kb) + bj * FT;
    const int c1 = mode == 0 ? kb : kb + nb;             // columns c0 .. min(c0 + FT, c1)
    c64* P = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    for (int q = threadIdx.x; q < FB * FT; q += 256) {
        const int m = q / FT, r = q - m * FT;
        c64 a = zero<double>(), b = zero<double>();
        if (m < nb) {
            if (i0 + r < nf) a = P[(int64_t)(kb + m) * nf + i0 + r];
            const int c = c0 + r;
            // Y(kb + m, c): the block row's solved entries; in mode 1 the block's inverse, unit diagonal
            if (c < c1) b = (mode == 1 && c - kb == m) ? mk<double>(1.0, 0.0)
                                                       : (mode == 1 && c - kb > m) ? zero<double>()
                                                                                   : P[(int64_t)c * nf + kb + m];
        }
        As[q] = a;
        Bs[q] = b;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    c64 acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = zero<double>();
    for (int m = 0; m < nb; ++m) {
        c64 a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = As[m * FT + tx + 16 * r];
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = Bs[m * FT + ty + 16 * c];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) cfma(acc[r][c], a[r], b[c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int j = c0 + ty + 16 * c;
        if (j >= c1) continue;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = i0 + tx + 16 * r;
            if (i >= nf) continue;
            c64& y = P[(int64_t)j * nf + i];
            y = (mode == 1 ? zero<double>() : y) - acc[r][c];
        }
    }
}

void launch_invert_tiled(const Fronts& F, const int64_t* front_list, int nfront, int max_nf, int max_nown, c64* panel,
                         int nops, cudaStream_t st) {
    if (nfront <= 0) return;
    raise_smem((const void*)inv_trail_kernel, TRAIL_SMEM);
    for (int kb = 0; kb < max_nown; kb += FB) {
        if (kb > 0) {
            inv_rows_kernel<<<dim3(ceil_div(kb, ROWS_CTA), nfront, nops), ROWS_CTA, 0, st>>>(F, front_list, kb, panel);
            GT_LAUNCH_CHECK();
        }
        inv_diag_kernel<<<dim3(nfront, nops), 32, 0, st>>>(F, front_list, kb, panel);
        GT_LAUNCH_CHECK();
        const int below = max_nf - kb - 1;
        if (below <= 0) continue;
        const int rt = ceil_div(below, FT);
        if (kb > 0) {
            inv_trail_kernel<<<dim3(rt * ceil_div(kb, FT), nfront, nops), 256, TRAIL_SMEM, st>>>(F, front_list, kb, panel, 0);
            GT_LAUNCH_CHECK();
        }
        inv_trail_kernel<<<dim3(rt, nfront, nops), 256, TRAIL_SMEM, st>>>(F, front_list, kb, panel, 1);
        GT_LAUNCH_CHECK();
    }
}

// Finish the solve panels: the own block gets its inverse below an explicit unit diagonal (moved from the
// upper triangle, which becomes zero; the pivots go to dinv as 1/D), and the FP32 column-major, FP32 / FP64
// row-major copies are written.
// r64 (the FP64 row-major copy) may be null: operators that keep their FP32 panels only
__global__ void panel_convert_kernel(Fronts F, c64* __restrict__ p64, c32* __restrict__ p32, c32* __restrict__ r32,
                                     c64* __restrict__ r64, c64* __restrict__ d64, c32* __restrict__ d32, int tiled_nf) {
    const int f = blockIdx.x;
    const int op = blockIdx.y;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const bool in_place = nf >= tiled_nf;                       // the blocked inversion: X below the diagonal
    const int64_t base = (int64_t)op * F.panel_total + F.panel_off[f];
    const int64_t dbase = (int64_t)op * F.nfac + F.own_start[f];
    for (int64_t q = threadIdx.x; q < (int64_t)nf * nown; q += blockDim.x) {
        int k = int(q / nf), i = int(q - (int64_t)k * nf);      // column-major element (i, k)
        if (i < k) {                                             // the upper triangle: zero
            if (in_place) {
                p32[base + q] = zero<float>();
                r32[base + (int64_t)i * nown + k] = zero<float>();
                if (r64) r64[base + (int64_t)i * nown + k] = zero<double>();
            }
            continue;                                            // (else with its partner below)
        }
        c64 v = p64[base + q];
        if (i == k) {
            const c64 dv = cdiv(mk<double>(1.0, 0.0), v);
            d64[dbase + i] = dv;
            d32[dbase + i] = cvt<float>(dv);
            v = mk<double>(1.0, 0.0);
            p64[base + q] = v;
        } else if (i < nown && !in_place) {
            // X[i, k] from its transposed position (k, i), which becomes zero
            const int64_t qt = (int64_t)i * nf + k;
            v = p64[base + qt];
            p64[base + q] = v;
            p64[base + qt] = zero<double>();
            p32[base + qt] = zero<float>();
            r32[base + (int64_t)k * nown + i] = zero<float>();
            if (r64) r64[base + (int64_t)k * nown + i] = zero<double>();
        }
        p32[base + q] = cvt<float>(v);
        r32[base + (int64_t)i * nown + k] = cvt<float>(v);
        if (r64) r64[base + (int64_t)i * nown + k] = v;
    }
}

void launch_panel_convert(const Fronts& F, c64* p64, c32* p32, c32* r32, c64* r64, c64* d64, c32* d32, int nops,
                          int tiled_nf, cudaStream_t st) {
    panel_convert_kernel<<<dim3(F.nfront, nops), 256, 0, st>>>(F, p64, p32, r32, r64, d64, d32, tiled_nf);
    GT_LAUNCH_CHECK();
}

// ------------------------------------------------------------------------------------------ solves
// z, y: [col][nfac] in factor order; uvec: [col][vec_total] update vectors; sd: [col][S*nx*ny] in node order.
// After the factorisation each front's panel holds P = [Linv_own; -L_bnd Linv_own] (nf x nown, unit
// diagonal, zeros above it) and dinv = 1/D of its pivots (selective inversion), so that a front's solves are
// two dense matrix-vector products without a sequential chain:
//   forward   out = P w_own: own rows z_own = dinv * out, boundary rows w_bnd + out go up as the update
//   backward  y_own = P^T [z_own; y_bnd]   (y_bnd: the ancestors' results, final)
// A task is (front, group of <= 8 columns sharing its operator, block of rows / columns); its warps split
// the block into 32-row (32-column) tiles and the product's inner dimension into segments whose partial sums
// meet in shared memory.  The launch shape is chosen per level so that the top of the tree, with few fronts,
// still spreads over every SM.  Panel elements are read once per task by consecutive lanes, LB loads in flight.
constexpr int LB = 8;
constexpr int SOLVE_THREADS = 512;

template <typename R>
static void smem_attr(const void* fn, size_t bytes) { raise_smem(fn, bytes); }

// two consecutive columns' entries of a k-major shared vector (one 16-byte load in FP32)
__device__ __forceinline__ void lds2(const c32* p, c32& a, c32& b) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    a = mk<float>(t.x, t.y);
    b = mk<float>(t.z, t.w);
}
__device__ __forceinline__ void lds2(const c64* p, c64& a, c64& b) {
    a = p[0];
    b = p[1];
}

// acc[c] += a * x[c] over all GC columns of one k-major shared row x (unused columns hold zeros)
template <typename R, int GC>
__device__ __forceinline__ void mac_row(cx<R>* acc, cx<R> a, const cx<R>* x) {
#pragma unroll
    for (int c2 = 0; c2 < GC / 2; ++c2) {
        cx<R> u, v;
        lds2(x + 2 * c2, u, v);
        cfma(acc[2 * c2], a, u);
        cfma(acc[2 * c2 + 1], a, v);
    }
    if constexpr (GC % 2 == 1) cfma(acc[GC - 1], a, x[GC - 1]);
}

// acc[c] += sum_{t < cnt} A[t * lda] x[t * xs + c]: A a strided run of panel elements (part of one row or
// column of a front's panel), x the matching k-major shared rows.  The first LB elements were loaded into
// l ahead of time (prefetch_run, issued before the shared rows were staged); LB loads in flight after that.
template <typename R>
__device__ __forceinline__ void prefetch_run(const cx<R>* __restrict__ A, int lda, int cnt, cx<R>* l) {
#pragma unroll
    for (int u = 0; u < LB; ++u) l[u] = u < cnt ? A[u * lda] : zero<R>();
}

template <typename R, int GC>
__device__ __forceinline__ void sweep(const cx<R>* __restrict__ A, int lda, const cx<R>* x, int xs, int cnt,
                                      const cx<R>* l0, cx<R>* acc) {
#pragma unroll
    for (int u = 0; u < LB; ++u)
        if (u < cnt) mac_row<R, GC>(acc, l0[u], x + u * xs);
    A += LB * lda;
    x += LB * xs;
    int t = LB;
    for (; t + LB <= cnt; t += LB) {
        cx<R> l[LB];
#pragma unroll
        for (int u = 0; u < LB; ++u) l[u] = A[u * lda];
#pragma unroll
        for (int u = 0; u < LB; ++u) mac_row<R, GC>(acc, l[u], x + u * xs);
        A += LB * lda;
        x += LB * xs;
    }
    for (; t < cnt; ++t) {
        mac_row<R, GC>(acc, *A, x);
        A += lda;
        x += xs;
    }
}

// The forward rows of front f for a group: own rows of w (s in factor order plus the children's updates)
// into ws (k-major, ldw = GC) and boundary rows r0 <= p < r1 into wt ([c][TR]).  Loads are issued four
// at a time per thread ahead of their stores.
template <typename R, int GC>
__device__ __forceinline__ void fwd_gather(const Fronts& F, int f, const int* gs, int gc, const cx<R>* __restrict__ sf,
                                           const cx<R>* __restrict__ uvec, cx<R>* ws, cx<R>* wt, int TR, int r0, int r1) {
    const int nown = (int)F.nown[f];
    const int64_t own0 = F.own_start[f];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int tot = gc * nown;
    for (int q = tot + tid; q < GC * nown; q += nth) ws[(q % nown) * GC + q / nown] = zero<R>();
    for (int q0 = tid; q0 < tot; q0 += 4 * nth) {
        cx<R> v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = min(q0 + u * nth, tot - 1), c = q / nown;
            v[u] = sf[(int64_t)gs[c] * F.nfac + own0 + (q - c * nown)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * nth;
            if (q < tot) ws[(q % nown) * GC + q / nown] = v[u];
        }
    }
    __syncthreads();
    for (int64_t ci = F.child_ptr[f]; ci < F.child_ptr[f + 1]; ++ci) {
        const int ch = (int)F.child_idx[ci];
        const int nb = (int)F.nbnd[ch], tc = gc * nb;
        const int64_t* map = F.cmap_idx + F.cmap_ptr[ci];
        const int64_t voff = F.vec_off[ch];
        for (int q0 = tid; q0 < tc; q0 += 4 * nth) {
            int p[4];
            cx<R> v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int q = min(q0 + u * nth, tc - 1), c = q / nb, i = q - c * nb;
                p[u] = (int)map[i];
                v[u] = uvec[(int64_t)gs[c] * F.vec_total + voff + i];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int q = q0 + u * nth;
                if (q >= tc) break;
                const int c = q / nb;
                if (p[u] < nown) ws[p[u] * GC + c] += v[u];
                else if (p[u] >= r0 && p[u] < r1) wt[c * TR + p[u] - r0] += v[u];
            }
        }
        __syncthreads();
    }
}

// Forward assembly of a front split over several blocks, once per (front, group): w_own to wasm (factor
// order), the children's updates of the boundary rows to the front's own update-vector slots.
template <typename R, int GC>
__global__ void __launch_bounds__(256) fwd_assemble_kernel(Fronts F, const int64_t* __restrict__ front_list,
                                                           const cx<R>* sf, cx<R>* __restrict__ uvec, cx<R>* wasm,
                                                           Groups G, int ldw, int TR) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* ws = reinterpret_cast<cx<R>*>(smem_raw);   // [k][GC]
    cx<R>* wt = ws + GC * ldw;                      // [c][TR] boundary rows
    const int g = blockIdx.x % G.ngroup;
    const int f = (int)front_list[blockIdx.x / G.ngroup];
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    for (int q = threadIdx.x; q < GC * TR; q += blockDim.x) wt[q] = zero<R>();
    __syncthreads();
    fwd_gather<R, GC>(F, f, gs, gc, sf, uvec, ws, wt, TR, nown, nf);
    for (int q = threadIdx.x; q < gc * nown; q += blockDim.x) {
        const int c = q / nown, r = q - c * nown;
        wasm[(int64_t)gs[c] * F.nfac + own0 + r] = ws[r * GC + c];
    }
    for (int q = threadIdx.x; q < gc * nbnd; q += blockDim.x) {
        const int c = q / nbnd, j = q - c * nbnd;
        uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + j] = wt[c * TR + j];
    }
}

// pre: the front was assembled by fwd_assemble_kernel (own rows in wasm, boundary rows in uvec)
template <typename R, int GC>
__global__ void __launch_bounds__(SOLVE_THREADS, 2) fwd_gemv_kernel(Fronts F, const int64_t* __restrict__ front_list, int nblk,
                                                                 int rt, int kseg, const cx<R>* __restrict__ panel,
                                                                 const cx<R>* __restrict__ dinv, const cx<R>* sf,
                                                                 cx<R>* __restrict__ z, cx<R>* __restrict__ uvec,
                                                                 const cx<R>* wasm, Groups G, int ldw, int pre) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int TR = 32 * rt;
    cx<R>* ws = reinterpret_cast<cx<R>*>(smem_raw);   // [k][GC] own rows of w
    cx<R>* wt = ws + GC * ldw;                      // [c][TR] the block's boundary rows of w
    cx<R>* red = wt + GC * TR;                      // [seg][c][TR] partial sums
    const int b = blockIdx.x % nblk, rest = blockIdx.x / nblk;
    const int g = rest % G.ngroup;
    const int f = (int)front_list[rest / G.ngroup];
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int r0 = b * TR;
    if (r0 >= nf) return;
    const int r1 = min(nf, r0 + TR);
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int64_t own0 = F.own_start[f];
    const int tid = threadIdx.x, nth = blockDim.x;
    const cx<R>* __restrict__ P = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int lane = tid & 31, warp = tid >> 5;
    const int tile = warp % rt, seg = warp / rt;
    const int rl = tile * 32 + lane, r = r0 + rl;
    // the tile's rows need columns k < min(nown, last row + 1) (P is zero above its diagonal)
    const int kmax = min(nown, r0 + tile * 32 + 32);
    const int ks = (kmax + kseg - 1) / kseg;
    const int k0 = min(kmax, seg * ks), k1 = min(kmax, k0 + ks);
    const bool valid = r < r1;
    // lanes past the block's rows sweep its last row (results dropped)
    const cx<R>* A = P + (int64_t)k0 * nf + min(r, r1 - 1);
    if (pre) {
        for (int q = tid; q < GC * nown; q += nth) {
            const int c = q / nown, r = q - c * nown;
            ws[r * GC + c] = c < gc ? wasm[(int64_t)gs[c] * F.nfac + own0 + r] : zero<R>();
        }
        for (int q = tid; q < GC * TR; q += nth) {
            const int c = q / TR, rr = q - c * TR, row = r0 + rr;
            wt[q] = (c < gc && row >= nown && row < r1)
                        ? uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + (row - nown)] : zero<R>();
        }
        __syncthreads();
    } else {
        for (int q = tid; q < GC * TR; q += nth) wt[q] = zero<R>();
        __syncthreads();
        fwd_gather<R, GC>(F, f, gs, gc, sf, uvec, ws, wt, TR, r0, r1);
    }
    cx<R> l0[LB];
    prefetch_run<R>(A, nf, k1 - k0, l0);
    cx<R> acc[GC];
#pragma unroll
    for (int c = 0; c < GC; ++c) acc[c] = zero<R>();
    sweep<R, GC>(A, nf, ws + k0 * GC, GC, k1 - k0, l0, acc);
    if (kseg > 1) {
#pragma unroll
        for (int c = 0; c < GC; ++c)
            if (c < gc) red[(seg * GC + c) * TR + rl] = acc[c];
        __syncthreads();
        for (int q = tid; q < gc * TR; q += nth) {
            const int c = q / TR, rr = q - c * TR;
            if (r0 + rr >= r1) continue;
            cx<R> v = red[c * TR + rr];
            for (int sg = 1; sg < kseg; ++sg) v += red[(sg * GC + c) * TR + rr];
            const int row = r0 + rr;
            if (row < nown) z[(int64_t)gs[c] * F.nfac + own0 + row] = dinv[(int64_t)op * F.nfac + own0 + row] * v;
            else uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + (row - nown)] = wt[c * TR + rr] + v;
        }
    } else if (valid) {
        if (r < nown) {
            const cx<R> dv = dinv[(int64_t)op * F.nfac + own0 + r];
#pragma unroll
            for (int c = 0; c < GC; ++c)
                if (c < gc) z[(int64_t)gs[c] * F.nfac + own0 + r] = dv * acc[c];
        } else {
#pragma unroll
            for (int c = 0; c < GC; ++c)
                if (c < gc) uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + (r - nown)] = wt[c * TR + rl] + acc[c];
        }
    }
}

template <typename R, int GC>
__global__ void __launch_bounds__(SOLVE_THREADS, 2) bwd_gemv_kernel(Fronts F, const int64_t* __restrict__ front_list, int nblk,
                                                                 int ct, int iseg, int cw,
                                                                 const cx<R>* __restrict__ panel_rm,
                                                                 const cx<R>* __restrict__ z, cx<R>* __restrict__ y,
                                                                 cx<R>* __restrict__ sd, Groups G, int ldv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int TC = cw * ct;       // a tile: cw columns, its warp's 32 / cw lane groups take alternate rows
    cx<R>* v = reinterpret_cast<cx<R>*>(smem_raw);    // [i - kb0][GC]: rows kb0 .. nf of [z_own; y_bnd]
    cx<R>* red = v + GC * ldv;                      // [seg][c][TC]
    const int b = blockIdx.x % nblk, rest = blockIdx.x / nblk;
    const int g = rest % G.ngroup;
    const int f = (int)front_list[rest / G.ngroup];
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int kb0 = b * TC;
    if (kb0 >= nown) return;
    const int kb1 = min(nown, kb0 + TC);
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int64_t own0 = F.own_start[f];
    const int64_t* bnd = F.bnd_idx + F.bnd_ptr[f];
    const int tid = threadIdx.x, nth = blockDim.x;
    const cx<R>* __restrict__ P = panel_rm + (int64_t)op * F.panel_total + F.panel_off[f];   // (nf x nown) row-major
    const int lane = tid & 31, warp = tid >> 5;
    const int nph = 32 / cw, ph = lane / cw;
    const int tile = warp % ct, seg = warp / ct;
    const int kl = tile * cw + (lane - ph * cw), k = kb0 + kl;
    // the tile's columns need rows i >= its first column (P is zero above its diagonal)
    const int it0 = min(nf, kb0 + tile * cw);
    const int is = (nf - it0 + iseg - 1) / iseg;
    const int i0 = min(nf, it0 + seg * is), i1 = min(nf, i0 + is);
    const int cnt = max(0, (i1 - i0 - ph + nph - 1) / nph);
    const bool valid = k < kb1;
    // lanes past the block's columns sweep its last column (results dropped)
    const cx<R>* A = P + (int64_t)(i0 + ph) * nown + min(k, kb1 - 1);
    cx<R> l0[LB];
    prefetch_run<R>(A, nph * nown, cnt, l0);
    const int nv = nf - kb0, tot = gc * nv;
    for (int q = gc * nv + tid; q < GC * nv; q += nth) {
        const int c = q / nv;
        v[(q - c * nv) * GC + c] = zero<R>();
    }
    for (int q0 = tid; q0 < tot; q0 += 4 * nth) {
        int64_t src[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = min(q0 + u * nth, tot - 1), c = q / nv, i = kb0 + (q - c * nv);
            src[u] = (int64_t)gs[c] * F.nfac + (i < nown ? own0 + i : bnd[i - nown]);
        }
        cx<R> x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = min(q0 + u * nth, tot - 1), c = q / nv, i = kb0 + (q - c * nv);
            x[u] = i < nown ? z[src[u]] : y[src[u]];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * nth;
            if (q < tot) v[(q % nv) * GC + q / nv] = x[u];
        }
    }
    __syncthreads();
    cx<R> acc[GC];
#pragma unroll
    for (int c = 0; c < GC; ++c) acc[c] = zero<R>();
    sweep<R, GC>(A, nph * nown, v + (i0 + ph - kb0) * GC, nph * GC, cnt, l0, acc);
    if (nph == 2) {
#pragma unroll
        for (int c = 0; c < GC; ++c) {
            acc[c].re += __shfl_xor_sync(0xffffffffu, acc[c].re, 16);
            acc[c].im += __shfl_xor_sync(0xffffffffu, acc[c].im, 16);
        }
    }
    if (iseg > 1) {
#pragma unroll
        for (int c = 0; c < GC; ++c)
            if (c < gc && ph == 0) red[(seg * GC + c) * TC + kl] = acc[c];
        __syncthreads();
        for (int q = tid; q < gc * TC; q += nth) {
            const int c = q / TC, kk = q - c * TC;
            if (kb0 + kk >= kb1) continue;
            cx<R> s = red[c * TC + kk];
            for (int sg = 1; sg < iseg; ++sg) s += red[(sg * GC + c) * TC + kk];
            y[(int64_t)gs[c] * F.nfac + own0 + kb0 + kk] = s;
            sd[(int64_t)gs[c] * F.nnode + F.iperm[own0 + kb0 + kk]] = s;
        }
    } else if (valid && ph == 0) {
        const int64_t node = F.iperm[own0 + k];
#pragma unroll
        for (int c = 0; c < GC; ++c)
            if (c < gc) {
                y[(int64_t)gs[c] * F.nfac + own0 + k] = acc[c];
                sd[(int64_t)gs[c] * F.nnode + node] = acc[c];
            }
    }
}

// Launch shape of a level, chosen from the level's fronts alone, never from the number of column groups in the
// solve: the split of the inner dimension sets the order in which partial sums meet, so a column's arithmetic
// (and rounding) must not depend on how many columns share the launch.  The choice assumes a nominal
// NOMINAL_GROUPS groups per front (the sweep batches 8 columns per group): with enough (front, group) tasks
// to fill the GPU a block takes a whole small front; otherwise a block takes one 32-row (32-column) tile and
// splits the inner dimension over warps.
constexpr int NOMINAL_GROUPS = 32;
static void solve_shape(int nfront_level, int ntile, int inner, int& per_blk, int& nseg) {
    const int fill = 8 * 152;
    const int64_t ntask = (int64_t)nfront_level * NOMINAL_GROUPS;
    if (ntask * ntile >= fill && ntile <= 4 && ntask >= fill / 2) {
        per_blk = ntile;
        nseg = 1;
    } else {
        per_blk = 1;
        nseg = std::max(1, std::min(SOLVE_THREADS / 32, (inner + 63) / 64));
    }
}

template <typename R, int GC>
static void fwd_level_gc(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                         const cx<R>* panel, const cx<R>* dinv, const cx<R>* sf, cx<R>* z, cx<R>* uvec, cx<R>* wasm,
                         const Groups& G, cudaStream_t st) {
    const int ntask = nf_level * G.ngroup;
    const int ntile = ceil_div(max_nf, 32);
    int rt, kseg;
    solve_shape(nf_level, ntile, max_nown, rt, kseg);
    const int nblk = ceil_div(ntile, rt), ldw = std::max(max_nown, 1);
    const int pre = nblk > 1;
    if (pre) {
        const int TRa = std::max(max_nf - 1, 1);
        const size_t sa = (size_t)GC * (ldw + TRa) * sizeof(cx<R>);
        smem_attr<R>((const void*)fwd_assemble_kernel<R, GC>, sa);
        fwd_assemble_kernel<R, GC><<<ntask, 256, sa, st>>>(F, front_list, sf, uvec, wasm, G, ldw, TRa);
        GT_LAUNCH_CHECK();
    }
    const size_t sm = (size_t)GC * (ldw + 32 * rt + (kseg > 1 ? kseg * 32 * rt : 0)) * sizeof(cx<R>);
    smem_attr<R>((const void*)fwd_gemv_kernel<R, GC>, sm);
    fwd_gemv_kernel<R, GC><<<ntask * nblk, 32 * rt * kseg, sm, st>>>(F, front_list, nblk, rt, kseg, panel, dinv, sf, z, uvec,
                                                                wasm, G, ldw, pre);
    GT_LAUNCH_CHECK();
}

template <typename R, int GC>
static void bwd_level_gc(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                         const cx<R>* panel_rm, const cx<R>* z, cx<R>* y, cx<R>* sd, const Groups& G, cudaStream_t st) {
    const int ntask = nf_level * G.ngroup;
    // tiles of 16 columns (two lane groups on alternate rows) where they waste fewer lanes than 32
    const int cw = ceil_div(max_nown, 16) * 16 - max_nown < ceil_div(max_nown, 32) * 32 - max_nown ? 16 : 32;
    const int ntile = ceil_div(max_nown, cw);
    int ct, iseg;
    solve_shape(nf_level, ntile, max_nf, ct, iseg);
    const int nblk = ceil_div(ntile, ct), ldv = std::max(max_nf, 1);
    const size_t sm = (size_t)GC * (ldv + (iseg > 1 ? iseg * cw * ct : 0)) * sizeof(cx<R>);
    smem_attr<R>((const void*)bwd_gemv_kernel<R, GC>, sm);
    bwd_gemv_kernel<R, GC><<<ntask * nblk, 32 * ct * iseg, sm, st>>>(F, front_list, nblk, ct, iseg, cw, panel_rm, z, y, sd,
                                                                 G, ldv);
    GT_LAUNCH_CHECK();
}

// the column-group widths the sweep kernels are built for: a front's rows for GC columns are staged in shared
// memory, so wide fronts take narrower groups (the panel is then read once per fewer columns)
template <typename R>
void launch_fwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel, const cx<R>* dinv, const cx<R>* sf, cx<R>* z, cx<R>* uvec, cx<R>* wasm,
                      const Groups& G, int gmax, cudaStream_t st) {
    switch (gmax) {
        case 8: fwd_level_gc<R, 8>(F, front_list, nf_level, max_nf, max_nown, panel, dinv, sf, z, uvec, wasm, G, st); return;
        case 4: fwd_level_gc<R, 4>(F, front_list, nf_level, max_nf, max_nown, panel, dinv, sf, z, uvec, wasm, G, st); return;
        case 2: fwd_level_gc<R, 2>(F, front_list, nf_level, max_nf, max_nown, panel, dinv, sf, z, uvec, wasm, G, st); return;
        case 1: fwd_level_gc<R, 1>(F, front_list, nf_level, max_nf, max_nown, panel, dinv, sf, z, uvec, wasm, G, st); return;
        default: throw CudaError{cudaErrorInvalidValue, "column group width must be 8, 4, 2 or 1"};
    }
}

template <typename R>
void launch_bwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel_rm, const cx<R>* z, cx<R>* y, cx<R>* sd, const Groups& G, int gmax,
                      cudaStream_t st) {
    switch (gmax) {
        case 8: bwd_level_gc<R, 8>(F, front_list, nf_level, max_nf, max_nown, panel_rm, z, y, sd, G, st); return;
        case 4: bwd_level_gc<R, 4>(F, front_list, nf_level, max_nf, max_nown, panel_rm, z, y, sd, G, st); return;
        case 2: bwd_level_gc<R, 2>(F, front_list, nf_level, max_nf, max_nown, panel_rm, z, y, sd, G, st); return;
        case 1: bwd_level_gc<R, 1>(F, front_list, nf_level, max_nf, max_nown, panel_rm, z, y, sd, G, st); return;
        default: throw CudaError{cudaErrorInvalidValue, "column group width must be 8, 4, 2 or 1"};
    }
}

template void launch_fwd_level<float>(const Fronts&, const int64_t*, int, int, int, const c32*, const c32*, const c32*, c32*, c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_fwd_level<double>(const Fronts&, const int64_t*, int, int, int, const c64*, const c64*, const c64*, c64*, c64*, c64*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<float>(const Fronts&, const int64_t*, int, int, int, const c32*, const c32*, c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<double>(const Fronts&, const int64_t*, int, int, int, const c64*, const c64*, c64*, c64*, const Groups&, int, cudaStream_t);

}  // namespace gt
