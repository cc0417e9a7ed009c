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

__global__ void factor_level_kernel(Fronts F, const int64_t* __restrict__ front_list, const c64* __restrict__ svals,
                                    c64* __restrict__ panel, c64* __restrict__ upd, int* __restrict__ status) {
    const int f = (int)front_list[blockIdx.x];
    const int op = blockIdx.y;
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    FrontView Fv{panel + (int64_t)op * F.panel_total + F.panel_off[f], upd + (int64_t)op * F.upd_total + F.upd_off[f], nf,
                 nown, nbnd};
    const int tid = threadIdx.x, nth = blockDim.x;
    // zero the front
    for (int64_t q = tid; q < (int64_t)nf * nown; q += nth) Fv.panel[q] = zero<double>();
    for (int64_t q = tid; q < (int64_t)nbnd * nbnd; q += nth) Fv.upd[q] = zero<double>();
    __syncthreads();
    // own columns of S
    const c64* sv = svals + (int64_t)op * F.nsv;
    for (int64_t e = F.ent_ptr[f] + tid; e < F.ent_ptr[f + 1]; e += nth) Fv.at(F.ent_row[e], F.ent_col[e]) += sv[F.ent_s[e]];
    __syncthreads();
    // children's update matrices, one child at a time (their boundaries overlap)
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
    // eliminate the own columns
    const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
    for (int k = 0; k < nown; ++k) {
        c64 d = Fv.panel[(int64_t)k * nf + k];
        double dd = d.re * d.re + d.im * d.im;
        if (!(dd > 1e-300) || !isfinite(dd)) {
            if (tid == 0) atomicOr(status, 1);
            d = mk<double>(1e-150, 0.0);
        }
        const c64 dinv = cdiv(mk<double>(1.0, 0.0), d);
        const c64* colk = Fv.panel + (int64_t)k * nf;
        for (int j = k + 1 + warp; j < nf; j += nwarp) {
            const c64 ljd = colk[j] * dinv;
            for (int i = j + lane; i < nf; i += 32) Fv.at(i, j) -= colk[i] * ljd;
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

// The factor's panels for the solves: FP32 column-major (forward), FP32 and FP64 row-major (backward).
__global__ void panel_convert_kernel(Fronts F, const c64* __restrict__ p64, c32* __restrict__ p32, c32* __restrict__ r32,
                                     c64* __restrict__ r64) {
    const int f = blockIdx.x;
    const int op = blockIdx.y;
    const int nown = (int)F.nown[f], nf = nown + (int)F.nbnd[f];
    const int64_t base = (int64_t)op * F.panel_total + F.panel_off[f];
    for (int64_t q = threadIdx.x; q < (int64_t)nf * nown; q += blockDim.x) {
        int k = int(q / nf), i = int(q - (int64_t)k * nf);      // column-major element (i, k)
        c64 v = p64[base + q];
        p32[base + q] = cvt<float>(v);
        r32[base + (int64_t)i * nown + k] = cvt<float>(v);
        r64[base + (int64_t)i * nown + k] = v;
    }
}

void launch_panel_convert(const Fronts& F, const c64* p64, c32* p32, c32* r32, c64* r64, int nops, cudaStream_t st) {
    panel_convert_kernel<<<dim3(F.nfront, nops), 256, 0, st>>>(F, p64, p32, r32, r64);
    GT_LAUNCH_CHECK();
}

// ------------------------------------------------------------------------------------------ solves
// z: [col][nfac] in factor order; uvec: [col][vec_total] update vectors.  Two forms, chosen per level:
//
// small fronts (nf <= 128, nown <= 64): one warp per task (a front and a group of <= 8 columns sharing its
//   operator), the front's rows in registers (row r on lane r mod 32), no block barrier.  Forward: a column
//   sweep of the column-major panel with the next column's loads issued before the current one is used.
//   Backward: a row sweep of the row-major copy: every boundary row (y known) updates the own rows, then the
//   own rows from the last.
// larger fronts: one block per task, w in shared memory [GMAXC][ldw]; the own block in blocks of 32 columns:
//   the 32 x 32 diagonal block by one warp per column, warp-synchronously, the rest by sweeps in which each
//   thread owns a row (forward, column-major panel) or a column (backward, row-major panel), every panel
//   element read once, coalesced, 8 loads in flight per thread.
constexpr int GMAXC = 8;
constexpr int TB = 32;
constexpr int RPL = 4;           // rows per lane of the small-front kernels (nf <= 128)
constexpr int SMALL_NF = 32 * RPL;
constexpr int SMALL_NOWN = 64;

template <typename R>
static void smem_attr(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) GT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

template <typename R>
__device__ __forceinline__ cx<R> shfl_cx(cx<R> v, int src) {
    return mk<R>(__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src));
}

template <typename R>
__global__ void __launch_bounds__(256) fwd_small_kernel(Fronts F, const int64_t* __restrict__ front_list, int ntask,
                                                        const cx<R>* __restrict__ panel, cx<R>* __restrict__ z,
                                                        cx<R>* __restrict__ uvec, Groups G) {
    const int lane = threadIdx.x & 31;
    const int task = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (task >= ntask) return;
    const int g = task % G.ngroup;
    const int f = (int)front_list[task / G.ngroup];
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const cx<R>* __restrict__ L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    // stage the rows in the warp's shared-memory region: own entries of s, children's update vectors added
    // one child at a time (their boundaries can share rows), then into registers
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* ws = reinterpret_cast<cx<R>*>(smem_raw) + (int64_t)(threadIdx.x >> 5) * GMAXC * SMALL_NF;
    for (int c = 0; c < gc; ++c)
        for (int r = lane; r < nf; r += 32)
            ws[c * SMALL_NF + r] = r < nown ? z[(int64_t)gs[c] * F.nfac + own0 + r] : zero<R>();
    __syncwarp();
    for (int64_t ci = F.child_ptr[f]; ci < F.child_ptr[f + 1]; ++ci) {
        const int ch = (int)F.child_idx[ci];
        const int nb = (int)F.nbnd[ch];
        const int64_t* map = F.cmap_idx + F.cmap_ptr[ci];
        for (int c = 0; c < gc; ++c) {
            const cx<R>* u = uvec + (int64_t)gs[c] * F.vec_total + F.vec_off[ch];
            for (int i = lane; i < nb; i += 32) ws[c * SMALL_NF + map[i]] += u[i];
        }
        __syncwarp();
    }
    cx<R> w[RPL][GMAXC];
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
        const int r = lane + 32 * q;
#pragma unroll
        for (int c = 0; c < GMAXC; ++c) w[q][c] = (c < gc && r < nf) ? ws[c * SMALL_NF + r] : zero<R>();
    }
    cx<R> lc[RPL], ln[RPL];
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
        const int r = lane + 32 * q;
        lc[q] = (nown > 0 && r < nf) ? L[r] : zero<R>();
    }
    for (int k = 0; k < nown; ++k) {
        const int q_k = k >> 5, src = k & 31;
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
            const int r = lane + 32 * q;
            ln[q] = (k + 1 < nown && r < nf) ? L[(int64_t)(k + 1) * nf + r] : zero<R>();
        }
        cx<R> zk[GMAXC];
#pragma unroll
        for (int c = 0; c < GMAXC; ++c) {
            cx<R> mine = zero<R>();
#pragma unroll
            for (int q = 0; q < RPL; ++q)
                if (q == q_k) mine = w[q][c];
            zk[c] = shfl_cx(mine, src);
        }
#pragma unroll
        for (int q = 0; q < RPL; ++q) {
            const int r = lane + 32 * q;
            if (r > k && r < nf) {
#pragma unroll
                for (int c = 0; c < GMAXC; ++c)
                    if (c < gc) w[q][c] -= lc[q] * zk[c];
            }
        }
#pragma unroll
        for (int q = 0; q < RPL; ++q) lc[q] = ln[q];
    }
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
        const int r = lane + 32 * q;
        if (r < nown) {
            const cx<R> d = L[(int64_t)r * nf + r];
#pragma unroll
            for (int c = 0; c < GMAXC; ++c)
                if (c < gc) z[(int64_t)gs[c] * F.nfac + own0 + r] = cdiv(w[q][c], d);
        } else if (r < nf) {
#pragma unroll
            for (int c = 0; c < GMAXC; ++c)
                if (c < gc) uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + (r - nown)] = w[q][c];
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(256) bwd_small_kernel(Fronts F, const int64_t* __restrict__ front_list, int ntask,
                                                        const cx<R>* __restrict__ panel_rm, cx<R>* __restrict__ z,
                                                        Groups G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int task = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (task >= ntask) return;
    cx<R>* ws = reinterpret_cast<cx<R>*>(smem_raw) + (int64_t)(threadIdx.x >> 5) * GMAXC * SMALL_NF;
    const int g = task % G.ngroup;
    const int f = (int)front_list[task / G.ngroup];
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const int64_t* bnd = F.bnd_idx + F.bnd_ptr[f];
    const cx<R>* __restrict__ L = panel_rm + (int64_t)op * F.panel_total + F.panel_off[f];   // (nf x nown) row-major
    for (int c = 0; c < gc; ++c) {
        const cx<R>* zc = z + (int64_t)gs[c] * F.nfac;
        for (int r = lane; r < nf; r += 32) ws[c * SMALL_NF + r] = zc[r < nown ? own0 + r : bnd[r - nown]];
    }
    __syncwarp();
    constexpr int OQ = SMALL_NOWN / 32;
    // boundary rows (y final): acc_k = sum_i L[i, k] y_i, independent over i (4 rows of loads in flight)
    cx<R> w[OQ][GMAXC];
#pragma unroll
    for (int q = 0; q < OQ; ++q)
#pragma unroll
        for (int c = 0; c < GMAXC; ++c) w[q][c] = zero<R>();
    for (int i0 = nown; i0 < nf; i0 += 4) {
        cx<R> l[4][OQ];
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int q = 0; q < OQ; ++q) {
                const int k = lane + 32 * q, i = i0 + ii;
                l[ii][q] = (i < nf && k < nown) ? L[(int64_t)i * nown + k] : zero<R>();
            }
#pragma unroll
        for (int ii = 0; ii < 4; ++ii) {
            const int i = min(i0 + ii, nf - 1);
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) {
                if (c >= gc) break;
                const cx<R> y = ws[c * SMALL_NF + i];
#pragma unroll
                for (int q = 0; q < OQ; ++q) w[q][c] += l[ii][q] * y;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < OQ; ++q) {
        const int k = lane + 32 * q;
#pragma unroll
        for (int c = 0; c < GMAXC; ++c) w[q][c] = (c < gc && k < nown) ? ws[c * SMALL_NF + k] - w[q][c] : zero<R>();
    }
    // own rows from the last: y_j final, own rows k < j updated
    cx<R> lc[OQ], ln[OQ];
#pragma unroll
    for (int q = 0; q < OQ; ++q) {
        const int k = lane + 32 * q;
        lc[q] = (nown >= 2 && k < nown - 1) ? L[(int64_t)(nown - 1) * nown + k] : zero<R>();
    }
    for (int j = nown - 1; j >= 1; --j) {
#pragma unroll
        for (int q = 0; q < OQ; ++q) {
            const int k = lane + 32 * q;
            ln[q] = (j - 1 >= 1 && k < j - 1) ? L[(int64_t)(j - 1) * nown + k] : zero<R>();
        }
        const int q_j = j >> 5, src = j & 31;
        cx<R> yj[GMAXC];
#pragma unroll
        for (int c = 0; c < GMAXC; ++c) {
            cx<R> mine = zero<R>();
#pragma unroll
            for (int q = 0; q < OQ; ++q)
                if (q == q_j) mine = w[q][c];
            yj[c] = shfl_cx(mine, src);
        }
#pragma unroll
        for (int q = 0; q < OQ; ++q) {
            const int k = lane + 32 * q;
            if (k < j) {
#pragma unroll
                for (int c = 0; c < GMAXC; ++c)
                    if (c < gc) w[q][c] -= lc[q] * yj[c];
            }
        }
#pragma unroll
        for (int q = 0; q < OQ; ++q) lc[q] = ln[q];
    }
#pragma unroll
    for (int q = 0; q < OQ; ++q) {
        const int r = lane + 32 * q;
        if (r < nown) {
#pragma unroll
            for (int c = 0; c < GMAXC; ++c)
                if (c < gc) z[(int64_t)gs[c] * F.nfac + own0 + r] = w[q][c];
        }
    }
}

template <typename R>
__device__ __forceinline__ void load_diag(cx<R>* Dsm, const cx<R>* __restrict__ L, int ld, int k0, int kb, bool rowmajor) {
    // Dsm[c * TB + r] = L[k0 + r, k0 + c] (column c, row r of the diagonal block)
    for (int q = threadIdx.x; q < TB * TB; q += blockDim.x) {
        int c = q / TB, r = q - c * TB;
        cx<R> v = zero<R>();
        if (c < kb && r < kb) v = rowmajor ? L[(int64_t)(k0 + r) * ld + k0 + c] : L[(int64_t)(k0 + c) * ld + k0 + r];
        Dsm[q] = v;
    }
}

template <typename R>
__global__ void __launch_bounds__(1024) fwd_block_kernel(Fronts F, const int64_t* __restrict__ front_list, int ntask,
                                                         const cx<R>* __restrict__ panel, cx<R>* __restrict__ z,
                                                         cx<R>* __restrict__ uvec, Groups G, int ldw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* Dsm = reinterpret_cast<cx<R>*>(smem_raw);
    cx<R>* w = Dsm + TB * TB;
    const int task = blockIdx.x;
    const int g = task % G.ngroup;
    const int f = (int)front_list[task / G.ngroup];
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const cx<R>* __restrict__ L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (int q = tid; q < gc * nf; q += nth) {
        int c = q / nf, r = q - c * nf;
        w[c * ldw + r] = r < nown ? z[(int64_t)gs[c] * F.nfac + own0 + r] : zero<R>();
    }
    __syncthreads();
    for (int64_t ci = F.child_ptr[f]; ci < F.child_ptr[f + 1]; ++ci) {
        const int ch = (int)F.child_idx[ci];
        const int nb = (int)F.nbnd[ch];
        const int64_t* map = F.cmap_idx + F.cmap_ptr[ci];
        for (int q = tid; q < nb * gc; q += nth) {
            int c = q / nb, i = q - c * nb;
            w[c * ldw + map[i]] += uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[ch] + i];
        }
        __syncthreads();
    }
    for (int k0 = 0; k0 < nown; k0 += TB) {
        const int kb = min(TB, nown - k0);
        load_diag<R>(Dsm, L, nf, k0, kb, false);
        __syncthreads();
        if (warp < gc) {                                 // unit lower triangular solve of the block
            cx<R>* wc = w + warp * ldw + k0;
            cx<R> v = lane < kb ? wc[lane] : zero<R>();
            for (int kk = 0; kk < kb - 1; ++kk) {
                cx<R> zk = shfl_cx(v, kk);
                if (lane > kk && lane < kb) v -= Dsm[kk * TB + lane] * zk;
            }
            if (lane < kb) wc[lane] = v;
        }
        __syncthreads();
        // rows below the block: w[c][i] -= sum_kk L[i, k0+kk] z[c][k0+kk], one thread per row
        for (int i = k0 + kb + tid; i < nf; i += nth) {
            cx<R> acc[GMAXC];
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) acc[c] = zero<R>();
            const cx<R>* Li = L + (int64_t)k0 * nf + i;
            for (int k8 = 0; k8 < kb; k8 += 8) {
                cx<R> l[8];
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) l[kk] = k8 + kk < kb ? Li[(int64_t)(k8 + kk) * nf] : zero<R>();
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
#pragma unroll
                    for (int c = 0; c < GMAXC; ++c)
                        if (c < gc) acc[c] += l[kk] * w[c * ldw + k0 + min(k8 + kk, kb - 1)];
            }
#pragma unroll
            for (int c = 0; c < GMAXC; ++c)
                if (c < gc) w[c * ldw + i] -= acc[c];
        }
        __syncthreads();
    }
    for (int q = tid; q < gc * nf; q += nth) {
        int c = q / nf, r = q - c * nf;
        if (r < nown) z[(int64_t)gs[c] * F.nfac + own0 + r] = cdiv(w[c * ldw + r], L[(int64_t)r * nf + r]);
        else uvec[(int64_t)gs[c] * F.vec_total + F.vec_off[f] + (r - nown)] = w[c * ldw + r];
    }
}

template <typename R>
__global__ void __launch_bounds__(1024) bwd_block_kernel(Fronts F, const int64_t* __restrict__ front_list, int ntask,
                                                         const cx<R>* __restrict__ panel, const cx<R>* __restrict__ panel_rm,
                                                         cx<R>* __restrict__ z, Groups G, int ldw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* Dsm = reinterpret_cast<cx<R>*>(smem_raw);
    cx<R>* w = Dsm + TB * TB;
    const int task = blockIdx.x;
    const int g = task % G.ngroup;
    const int f = (int)front_list[task / G.ngroup];
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const int64_t* bnd = F.bnd_idx + F.bnd_ptr[f];
    const cx<R>* __restrict__ L = panel_rm + (int64_t)op * F.panel_total + F.panel_off[f];   // (nf x nown) row-major
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (int q = tid; q < gc * nf; q += nth) {
        int c = q / nf, r = q - c * nf;
        w[c * ldw + r] = z[(int64_t)gs[c] * F.nfac + (r < nown ? own0 + r : bnd[r - nown])];
    }
    __syncthreads();
    // w[c][k] -= sum_{rows j in [j0, j1)} L[j, k] y[c][j], one thread per own column k < kmax
    auto sweep = [&](int j0, int j1, int kmax) {
        for (int k = tid; k < kmax; k += nth) {
            cx<R> acc[GMAXC];
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) acc[c] = zero<R>();
            for (int j8 = j0; j8 < j1; j8 += 8) {
                cx<R> l[8];
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) l[jj] = j8 + jj < j1 ? L[(int64_t)(j8 + jj) * nown + k] : zero<R>();
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
#pragma unroll
                    for (int c = 0; c < GMAXC; ++c)
                        if (c < gc) acc[c] += l[jj] * w[c * ldw + min(j8 + jj, j1 - 1)];
            }
#pragma unroll
            for (int c = 0; c < GMAXC; ++c)
                if (c < gc) w[c * ldw + k] -= acc[c];
        }
    };
    // the boundary rows (final from the ancestors): w[c][k] -= sum_{i >= nown} L[i, k] y[c][i] as column dot
    // products of the column-major panel, one warp per own column k, lanes down the rows
    {
        const cx<R>* __restrict__ Lc = panel + (int64_t)op * F.panel_total + F.panel_off[f];
        const int nwarp = nth >> 5;
        for (int k = warp; k < nown; k += nwarp) {
            const cx<R>* Lk = Lc + (int64_t)k * nf;
            cx<R> acc[GMAXC];
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) acc[c] = zero<R>();
#pragma unroll 4
            for (int i = nown + lane; i < nf; i += 32) {
                const cx<R> l = Lk[i];
#pragma unroll
                for (int c = 0; c < GMAXC; ++c)
                    if (c < gc) acc[c] += l * w[c * ldw + i];
            }
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) {
                if (c >= gc) break;
                R re = acc[c].re, im = acc[c].im;
                for (int o = 16; o > 0; o >>= 1) {
                    re += __shfl_xor_sync(0xffffffffu, re, o);
                    im += __shfl_xor_sync(0xffffffffu, im, o);
                }
                if (lane == 0) w[c * ldw + k] -= mk<R>(re, im);
            }
        }
    }
    __syncthreads();
    const int nblk = (nown + TB - 1) / TB;
    for (int b = nblk - 1; b >= 0; --b) {
        const int k0 = b * TB, kb = min(TB, nown - k0);
        load_diag<R>(Dsm, L, nown, k0, kb, true);
        __syncthreads();
        if (warp < gc) {                                 // unit upper (L^T) solve of the block from the bottom
            cx<R>* wc = w + warp * ldw + k0;
            cx<R> v = lane < kb ? wc[lane] : zero<R>();
            for (int kk = kb - 1; kk > 0; --kk) {
                cx<R> yk = shfl_cx(v, kk);
                if (lane < kk) v -= Dsm[lane * TB + kk] * yk;    // L[k0+kk, k0+lane]
            }
            if (lane < kb) wc[lane] = v;
        }
        __syncthreads();
        if (k0 > 0) {
            sweep(k0, k0 + kb, k0);                      // this block's rows update the own columns above it
            __syncthreads();
        }
    }
    for (int q = tid; q < gc * nown; q += nth) {
        int c = q / nown, r = q - c * nown;
        z[(int64_t)gs[c] * F.nfac + own0 + r] = w[c * ldw + r];
    }
}


static int block_threads(int max_nf) { return max_nf > 512 ? 1024 : max_nf > 192 ? 512 : 256; }

template <typename R>
void launch_fwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel, cx<R>* z, cx<R>* uvec, const Groups& G, int gmax, cudaStream_t st) {
    if (gmax > GMAXC) throw CudaError{cudaErrorInvalidValue, "column group larger than the solve kernels take"};
    const int ntask = nf_level * G.ngroup;
    if (max_nf <= SMALL_NF && max_nown <= SMALL_NOWN) {
        const size_t sm = (size_t)8 * GMAXC * SMALL_NF * sizeof(cx<R>);
        smem_attr<R>((const void*)fwd_small_kernel<R>, sm);
        fwd_small_kernel<R><<<ceil_div(ntask, 8), 256, sm, st>>>(F, front_list, ntask, panel, z, uvec, G);
    } else {
        const int ldw = max_nf | 1;
        size_t sm = (size_t)(TB * TB + (size_t)GMAXC * ldw) * sizeof(cx<R>);
        smem_attr<R>((const void*)fwd_block_kernel<R>, sm);
        fwd_block_kernel<R><<<ntask, block_threads(max_nf), sm, st>>>(F, front_list, ntask, panel, z, uvec, G, ldw);
    }
    GT_LAUNCH_CHECK();
}

template <typename R>
void launch_bwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel, const cx<R>* panel_rm, cx<R>* z, const Groups& G, int gmax, cudaStream_t st) {
    if (gmax > GMAXC) throw CudaError{cudaErrorInvalidValue, "column group larger than the solve kernels take"};
    const int ntask = nf_level * G.ngroup;
    if (max_nf <= SMALL_NF && max_nown <= SMALL_NOWN) {
        const size_t sm = (size_t)8 * GMAXC * SMALL_NF * sizeof(cx<R>);
        smem_attr<R>((const void*)bwd_small_kernel<R>, sm);
        bwd_small_kernel<R><<<ceil_div(ntask, 8), 256, sm, st>>>(F, front_list, ntask, panel_rm, z, G);
    } else {
        const int ldw = max_nf | 1;
        size_t sm = (size_t)(TB * TB + (size_t)GMAXC * ldw) * sizeof(cx<R>);
        smem_attr<R>((const void*)bwd_block_kernel<R>, sm);
        bwd_block_kernel<R><<<ntask, block_threads(max_nf), sm, st>>>(F, front_list, ntask, panel, panel_rm, z, G, ldw);
    }
    GT_LAUNCH_CHECK();
}

template void launch_fwd_level<float>(const Fronts&, const int64_t*, int, int, int, const c32*, c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_fwd_level<double>(const Fronts&, const int64_t*, int, int, int, const c64*, c64*, c64*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<float>(const Fronts&, const int64_t*, int, int, int, const c32*, const c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<double>(const Fronts&, const int64_t*, int, int, int, const c64*, const c64*, c64*, const Groups&, int, cudaStream_t);

}  // namespace gt
