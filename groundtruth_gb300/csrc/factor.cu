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

__global__ void panel_to32_kernel(const c64* __restrict__ p64, c32* __restrict__ p32, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p32[i] = cvt<float>(p64[i]);
}

void launch_panel_to32(const c64* p64, c32* p32, int64_t n, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 8192);
    panel_to32_kernel<<<std::max(blocks, 1), 256, 0, st>>>(p64, p32, n);
    GT_LAUNCH_CHECK();
}

// ------------------------------------------------------------------------------------------ solves
// z: [col][nfac] in factor order; uvec: [col][vec_total] update vectors.  Shared memory: w [GMAXC][ldw] (the
// front's rows for each of the group's columns, column-major so that consecutive threads touch consecutive
// rows) and the current 32 x 32 diagonal block of the panel.  The own block is processed in blocks of 32
// columns: the diagonal block by one warp per column, warp-synchronously (the lanes hold the block's 32
// rows); the rest of the front by sweeps in which every panel element is read once, coalesced, with the
// 32 loads of a block row issued back to back.
constexpr int GMAXC = 8;
constexpr int TB = 32;

template <typename R>
__device__ __forceinline__ void load_diag(cx<R>* Dsm, const cx<R>* __restrict__ L, int nf, int k0, int kb) {
    for (int q = threadIdx.x; q < TB * TB; q += blockDim.x) {
        int c = q / TB, r = q - c * TB;                 // column c, row r of the block
        Dsm[q] = (c < kb && r < kb) ? L[(int64_t)(k0 + c) * nf + k0 + r] : zero<R>();
    }
}

template <typename R>
__global__ void __launch_bounds__(1024) fwd_level_kernel(Fronts F, const int64_t* __restrict__ front_list,
                                                         const cx<R>* __restrict__ panel, cx<R>* __restrict__ z,
                                                         cx<R>* __restrict__ uvec, Groups G, int ldw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* Dsm = reinterpret_cast<cx<R>*>(smem_raw);
    cx<R>* w = Dsm + TB * TB;
    const int f = (int)front_list[blockIdx.x];
    const int g = blockIdx.y;
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
        load_diag<R>(Dsm, L, nf, k0, kb);
        __syncthreads();
        if (warp < gc) {                                 // unit lower triangular solve of the block
            cx<R>* wc = w + warp * ldw + k0;
            cx<R> v = lane < kb ? wc[lane] : zero<R>();
            for (int kk = 0; kk < kb - 1; ++kk) {
                cx<R> zk = mk<R>(__shfl_sync(0xffffffffu, v.re, kk), __shfl_sync(0xffffffffu, v.im, kk));
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
            if (kb == TB) {
#pragma unroll
                for (int k8 = 0; k8 < TB; k8 += 8) {
                    cx<R> l[8];
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk) l[kk] = Li[(int64_t)(k8 + kk) * nf];
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk)
#pragma unroll
                        for (int c = 0; c < GMAXC; ++c)
                            if (c < gc) acc[c] += l[kk] * w[c * ldw + k0 + k8 + kk];
                }
            } else {
                for (int kk = 0; kk < kb; ++kk) {
                    const cx<R> lv = Li[(int64_t)kk * nf];
#pragma unroll
                    for (int c = 0; c < GMAXC; ++c)
                        if (c < gc) acc[c] += lv * w[c * ldw + k0 + kk];
                }
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
__global__ void __launch_bounds__(1024) bwd_level_kernel(Fronts F, const int64_t* __restrict__ front_list,
                                                         const cx<R>* __restrict__ panel, cx<R>* __restrict__ z, Groups G,
                                                         int ldw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* Dsm = reinterpret_cast<cx<R>*>(smem_raw);
    cx<R>* w = Dsm + TB * TB;
    const int f = (int)front_list[blockIdx.x];
    const int g = blockIdx.y;
    const int* gs = G.gslot + G.gptr[g];
    const int gc = G.gptr[g + 1] - G.gptr[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const int64_t* bnd = F.bnd_idx + F.bnd_ptr[f];
    const cx<R>* __restrict__ L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int q = tid; q < gc * nf; q += blockDim.x) {
        int c = q / nf, r = q - c * nf;
        w[c * ldw + r] = z[(int64_t)gs[c] * F.nfac + (r < nown ? own0 + r : bnd[r - nown])];
    }
    __syncthreads();
    const int nblk = (nown + TB - 1) / TB;
    for (int b = nblk - 1; b >= 0; --b) {
        const int k0 = b * TB, kb = min(TB, nown - k0), k1 = k0 + kb;
        // w[c][k] -= sum_{i >= k1} L[i, k] y[c][i] for the block's columns: one warp per column k
        for (int kk = warp; kk < kb; kk += nwarp) {
            const cx<R>* Lk = L + (int64_t)(k0 + kk) * nf;
            cx<R> acc[GMAXC];
#pragma unroll
            for (int c = 0; c < GMAXC; ++c) acc[c] = zero<R>();
#pragma unroll 4
            for (int i = k1 + lane; i < nf; i += 32) {
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
                if (lane == 0) w[c * ldw + k0 + kk] -= mk<R>(re, im);
            }
        }
        load_diag<R>(Dsm, L, nf, k0, kb);
        __syncthreads();
        if (warp < gc) {                                 // unit upper (L^T) solve of the block from the bottom
            cx<R>* wc = w + warp * ldw + k0;
            cx<R> v = lane < kb ? wc[lane] : zero<R>();
            for (int kk = kb - 1; kk > 0; --kk) {
                cx<R> yk = mk<R>(__shfl_sync(0xffffffffu, v.re, kk), __shfl_sync(0xffffffffu, v.im, kk));
                if (lane < kk) v -= Dsm[lane * TB + kk] * yk;    // L[k0+kk, k0+lane]
            }
            if (lane < kb) wc[lane] = v;
        }
        __syncthreads();
    }
    for (int q = tid; q < gc * nown; q += blockDim.x) {
        int c = q / nown, r = q - c * nown;
        z[(int64_t)gs[c] * F.nfac + own0 + r] = w[c * ldw + r];
    }
}

template <typename R>
static void smem_attr(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) GT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

static int solve_threads(int max_nf) { return max_nf > 512 ? 1024 : max_nf > 192 ? 512 : 256; }

template <typename R>
void launch_fwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const cx<R>* panel,
                      cx<R>* z, cx<R>* uvec, const Groups& G, int gmax, cudaStream_t st) {
    if (gmax > GMAXC) throw CudaError{cudaErrorInvalidValue, "column group larger than the solve kernels take"};
    const int ldw = max_nf | 1;
    size_t sm = (size_t)(TB * TB + (size_t)ldw * GMAXC) * sizeof(cx<R>);
    smem_attr<R>((const void*)fwd_level_kernel<R>, sm);
    fwd_level_kernel<R><<<dim3(nf_level, G.ngroup), solve_threads(max_nf), sm, st>>>(F, front_list, panel, z, uvec, G, ldw);
    GT_LAUNCH_CHECK();
}

template <typename R>
void launch_bwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const cx<R>* panel,
                      cx<R>* z, const Groups& G, int gmax, cudaStream_t st) {
    if (gmax > GMAXC) throw CudaError{cudaErrorInvalidValue, "column group larger than the solve kernels take"};
    const int ldw = max_nf | 1;
    size_t sm = (size_t)(TB * TB + (size_t)ldw * GMAXC) * sizeof(cx<R>);
    smem_attr<R>((const void*)bwd_level_kernel<R>, sm);
    bwd_level_kernel<R><<<dim3(nf_level, G.ngroup), solve_threads(max_nf), sm, st>>>(F, front_list, panel, z, G, ldw);
    GT_LAUNCH_CHECK();
}

template void launch_fwd_level<float>(const Fronts&, const int64_t*, int, int, const c32*, c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_fwd_level<double>(const Fronts&, const int64_t*, int, int, const c64*, c64*, c64*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<float>(const Fronts&, const int64_t*, int, int, const c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<double>(const Fronts&, const int64_t*, int, int, const c64*, c64*, const Groups&, int, cudaStream_t);

}  // namespace gt
