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
// z: [col][nfac] in factor order; uvec: [col][vec_total] update vectors; w in shared memory [nf][gc]
template <typename R>
__global__ void fwd_level_kernel(Fronts F, const int64_t* __restrict__ front_list, const cx<R>* __restrict__ panel,
                                 cx<R>* __restrict__ z, cx<R>* __restrict__ uvec, Groups G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* w = reinterpret_cast<cx<R>*>(smem_raw);
    const int f = (int)front_list[blockIdx.x];
    const int g = blockIdx.y;
    const int col0 = G.col0[g], gc = G.ncol[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const cx<R>* L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int q = tid; q < nf * gc; q += nth) {
        int r = q / gc, c = q - r * gc;
        w[q] = r < nown ? z[(int64_t)(col0 + c) * F.nfac + own0 + r] : zero<R>();
    }
    __syncthreads();
    for (int64_t ci = F.child_ptr[f]; ci < F.child_ptr[f + 1]; ++ci) {
        const int ch = (int)F.child_idx[ci];
        const int nb = (int)F.nbnd[ch];
        const int64_t* map = F.cmap_idx + F.cmap_ptr[ci];
        for (int q = tid; q < nb * gc; q += nth) {
            int i = q / gc, c = q - i * gc;
            w[map[i] * gc + c] += uvec[(int64_t)(col0 + c) * F.vec_total + F.vec_off[ch] + i];
        }
        __syncthreads();
    }
    for (int k = 0; k < nown; ++k) {
        const cx<R>* Lk = L + (int64_t)k * nf;
        const int rows = nf - k - 1;
        for (int q = tid; q < rows * gc; q += nth) {
            int i = k + 1 + q / gc, c = q % gc;
            w[i * gc + c] -= Lk[i] * w[k * gc + c];
        }
        __syncthreads();
    }
    for (int q = tid; q < nf * gc; q += nth) {
        int r = q / gc, c = q - r * gc;
        if (r < nown) z[(int64_t)(col0 + c) * F.nfac + own0 + r] = cdiv(w[q], L[(int64_t)r * nf + r]);
        else uvec[(int64_t)(col0 + c) * F.vec_total + F.vec_off[f] + (r - nown)] = w[q];
    }
}

template <typename R>
__global__ void bwd_level_kernel(Fronts F, const int64_t* __restrict__ front_list, const cx<R>* __restrict__ panel,
                                 cx<R>* __restrict__ z, Groups G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* w = reinterpret_cast<cx<R>*>(smem_raw);
    const int f = (int)front_list[blockIdx.x];
    const int g = blockIdx.y;
    const int col0 = G.col0[g], gc = G.ncol[g], op = G.op[g];
    const int nown = (int)F.nown[f], nbnd = (int)F.nbnd[f], nf = nown + nbnd;
    const int64_t own0 = F.own_start[f];
    const int64_t* bnd = F.bnd_idx + F.bnd_ptr[f];
    const cx<R>* L = panel + (int64_t)op * F.panel_total + F.panel_off[f];
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int q = tid; q < nf * gc; q += nth) {
        int r = q / gc, c = q - r * gc;
        int64_t idx = r < nown ? own0 + r : bnd[r - nown];
        w[q] = z[(int64_t)(col0 + c) * F.nfac + idx];
    }
    __syncthreads();
    // boundary part: w_k -= sum_i L[nown+i, k] y_bnd[i], one warp per (k, column)
    const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
    for (int q = warp; q < nown * gc; q += nwarp) {
        int k = q / gc, c = q - k * gc;
        const cx<R>* Lk = L + (int64_t)k * nf + nown;
        cx<R> acc = zero<R>();
        for (int i = lane; i < nbnd; i += 32) acc += Lk[i] * w[(nown + i) * gc + c];
        for (int o = 16; o > 0; o >>= 1) {
            acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
            acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
        }
        if (lane == 0) w[k * gc + c] -= acc;
    }
    __syncthreads();
    // own block, k descending: y_k final, then w_k' -= L[k, k'] y_k for k' < k
    for (int k = nown - 1; k > 0; --k) {
        for (int q = tid; q < k * gc; q += nth) {
            int kk = q / gc, c = q - kk * gc;
            w[kk * gc + c] -= L[(int64_t)kk * nf + k] * w[k * gc + c];
        }
        __syncthreads();
    }
    for (int q = tid; q < nown * gc; q += nth) {
        int r = q / gc, c = q - r * gc;
        z[(int64_t)(col0 + c) * F.nfac + own0 + r] = w[q];
    }
}

template <typename R>
static void smem_attr(const void* fn, size_t bytes) {
    if (bytes > 48 * 1024) GT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

template <typename R>
void launch_fwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const cx<R>* panel,
                      cx<R>* z, cx<R>* uvec, const Groups& G, int gmax, cudaStream_t st) {
    size_t sm = (size_t)max_nf * gmax * sizeof(cx<R>);
    smem_attr<R>((const void*)fwd_level_kernel<R>, sm);
    int threads = max_nf * gmax >= 512 ? 512 : 256;
    fwd_level_kernel<R><<<dim3(nf_level, G.ngroup), threads, sm, st>>>(F, front_list, panel, z, uvec, G);
    GT_LAUNCH_CHECK();
}

template <typename R>
void launch_bwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const cx<R>* panel,
                      cx<R>* z, const Groups& G, int gmax, cudaStream_t st) {
    size_t sm = (size_t)max_nf * gmax * sizeof(cx<R>);
    smem_attr<R>((const void*)bwd_level_kernel<R>, sm);
    int threads = max_nf * gmax >= 512 ? 512 : 256;
    bwd_level_kernel<R><<<dim3(nf_level, G.ngroup), threads, sm, st>>>(F, front_list, panel, z, G);
    GT_LAUNCH_CHECK();
}

template void launch_fwd_level<float>(const Fronts&, const int64_t*, int, int, const c32*, c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_fwd_level<double>(const Fronts&, const int64_t*, int, int, const c64*, c64*, c64*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<float>(const Fronts&, const int64_t*, int, int, const c32*, c32*, const Groups&, int, cudaStream_t);
template void launch_bwd_level<double>(const Fronts&, const int64_t*, int, int, const c64*, c64*, const Groups&, int, cudaStream_t);

}  // namespace gt
