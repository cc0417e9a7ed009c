// Low-rank branch update of the Schur complement (GroundTruth: PlaneStack.with_branches, peec.py:1871-1912,
// and the derived stack's _factorise, peec.py:2354-2377).  A derived stack adds k branches to a base whose
// Schur complement S is factorised; its own is S' = S + U diag(1/z) U^T with U the incidence of the new
// branches over the kept nodes (+1 at end a, -1 at end b).  By the Woodbury identity
//     S'^-1 v = y - W (Z + U^T W)^-1 U^T y,   y = S^-1 v,   W = S^-1 U,   Z = diag(z),
// so the base's triangular sweeps serve the derived stack, followed by a rank-k correction of y.
// W (node order, zero at nodes that are not kept) and Minv = (Z + U^T W)^-1 are made once per
// factorisation by gt_operators_derive.
#include "kernels.h"

namespace gt {

// the correction's coefficients per column: c = Minv (y[a] - y[b]) over the new branches; one block per
// column, thread i < k gathers branch i's ends, then thread i forms c_i.  c is written to cbuf [col][ldc].
template <typename R>
__global__ void __launch_bounds__(LOWRANK_MAX) lowrank_coef_kernel(const cx<R>* __restrict__ sd, int64_t nnode, int k,
                                                                    const int* __restrict__ ends,
                                                                    const cx<R>* __restrict__ minv,
                                                                    const int* __restrict__ col_fact,
                                                                    const int* __restrict__ col_list,
                                                                    cx<R>* __restrict__ cbuf, int64_t ldc) {
    __shared__ cx<R> t[LOWRANK_MAX];
    const int col = col_list ? col_list[blockIdx.x] : blockIdx.x;
    const int f = col_fact[col];
    const cx<R>* y = sd + (int64_t)col * nnode;
    const int i = threadIdx.x;
    if (i < k) t[i] = y[ends[2 * i]] - y[ends[2 * i + 1]];
    __syncthreads();
    if (i < k) {
        const cx<R>* M = minv + ((int64_t)f * k + i) * k;
        cx<R> c = zero<R>();
        for (int j = 0; j < k; ++j) c += M[j] * t[j];
        cbuf[(int64_t)col * ldc + i] = c;
    }
}

// y -= W c over every node of the column; grid (node chunks, columns)
template <typename R>
__global__ void __launch_bounds__(256) lowrank_apply_kernel(cx<R>* __restrict__ sd, int64_t nnode, int k,
                                                            const cx<R>* __restrict__ w,
                                                            const int* __restrict__ col_fact,
                                                            const int* __restrict__ col_list,
                                                            const cx<R>* __restrict__ cbuf, int64_t ldc) {
    __shared__ cx<R> c[LOWRANK_MAX];
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int f = col_fact[col];
    if (threadIdx.x < k) c[threadIdx.x] = cbuf[(int64_t)col * ldc + threadIdx.x];
    __syncthreads();
    cx<R>* y = sd + (int64_t)col * nnode;
    const cx<R>* W = w + (int64_t)f * k * nnode;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnode; q += (int64_t)gridDim.x * blockDim.x) {
        cx<R> acc = zero<R>();
        for (int j = 0; j < k; ++j) acc += c[j] * W[(int64_t)j * nnode + q];
        y[q] -= acc;
    }
}

template <typename R>
void launch_lowrank(cx<R>* sd, int64_t nnode, int ncol, int k, const int* ends, const cx<R>* w, const cx<R>* minv,
                    const int* col_fact, const int* col_list, cx<R>* cbuf, int64_t ldc, cudaStream_t st) {
    if (k < 1 || k > LOWRANK_MAX || ncol < 1) return;
    lowrank_coef_kernel<R><<<ncol, LOWRANK_MAX, 0, st>>>(sd, nnode, k, ends, minv, col_fact, col_list, cbuf, ldc);
    GT_LAUNCH_CHECK();
    const int chunks = (int)std::min<int64_t>((nnode + 255) / 256, 304);
    lowrank_apply_kernel<R><<<dim3(chunks, ncol), 256, 0, st>>>(sd, nnode, k, w, col_fact, col_list, cbuf, ldc);
    GT_LAUNCH_CHECK();
}

// right-hand sides U e_j in factor order: column c = f * k + j (of the batch starting at c0) gets +1 at the
// factor index of branch j's end a and -1 at that of end b (ends that are not kept get nothing); s is zero
// on entry
template <typename R>
__global__ void lowrank_rhs_kernel(cx<R>* __restrict__ s, int64_t nfac, int c0, int ncol, int k,
                                   const int* __restrict__ ends, const int64_t* __restrict__ perm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncol) return;
    const int j = (c0 + q) % k;
    const int64_t fa = perm[ends[2 * j]], fb = perm[ends[2 * j + 1]];
    cx<R>* sc = s + (int64_t)q * nfac;
    if (fa >= 0) sc[fa] = mk<R>(R(1), R(0));
    if (fb >= 0) sc[fb] = mk<R>(R(-1), R(0));
}

// U^T W: g[c][i] = W_c[a_i] - W_c[b_i] for the ncol columns of w (node order) of one batch
__global__ void lowrank_gather_kernel(const c64* __restrict__ w, int64_t nnode, int ncol, int k,
                                      const int* __restrict__ ends, c64* __restrict__ g) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncol * k) return;
    const int c = q / k, i = q - c * k;
    const c64* wc = w + (int64_t)c * nnode;
    g[q] = wc[ends[2 * i]] - wc[ends[2 * i + 1]];
}

template <typename D, typename S>
__global__ void lowrank_convert_kernel(const cx<S>* __restrict__ a, cx<D>* __restrict__ b, int64_t n) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        b[q] = cvt<D>(a[q]);
}

template <typename R>
void launch_lowrank_rhs(cx<R>* s, int64_t nfac, int c0, int ncol, int k, const int* ends, const int64_t* perm,
                        cudaStream_t st) {
    lowrank_rhs_kernel<R><<<(ncol + 127) / 128, 128, 0, st>>>(s, nfac, c0, ncol, k, ends, perm);
    GT_LAUNCH_CHECK();
}
template void launch_lowrank_rhs<float>(c32*, int64_t, int, int, int, const int*, const int64_t*, cudaStream_t);
template void launch_lowrank_rhs<double>(c64*, int64_t, int, int, int, const int*, const int64_t*, cudaStream_t);

void launch_lowrank_gather(const c64* w, int64_t nnode, int ncol, int k, const int* ends, c64* g, cudaStream_t st) {
    lowrank_gather_kernel<<<(ncol * k + 127) / 128, 128, 0, st>>>(w, nnode, ncol, k, ends, g);
    GT_LAUNCH_CHECK();
}

void launch_lowrank_to32(const c64* a, c32* b, int64_t n, cudaStream_t st) {
    lowrank_convert_kernel<float, double><<<(int)std::min<int64_t>((n + 255) / 256, 1216), 256, 0, st>>>(a, b, n);
    GT_LAUNCH_CHECK();
}

void launch_lowrank_to64(const c32* a, c64* b, int64_t n, cudaStream_t st) {
    lowrank_convert_kernel<double, float><<<(int)std::min<int64_t>((n + 255) / 256, 1216), 256, 0, st>>>(a, b, n);
    GT_LAUNCH_CHECK();
}

template void launch_lowrank<float>(c32*, int64_t, int, int, const int*, const c32*, const c32*, const int*,
                                    const int*, c32*, int64_t, cudaStream_t);
template void launch_lowrank<double>(c64*, int64_t, int, int, const int*, const c64*, const c64*, const int*,
                                     const int*, c64*, int64_t, cudaStream_t);

}  // namespace gt
