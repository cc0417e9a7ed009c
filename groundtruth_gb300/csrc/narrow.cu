// Strips narrower than the pitch (GroundTruth: PlaneStack._widths, peec.py:1732-1820; Lp_matvec's correction,
// peec.py:2129-2132; the resistance over the strip's width, _impedances, peec.py:2150-2160).  The FFT passes
// treat every strip as a full square; the few strips whose copper is narrower (a neck, a partly covered
// border) get their corrections here, after the passes, as a sparse row list:
//     out[p] += z_k (1/w_p - 1) x[p] + j omega (dL_p x[p] + sum_q M[p,q] x[q])      (system product)
// with the sign flipped for a residual (rhs - K x) and without the resistance and j omega for L_p alone.  The
// same rows carry a split layer's face coupling (PlaneStack._twin_z, peec.py:2186-2197; the product's
// top[tw_a] += Z12 I[tw_b] and back, peec.py:3054-3056): out[p] += z_mut / width x[partner].
#include "kernels.h"

namespace gt {

// one thread per (row, column); grid (row chunks, columns)
template <typename R>
__global__ void __launch_bounds__(128) narrow_kernel(Narrow nw, const cx<R>* __restrict__ x, cx<R>* __restrict__ out,
                                                    int64_t ld, int S, const int* __restrict__ col_op,
                                                    const double* __restrict__ omega, const c64* __restrict__ zs,
                                                    const c64* __restrict__ zmut, int mode,
                                                    const int* __restrict__ col_list) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nw.nrow) return;
    const int col = col_list ? col_list[blockIdx.y] : blockIdx.y;
    const int op = col_op ? col_op[col] : 0;
    const cx<R>* xc = x + (int64_t)col * ld;
    const int64_t p = nw.pos[q];
    cx<R> acc = R(nw.dl[q]) * xc[p];
    for (int64_t e = nw.ptr[q]; e < nw.ptr[q + 1]; ++e) acc += R(nw.val[e]) * xc[nw.col[e]];
    cx<R> y;
    if (mode == 2) {
        y = acc;
    } else {
        const cx<R> z = cvt<R>(zs[(int64_t)op * S + nw.sheet[q]]);
        y = R(nw.rdelta[q]) * (z * xc[p]) + R(omega[op]) * jmul(acc);
        if (nw.rre) y += (R(nw.rre[q]) * z.re) * xc[p];           // a resistance factor: the real part only
        if (nw.partner && nw.partner[q] >= 0) {     // the face coupling of a split layer's two strips
            const cx<R> zm = cvt<R>(zmut[(int64_t)op * nw.ntw + nw.twin[q]]);
            y += R(nw.tw_fac[q]) * (zm * xc[nw.partner[q]]);
            if (nw.twre) y += (R(nw.twre[q]) * zm.re) * xc[nw.partner[q]];
        }
        if (mode == 1) y = zero<R>() - y;
    }
    out[(int64_t)col * ld + p] += y;
}

template <typename R>
void launch_narrow(const Narrow& nw, const cx<R>* x, cx<R>* out, int64_t ld, int ncol, int S, const int* col_op,
                   const double* omega, const c64* zs, const c64* zmut, int mode, const int* col_list,
                   cudaStream_t st) {
    if (nw.nrow == 0 || ncol < 1) return;
    narrow_kernel<R><<<dim3((unsigned)((nw.nrow + 127) / 128), ncol), 128, 0, st>>>(nw, x, out, ld, S, col_op, omega,
                                                                                   zs, zmut, mode, col_list);
    GT_LAUNCH_CHECK();
}

template void launch_narrow<float>(const Narrow&, const c32*, c32*, int64_t, int, int, const int*, const double*,
                                   const c64*, const c64*, int, const int*, cudaStream_t);
template void launch_narrow<double>(const Narrow&, const c64*, c64*, int64_t, int, int, const int*, const double*,
                                    const c64*, const c64*, int, const int*, cudaStream_t);

}  // namespace gt
