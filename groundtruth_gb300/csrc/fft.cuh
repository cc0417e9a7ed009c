// Shared-memory FFTs for the L_p product.
//
// Rows of length P = 2^a or 3 * 2^a (a >= 3) are transformed in place in shared memory by Stockham
// autosort stages (radix 3 first when present, then radix 8, then one radix 2 or 4): a stage with radix R
// after stages of total length Ns reads element j + r P/R, multiplies by W_P^{(j mod Ns) r P/(Ns R)},
// takes the R-point DFT in registers and writes (j div Ns) Ns R + (j mod Ns) + r Ns; after the last stage
// the row is in natural order.  Each row is worked by a team of P/8 threads (one radix-8 butterfly per
// thread per stage; radix 4/2/3 stages give a thread 2/4/3 butterflies).  Every thread of the block
// passes every barrier.  Twiddles W_P^m = exp(-2 pi i m / P), m < P, come from a table computed on the
// host in FP64 (rounded once to the working precision).
#pragma once
#include "common.cuh"

namespace gt {

// Shared-memory index of row element i: one padding slot per 32 elements, so that the power-of-two
// strides of the Stockham stages fall on different banks.
__device__ __forceinline__ int spad(int i) { return i + (i >> 5); }
// row stride (elements) for rows of length P
__host__ __device__ __forceinline__ int srow(int P) { return P + (P >> 5) + 1; }

template <typename R> struct FftConst;
template <> struct FftConst<float> { static constexpr float h = 0.70710678118654752440f, s3 = 0.86602540378443864676f; };
template <> struct FftConst<double> { static constexpr double h = 0.70710678118654752440, s3 = 0.86602540378443864676; };

// multiply by -j (forward) or +j (inverse)
template <typename R, bool INV> __device__ __forceinline__ cx<R> mj(cx<R> a) {
    return INV ? mk<R>(-a.im, a.re) : mk<R>(a.im, -a.re);
}

template <typename R, bool INV> __device__ __forceinline__ void dft2(cx<R>* v) {
    cx<R> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
}

template <typename R, bool INV> __device__ __forceinline__ void dft4(cx<R>* v) {
    cx<R> t0 = v[0] + v[2], t1 = v[0] - v[2], t2 = v[1] + v[3], t3 = mj<R, INV>(v[1] - v[3]);
    v[0] = t0 + t2;
    v[1] = t1 + t3;
    v[2] = t0 - t2;
    v[3] = t1 - t3;
}

template <typename R, bool INV> __device__ __forceinline__ void dft3(cx<R>* v) {
    // W3 = -1/2 -+ j sqrt(3)/2
    const R s = INV ? FftConst<R>::s3 : -FftConst<R>::s3;
    cx<R> a = v[0], b = v[1], c = v[2];
    cx<R> sum = b + c, dif = b - c;
    v[0] = a + sum;
    cx<R> m = mk<R>(a.re - R(0.5) * sum.re, a.im - R(0.5) * sum.im);
    cx<R> r = mk<R>(-s * dif.im, s * dif.re);  // j s (b - c)
    v[1] = m + r;
    v[2] = m - r;
}

template <typename R, bool INV> __device__ __forceinline__ void dft8(cx<R>* v) {
    const R h = FftConst<R>::h;
    // split into even / odd, two 4-point DFTs, combine with W8^k
    cx<R> e[4] = {v[0], v[2], v[4], v[6]};
    cx<R> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<R, INV>(e);
    dft4<R, INV>(o);
    // W8^1 = h (1 -+ j), W8^2 = -+ j, W8^3 = h (-1 -+ j)
    cx<R> o1 = INV ? mk<R>(h * (o[1].re - o[1].im), h * (o[1].re + o[1].im))
                   : mk<R>(h * (o[1].re + o[1].im), h * (o[1].im - o[1].re));
    cx<R> o2 = mj<R, INV>(o[2]);
    cx<R> o3 = INV ? mk<R>(-h * (o[3].re + o[3].im), h * (o[3].re - o[3].im))
                   : mk<R>(h * (o[3].im - o[3].re), -h * (o[3].re + o[3].im));
    v[0] = e[0] + o[0];
    v[4] = e[0] - o[0];
    v[1] = e[1] + o1;
    v[5] = e[1] - o1;
    v[2] = e[2] + o2;
    v[6] = e[2] - o2;
    v[3] = e[3] + o3;
    v[7] = e[3] - o3;
}

// the same transforms when the upper half of the inputs is zero (v[RAD/2 ..] not read)
template <typename R, bool INV> __device__ __forceinline__ void dft4_h(cx<R>* v) {
    const cx<R> a = v[0], b = v[1], jb = mj<R, INV>(v[1]);
    v[0] = a + b;
    v[1] = a + jb;
    v[2] = a - b;
    v[3] = a - jb;
}

template <typename R, bool INV> __device__ __forceinline__ void dft8_h(cx<R>* v) {
    const R h = FftConst<R>::h;
    cx<R> e[4] = {v[0], v[2], zero<R>(), zero<R>()};
    cx<R> o[4] = {v[1], v[3], zero<R>(), zero<R>()};
    dft4_h<R, INV>(e);
    dft4_h<R, INV>(o);
    cx<R> o1 = INV ? mk<R>(h * (o[1].re - o[1].im), h * (o[1].re + o[1].im))
                   : mk<R>(h * (o[1].re + o[1].im), h * (o[1].im - o[1].re));
    cx<R> o2 = mj<R, INV>(o[2]);
    cx<R> o3 = INV ? mk<R>(-h * (o[3].re + o[3].im), h * (o[3].re - o[3].im))
                   : mk<R>(h * (o[3].im - o[3].re), -h * (o[3].re + o[3].im));
    v[0] = e[0] + o[0];
    v[4] = e[0] - o[0];
    v[1] = e[1] + o1;
    v[5] = e[1] - o1;
    v[2] = e[2] + o2;
    v[6] = e[2] - o2;
    v[3] = e[3] + o3;
    v[7] = e[3] - o3;
}

template <typename R, bool INV, int RAD> __device__ __forceinline__ void dftr_h(cx<R>* v) {
    if constexpr (RAD == 2) v[1] = v[0];
    else if constexpr (RAD == 4) dft4_h<R, INV>(v);
    else dft8_h<R, INV>(v);
}

template <typename R, bool INV, int RAD> __device__ __forceinline__ void dftr(cx<R>* v) {
    if constexpr (RAD == 2) dft2<R, INV>(v);
    else if constexpr (RAD == 3) dft3<R, INV>(v);
    else if constexpr (RAD == 4) dft4<R, INV>(v);
    else dft8<R, INV>(v);
}

// One Stockham stage on the calling team's row.  row: the row's first element; t: thread within the team.
template <typename R, bool INV, int RAD>
__device__ __forceinline__ void fft_stage(cx<R>* row, bool active, int P, int Ns, const cx<R>* __restrict__ tw,
                                          int team, int t) {
    constexpr int NB = (8 + RAD - 1) / RAD;
    const int nbf = P / RAD;
    const int stride = P / (Ns * RAD);
    cx<R> v[NB][RAD];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        int j = t + q * team;
        if (active && j < nbf) {
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[q][r] = row[spad(j + r * nbf)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        int j = t + q * team;
        if (active && j < nbf) {
            int k = j % Ns;
            if (k) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) {
                    cx<R> w = tw[k * r * stride];
                    if (INV) w.im = -w.im;
                    v[q][r] = v[q][r] * w;
                }
            }
            dftr<R, INV, RAD>(v[q]);
            int base = (j / Ns) * Ns * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; ++r) row[spad(base + r * Ns)] = v[q][r];
        }
    }
    __syncthreads();
}

// Transform one row per team in place.  All threads of the block call this.
template <typename R, bool INV>
__device__ void fft_row(cx<R>* row, bool active, int P, const cx<R>* __restrict__ tw, int team, int t) {
    int rest = P;
    int Ns = 1;
    if (rest % 3 == 0) {
        fft_stage<R, INV, 3>(row, active, P, Ns, tw, team, t);
        Ns *= 3;
        rest /= 3;
    }
    while (rest % 8 == 0) {
        fft_stage<R, INV, 8>(row, active, P, Ns, tw, team, t);
        Ns *= 8;
        rest /= 8;
    }
    if (rest == 4) fft_stage<R, INV, 4>(row, active, P, Ns, tw, team, t);
    else if (rest == 2) fft_stage<R, INV, 2>(row, active, P, Ns, tw, team, t);
}


// --- the same transform with the length known at compile time: every stride, plan step and index
// division constant-folds (the runtime form above serves the lengths without a specialisation).
// Pruning for the zero-padded convolution (P a power of two): HIN, the row's upper half is zero on input
// (the first stage reads only j + r P/RAD with r < RAD/2); HOUT, only the lower half of the output is
// wanted (the last stage, whose outputs are j + r P/RAD, computes and stores r < RAD/2 only).
template <typename R, bool INV, int RAD, int P, int NS, bool HIN, bool HOUT>
__device__ __forceinline__ void fft_stage_c(cx<R>* row, bool active, const cx<R>* __restrict__ tw, int t) {
    constexpr int TEAM = P / 8;
    constexpr int NB = (8 + RAD - 1) / RAD;
    constexpr int NBF = P / RAD;
    constexpr int STRIDE = P / (NS * RAD);
    constexpr int RIN = HIN ? RAD / 2 : RAD, ROUT = HOUT ? RAD / 2 : RAD;
    cx<R> v[NB][RAD];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int j = t + q * TEAM;
        if (active && j < NBF) {
#pragma unroll
            for (int r = 0; r < RIN; ++r) v[q][r] = row[spad(j + r * NBF)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const int j = t + q * TEAM;
        if (active && j < NBF) {
            const int k = j % NS;
            if (NS > 1 && k) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) {
                    cx<R> w = tw[k * r * STRIDE];
                    if (INV) w.im = -w.im;
                    v[q][r] = v[q][r] * w;
                }
            }
            if constexpr (HIN) dftr_h<R, INV, RAD>(v[q]);
            else dftr<R, INV, RAD>(v[q]);
            const int base = (j / NS) * NS * RAD + k;
#pragma unroll
            for (int r = 0; r < ROUT; ++r) row[spad(base + r * NS)] = v[q][r];
        }
    }
    __syncthreads();
}

template <typename R, bool INV, int P, int NS, bool HIN, bool HOUT>
__device__ __forceinline__ void fft_stages_c(cx<R>* row, bool active, const cx<R>* __restrict__ tw, int t) {
    constexpr int REST = P / NS;
    if constexpr (REST > 1) {
        constexpr int RAD = (NS == 1 && P % 3 == 0) ? 3 : (REST % 8 == 0 ? 8 : REST);
        constexpr bool first = NS == 1, last = REST == RAD, pow2 = (P & (P - 1)) == 0;
        fft_stage_c<R, INV, RAD, P, NS, HIN && first && pow2, HOUT && last && pow2>(row, active, tw, t);
        fft_stages_c<R, INV, P, NS * RAD, HIN, HOUT>(row, active, tw, t);
    }
}

// P = 0: the runtime form with length p (no pruning).  HIN / HOUT as for fft_stage_c.
template <typename R, bool INV, int P, bool HIN = false, bool HOUT = false>
__device__ __forceinline__ void fft_row_t(cx<R>* row, bool active, int p, const cx<R>* __restrict__ tw, int team, int t) {
    if constexpr (P == 0) fft_row<R, INV>(row, active, p, tw, team, t);
    else fft_stages_c<R, INV, P, 1, HIN, HOUT>(row, active, tw, t);
}

}  // namespace gt
