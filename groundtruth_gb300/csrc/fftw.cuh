// Warp-level FFTs of length 512 for the L_p passes, data held in registers.
//
// A row of 512 complex values is worked by one warp, 16 values per lane, as 512 = 16 x 32:
//   forward  X[k1 + 16 k2] = sum_t W32^(t k2) W512^(t k1) sum_r x[t + 32 r] W16^(r k1)
//            lane t holds x[t + 32 r] (r = 0..15): a 16-point DFT over r in registers, the twiddle
//            W512^(t k1), one exchange through the warp's shared-memory tile (16 x 32, rows padded to 33),
//            then lane k1 (of a half warp) takes a 32-point DFT over t in registers and holds X[k1 + 16 k2]
//            for k2 = 0..31 in natural order.
//   inverse  x[t + 32 r] = sum_k1 W16^(-r k1) W512^(-t k1) sum_k2 X[k1 + 16 k2] W32^(-t k2)
//            the same steps backwards: lane k1's 32-point inverse DFT over k2, the exchange, the twiddle
//            W512^(-t k1) by lane t, and its 16-point inverse DFT over k1.
// A warp carries two rows at once (lanes 0-15 and 16-31 take the 32-point DFTs of rows 0 and 1), so each
// exchange moves 2 x 512 values through 2 x 16 x 33 slots of shared memory: one store and one load per
// value and transform, against two of each for a radix-8 Stockham pass.  Nothing is shared between
// warps: __syncwarp() orders the exchanges and no block-wide barrier is taken.
//
// The register DFTs below take their inner twiddles W32^m (and W16, W8, W4 as its powers) from literal
// tables; the quarter and half turns are exact sign swaps.  The W512 twiddles are the host-computed FP64
// table rounded to the working precision (the one the Stockham passes use), combined from W^t, W^2t, W^4t,
// W^8t by at most three products, once per lane for both of its rows.
#pragma once
#include "common.cuh"

namespace gt {

// cos(2 pi i / 32), a literal once i is known at compile time (the unrolled loops make it so); sin(2 pi i / 32)
// is cos(2 pi (i - 8) / 32)
template <typename R> __device__ __forceinline__ R cos32(int i) {
    switch (i & 31) {
        case 0: return R(1.0);
        case 1: return R(9.80785280403230431e-01);
        case 2: return R(9.23879532511286738e-01);
        case 3: return R(8.31469612302545236e-01);
        case 4: return R(7.07106781186547573e-01);
        case 5: return R(5.55570233019602289e-01);
        case 6: return R(3.82683432365089837e-01);
        case 7: return R(1.95090322016128331e-01);
        case 8: return R(0.0);
        case 9: return R(-1.95090322016128193e-01);
        case 10: return R(-3.82683432365089726e-01);
        case 11: return R(-5.55570233019601956e-01);
        case 12: return R(-7.07106781186547462e-01);
        case 13: return R(-8.31469612302545347e-01);
        case 14: return R(-9.23879532511286738e-01);
        case 15: return R(-9.80785280403230431e-01);
        case 16: return R(-1.0);
        case 17: return R(-9.80785280403230431e-01);
        case 18: return R(-9.23879532511286850e-01);
        case 19: return R(-8.31469612302545458e-01);
        case 20: return R(-7.07106781186547684e-01);
        case 21: return R(-5.55570233019602178e-01);
        case 22: return R(-3.82683432365090337e-01);
        case 23: return R(-1.95090322016128664e-01);
        case 24: return R(0.0);
        case 25: return R(1.95090322016128304e-01);
        case 26: return R(3.82683432365090004e-01);
        case 27: return R(5.55570233019601845e-01);
        case 28: return R(7.07106781186547351e-01);
        case 29: return R(8.31469612302545236e-01);
        case 30: return R(9.23879532511286516e-01);
        case 31: return R(9.80785280403230320e-01);
    }
    return R(0);
}

// a * W_N^m with m known once the loops are unrolled (N divides 32): exact for the quarter turns
template <typename R, bool INV, int N>
__device__ __forceinline__ cx<R> wtw(cx<R> a, int m) {
    m &= N - 1;
    if (m == 0) return a;
    if (4 * m == N) return INV ? mk<R>(-a.im, a.re) : mk<R>(a.im, -a.re);
    if (2 * m == N) return mk<R>(-a.re, -a.im);
    if (4 * m == 3 * N) return INV ? mk<R>(a.im, -a.re) : mk<R>(-a.im, a.re);
    const int i = m * (32 / N);
    const R c = cos32<R>(i), s = cos32<R>(i - 8);
    // forward multiplies by c - j s, inverse by c + j s
    return INV ? mk<R>(a.re * c - a.im * s, a.im * c + a.re * s) : mk<R>(a.re * c + a.im * s, a.im * c - a.re * s);
}

template <typename R, bool INV> __device__ __forceinline__ void w4(cx<R>& a0, cx<R>& a1, cx<R>& a2, cx<R>& a3) {
    const cx<R> t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, d = a1 - a3;
    const cx<R> t3 = INV ? mk<R>(-d.im, d.re) : mk<R>(d.im, -d.re);
    a0 = t0 + t2;
    a1 = t1 + t3;
    a2 = t0 - t2;
    a3 = t1 - t3;
}

// N-point DFT (N = 4, 8, 16, 32) of v[0 .. N) in natural order, in place, as A x B with A = 4:
// X[ka + 4 kb] = sum_b W_N^(b ka) W_B^(b kb) sum_a v[B a + b] W_4^(a ka).  HALF: v[N/2 ..] are zero and
// not read.  LO: only X[0 .. N/2) are wanted (the rest are left undefined).
template <typename R, bool INV, int N, bool HALF = false, bool LO = false>
__device__ __forceinline__ void rdft(cx<R>* v) {
    if constexpr (N == 2) {
        const cx<R> a = v[0], b = HALF ? zero<R>() : v[1];
        v[0] = a + b;
        v[1] = a - b;
    } else if constexpr (N == 4) {
        if constexpr (HALF) {
            const cx<R> a = v[0], b = v[1];
            const cx<R> jb = INV ? mk<R>(-b.im, b.re) : mk<R>(b.im, -b.re);
            v[0] = a + b;
            v[1] = a + jb;
            v[2] = a - b;
            v[3] = a - jb;
        } else {
            w4<R, INV>(v[0], v[1], v[2], v[3]);
        }
    } else {
        constexpr int A = 4, B = N / 4;
        cx<R> u[N];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            // inputs v[B a + b], a = 0..3; with HALF only a < 2 are nonzero
            cx<R> a0 = v[b], a1 = v[B + b];
            cx<R> a2 = HALF ? zero<R>() : v[2 * B + b], a3 = HALF ? zero<R>() : v[3 * B + b];
            if constexpr (HALF) {
                const cx<R> ja1 = INV ? mk<R>(-a1.im, a1.re) : mk<R>(a1.im, -a1.re);
                u[b * A + 0] = a0 + a1;
                u[b * A + 1] = a0 + ja1;
                u[b * A + 2] = a0 - a1;
                u[b * A + 3] = a0 - ja1;
            } else {
                w4<R, INV>(a0, a1, a2, a3);
                u[b * A + 0] = a0;
                u[b * A + 1] = a1;
                u[b * A + 2] = a2;
                u[b * A + 3] = a3;
            }
        }
        // twiddle, then the B-point DFTs over b, one per ka; LO keeps ka + 4 kb < N/2, i.e. kb < B/2
#pragma unroll
        for (int ka = 0; ka < A; ++ka) {
            cx<R> t[B];
#pragma unroll
            for (int b = 0; b < B; ++b) t[b] = wtw<R, INV, N>(u[b * A + ka], b * ka);
            rdft<R, INV, B>(t);
#pragma unroll
            for (int kb = 0; kb < (LO ? B / 2 : B); ++kb) v[ka + A * kb] = t[kb];
        }
    }
}

// a * w for w the table entry, conjugated for the inverse
template <typename R, bool INV> __device__ __forceinline__ cx<R> twm(cx<R> a, cx<R> w) {
    return INV ? mk<R>(a.re * w.re + a.im * w.im, a.im * w.re - a.re * w.im) : a * w;
}

// v0[k] and v1[k] *= W512^(+-t k), k = 1..15 (the two rows a lane holds share its twiddles), from the table
// entries W^t, W^2t, W^4t, W^8t (tw: W512^m, m < 512); each power the product of at most four of them, made once
// as it is used
template <typename R, bool INV>
__device__ __forceinline__ void tw512_lane2(cx<R>* v0, cx<R>* v1, int t, const cx<R>* __restrict__ tw) {
    const cx<R> w1 = tw[t], w2 = tw[2 * t], w4 = tw[4 * t], w8 = tw[8 * t];
    v0[8] = twm<R, INV>(v0[8], w8);
    v1[8] = twm<R, INV>(v1[8], w8);
#pragma unroll
    for (int k = 1; k < 8; ++k) {
        cx<R> w = (k & 1) ? w1 : ((k & 2) ? w2 : w4);
        if ((k & 1) && (k & 2)) w = w * w2;
        if ((k & 3) && (k & 4)) w = w * w4;
        const cx<R> wh = w * w8;
        v0[k] = twm<R, INV>(v0[k], w);
        v1[k] = twm<R, INV>(v1[k], w);
        v0[k + 8] = twm<R, INV>(v0[k + 8], wh);
        v1[k + 8] = twm<R, INV>(v1[k + 8], wh);
    }
}

// the warp's exchange tile: two rows of 16 x 33 slots
constexpr int WX_ROW = 16 * 33;
constexpr int WX_SLOTS = 2 * WX_ROW;

// Forward 512-point FFT of two rows.  On entry lane t holds x_q[t + 32 r] in v[q][r] for rows q = 0, 1
// (HALF: only r < 8, the rows' upper halves zero).  On exit lane L = 16 q + k1 holds X_q[k1 + 16 k2] in
// u[k2], k2 = 0..31.
template <typename R, bool HALF>
__device__ __forceinline__ void fft512_fwd2(cx<R> (&v)[2][16], cx<R> (&u)[32], cx<R>* __restrict__ sx,
                                            const cx<R>* __restrict__ tw) {
    const int lane = threadIdx.x & 31;
    rdft<R, false, 16, HALF>(v[0]);
    rdft<R, false, 16, HALF>(v[1]);
    tw512_lane2<R, false>(v[0], v[1], lane, tw);
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) sx[q * WX_ROW + k1 * 33 + lane] = v[q][k1];
    __syncwarp();
    const int q = lane >> 4, k1 = lane & 15;
#pragma unroll
    for (int t = 0; t < 32; ++t) u[t] = sx[q * WX_ROW + k1 * 33 + t];
    __syncwarp();
    rdft<R, false, 32>(u);
}

// Inverse 512-point FFT of two rows, the reverse of fft512_fwd2: on entry lane L = 16 q + k1 holds
// X_q[k1 + 16 k2] in u[k2]; on exit lane t holds x_q[t + 32 r] in v[q][r] for r < 8 (LO) or r < 16.
template <typename R, bool LO>
__device__ __forceinline__ void fft512_inv2(cx<R> (&u)[32], cx<R> (&v)[2][16], cx<R>* __restrict__ sx,
                                            const cx<R>* __restrict__ tw) {
    const int lane = threadIdx.x & 31;
    rdft<R, true, 32>(u);
    {
        const int q = lane >> 4, k1 = lane & 15;
#pragma unroll
        for (int t = 0; t < 32; ++t) sx[q * WX_ROW + k1 * 33 + t] = u[t];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) v[q][k1] = sx[q * WX_ROW + k1 * 33 + lane];
    __syncwarp();
    tw512_lane2<R, true>(v[0], v[1], lane, tw);
    rdft<R, true, 16, false, LO>(v[0]);
    rdft<R, true, 16, false, LO>(v[1]);
}

}  // namespace gt
