// The partial-inductance product and the strip rows of the system product, as three FFT passes per strip
// orientation over a batch of columns (GroundTruth: PlaneStack.Lp_matvec / _conv, peec.py:2054-2135, and
// the strip rows of _HostMath.matvec, peec.py:3043-3062).
//
// An orientation's currents are a grid (S, n0, n1) of the dense vector; the FFT grid is (P0, P1) with
// P >= 2n - 1 per axis, so the circular convolution equals the linear one on the grid.  P is even, so
// n <= P / 2: forward transforms see a zero upper half and inverse ones are read in their lower half only
// (the pruned stages of fft.cuh).
//   pass A  row FFTs (length P1) of the n0 rows, zero padded; written transposed T[col][s][c][i]
//   pass B  per pixel column c: column FFTs (length P0) of all sheets, the per-pixel S x S real spectrum
//           multiply-add (the quadrant mirrored: K(p0, p1) = Kq(min(p0, P0-p0), min(p1, P1-p1))), inverse
//           column FFTs; rows i < n0 written back in place
//   pass C  inverse row FFTs, then the fused epilogue on the strips:
//           out = R_t x + j w L_p x - (V[a] - V[b])     (or rhs - that, for residuals; or L_p x alone)
// The spectrum is stored (Q1, Q0, S, S) and pre-scaled by 1/(P0 P1).
#include <type_traits>

#include "common.cuh"
#include "fft.cuh"
#include "fftw.cuh"
#include "kernels.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdlib>

namespace gt {

constexpr int MAXS = 8;

template <typename R, int PL>
__global__ void __launch_bounds__(1024) lp_pass_a(const cx<R>* __restrict__ x, int64_t ldx, int64_t off, int S, int n0, int n1, int P1,
                          int rows, const cx<R>* __restrict__ tw, cx<R>* __restrict__ T, const int* __restrict__ col_list,
                          int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
    const int P = PL ? PL : P1;                  // compile-time when specialised
    const int stride = srow(P);
    const int i0 = blockIdx.x * rows;
    const int s = blockIdx.y;
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const cx<R>* xs = x + (int64_t)col * ldx + off + (int64_t)s * n0 * n1;
    // each team loads, transforms and keeps its own row
    const int team = P / 8;
    const int r = threadIdx.x / team, t = threadIdx.x - r * team;
    const int i = i0 + r;
    if (r < rows) {
        cx<R>* row = buf + r * stride;
        for (int j = t; j < P; j += team) row[spad(j)] = (i < n0 && j < n1) ? xs[(int64_t)i * n1 + j] : zero<R>();
    }
    __syncthreads();
    fft_row_t<R, false, PL, true, false>(buf + r * stride, r < rows, P, tw, team, t);
    // written transposed: rows (a power of two) consecutive entries per frequency column
    cx<R>* Ts = T + ((int64_t)blockIdx.z * S + s) * (int64_t)P * ldt;
    const int lr = __ffs(rows) - 1;
    for (int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
        const int c = idx >> lr, rr = idx & (rows - 1);
        if (i0 + rr < n0) Ts[(int64_t)c * ldt + i0 + rr] = buf[rr * stride + spad(c)];
    }
}

template <typename R, int PL>
__global__ void __launch_bounds__(1024) lp_pass_b(int S, int n0, int P0, int P1, int ncol, int bt, const R* __restrict__ spec,
                          const cx<R>* __restrict__ tw, cx<R>* __restrict__ T, int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
    const int P = PL ? PL : P0;                  // compile-time when specialised
    const int stride = srow(P);
    const int c = blockIdx.x;
    const int b0 = blockIdx.y * bt;
    const int nb = min(bt, ncol - b0);
    const int nrows = nb * S;
    // each team loads, transforms and stores its own rows (column b, sheet s): rows r0 + slot for r0 = 0,
    // nslot, ... (more rows than a block's threads hold teams for: six sheets at P = 2048)
    const int team = P / 8, nslot = blockDim.x / team;
    const int slot = threadIdx.x / team, t = threadIdx.x - slot * team;
    for (int r0 = 0; r0 < nrows; r0 += nslot) {
        const int row = r0 + slot;
        if (row < nrows) {
            const int rb = row / S, rs = row - rb * S;
            const cx<R>* Trow = T + (((int64_t)(b0 + rb) * S + rs) * P1 + c) * ldt;
            for (int p = t; p < P; p += team) buf[row * stride + spad(p)] = p < n0 ? Trow[p] : zero<R>();
        }
        __syncthreads();
        fft_row_t<R, false, PL, true, false>(buf + min(row, nrows - 1) * stride, row < nrows, P, tw, team, t);
    }
    // spectrum multiply-add over sheets, one (column, pixel) per thread iteration
    const int Q0 = P / 2 + 1;
    const int q1 = min(c, P1 - c);
    const R* Kc = spec + (int64_t)q1 * Q0 * S * S;
    for (int idx = threadIdx.x; idx < nb * P; idx += blockDim.x) {
        const int b = idx / P, p = idx - b * P;
        const int q0 = min(p, P - p);
        const R* K = Kc + (int64_t)q0 * S * S;
        cx<R> u[MAXS];
#pragma unroll
        for (int s = 0; s < MAXS; ++s)
            if (s < S) u[s] = buf[(b * S + s) * stride + spad(p)];
#pragma unroll
        for (int tt = 0; tt < MAXS; ++tt) {
            if (tt < S) {
                cx<R> acc = zero<R>();
#pragma unroll
                for (int s = 0; s < MAXS; ++s)
                    if (s < S) {
                        R k = __ldg(K + tt * S + s);
                        acc.re += k * u[s].re;
                        acc.im += k * u[s].im;
                    }
                buf[(b * S + tt) * stride + spad(p)] = acc;
            }
        }
    }
    __syncthreads();
    for (int r0 = 0; r0 < nrows; r0 += nslot) {
        const int row = r0 + slot;
        fft_row_t<R, true, PL, false, true>(buf + min(row, nrows - 1) * stride, row < nrows, P, tw, team, t);
        if (row < nrows) {
            const int rb = row / S, rs = row - rb * S;
            cx<R>* Trow = T + (((int64_t)(b0 + rb) * S + rs) * P1 + c) * ldt;
            for (int p = t; p < n0; p += team) Trow[p] = buf[row * stride + spad(p)];
        }
    }
}

// Pass B for P a power of 8 (all stages radix 8) with the spectrum multiply fused in registers.  A team of
// P / 8 threads takes one column b and all S sheets of it; thread t owns butterfly t of every stage.  The
// forward transform's last stage leaves thread t holding the pixels t + r P/8 (r < 8), exactly the inputs of
// the inverse transform's first stage, so the S x S multiply-add runs on registers between the two.  The
// first forward stage reads the (half-empty) column straight from T, the last inverse stage writes its lower
// half straight back; the stages between alternate two shared buffers (one barrier per stage).
__host__ __device__ constexpr int lp_srow(int P) { return P + (P >> 5) + 1; }

template <typename R, bool INV, int P, int NS, int S>
__device__ __forceinline__ void b8_stage(const cx<R>* src, cx<R>* dst, int t, const cx<R>* __restrict__ tw) {
    constexpr int NBF = P / 8, STRIDE = P / (NS * 8), ST = lp_srow(P);
    const int k = t % NS;
    const int base = (t / NS) * NS * 8 + k;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        cx<R> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = src[s * ST + spad(t + r * NBF)];
        if (k) {
#pragma unroll
            for (int r = 1; r < 8; ++r) {
                cx<R> w = tw[k * r * STRIDE];
                if (INV) w.im = -w.im;
                v[r] = v[r] * w;
            }
        }
        dft8<R, INV>(v);
#pragma unroll
        for (int r = 0; r < 8; ++r) dst[s * ST + spad(base + r * NS)] = v[r];
    }
}

// the stages with NS0 <= NS < NSEND, from buffer `cur` on; returns the buffer holding the result
template <typename R, bool INV, int P, int NS, int NSEND, int S>
__device__ __forceinline__ int b8_stages(cx<R>* b0, cx<R>* b1, int cur, int t, const cx<R>* __restrict__ tw) {
    if constexpr (NS < NSEND) {
        b8_stage<R, INV, P, NS, S>(cur ? b1 : b0, cur ? b0 : b1, t, tw);
        __syncthreads();
        return b8_stages<R, INV, P, NS * 8, NSEND, S>(b0, b1, 1 - cur, t, tw);
    } else {
        return cur;
    }
}

template <typename R, int P, int S>
__global__ void __launch_bounds__(512) lp_pass_b8(int n0, int P1, int ncol, int bt, const R* __restrict__ spec,
                                                  const cx<R>* __restrict__ tw, cx<R>* __restrict__ T, int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int TEAM = P / 8, NBF = P / 8, ST = lp_srow(P), Q0 = P / 2 + 1;
    const int c = blockIdx.x;
    const int tb = threadIdx.x / TEAM, t = threadIdx.x % TEAM;
    const int b = blockIdx.y * bt + tb;
    const bool act = b < ncol;
    cx<R>* b0 = reinterpret_cast<cx<R>*>(smem_raw) + tb * S * ST;
    cx<R>* b1 = reinterpret_cast<cx<R>*>(smem_raw) + (bt + tb) * S * ST;
    cx<R>* Trow = T + ((int64_t)min(b, ncol - 1) * S * P1 + c) * ldt;     // sheet s at + s * P1 * ldt
    cx<R> v[S][8];
    // forward stage 1 (NS = 1) from T: inputs t + r P/8, the upper half zero
#pragma unroll
    for (int s = 0; s < S; ++s) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int p = t + r * NBF;
            v[s][r] = (act && p < n0) ? Trow[(int64_t)s * P1 * ldt + p] : zero<R>();
        }
        dft8_h<R, false>(v[s]);
#pragma unroll
        for (int r = 0; r < 8; ++r) b0[s * ST + spad(t * 8 + r)] = v[s][r];
    }
    __syncthreads();
    int cur = b8_stages<R, false, P, 8, P / 8, S>(b0, b1, 0, t, tw);
    // forward last stage (NS = P/8): pixels t + r P/8 stay in registers
    {
        const cx<R>* src = cur ? b1 : b0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
#pragma unroll
            for (int r = 0; r < 8; ++r) v[s][r] = src[s * ST + spad(t + r * NBF)];
            if (t) {
#pragma unroll
                for (int r = 1; r < 8; ++r) v[s][r] = v[s][r] * tw[t * r];
            }
            dft8<R, false>(v[s]);
        }
    }
    // spectrum multiply-add over sheets at pixel (p, c), K(p, c) = Kq(min(p, P-p), min(c, P1-c))
    {
        const R* Kc = spec + (int64_t)min(c, P1 - c) * Q0 * S * S;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int p = t + r * NBF;
            const R* K = Kc + (int64_t)min(p, P - p) * S * S;
            cx<R> u[S];
#pragma unroll
            for (int s = 0; s < S; ++s) u[s] = v[s][r];
#pragma unroll
            for (int s = 0; s < S; ++s) {
                cx<R> acc = zero<R>();
#pragma unroll
                for (int q = 0; q < S; ++q) {
                    const R kk = __ldg(K + s * S + q);
                    acc.re += kk * u[q].re;
                    acc.im += kk * u[q].im;
                }
                v[s][r] = acc;
            }
        }
    }
    // inverse stage 1 (NS = 1) on the registers, into the buffer the last forward stage did not read
    {
        cx<R>* dst = cur ? b0 : b1;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            dft8<R, true>(v[s]);
#pragma unroll
            for (int r = 0; r < 8; ++r) dst[s * ST + spad(t * 8 + r)] = v[s][r];
        }
    }
    __syncthreads();
    cur = b8_stages<R, true, P, 8, P / 8, S>(b0, b1, 1 - cur, t, tw);
    // inverse last stage (NS = P/8): the lower half (r < 4) straight to T
    {
        const cx<R>* src = cur ? b1 : b0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            cx<R> w8[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) w8[r] = src[s * ST + spad(t + r * NBF)];
            if (t) {
#pragma unroll
                for (int r = 1; r < 8; ++r) {
                    cx<R> w = tw[t * r];
                    w.im = -w.im;
                    w8[r] = w8[r] * w;
                }
            }
            dft8<R, true>(w8);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int p = t + r * NBF;
                if (act && p < n0) Trow[(int64_t)s * P1 * ldt + p] = w8[r];
            }
        }
    }
}

// Pass B for P0 = 512 in FP32, one warp per pair of rows (fftw.cuh): the two sheets of a column (S = 2) or
// two columns of one sheet (S = 1).  The warp loads the rows' lower halves (i < n0 <= 256) straight from T,
// transforms them, multiplies by the S x S spectrum at its pixels (lane 16 s + k1 holds sheet s at
// p = k1 + 16 k2 and takes the other sheet's value from lane 16 (1 - s) + k1 by a shuffle), transforms
// back and stores the lower halves.  Warps share nothing but the block's spectrum reads (L1).
constexpr int BW_WARPS = 4;
#ifndef GT_BW_MINB
#define GT_BW_MINB 4        // blocks per SM the register budget is cut for (128 registers)
#endif

template <int S>
__global__ void __launch_bounds__(BW_WARPS * 32, GT_BW_MINB) lp_pass_bw(int n0, int P1, int ncol, const float* __restrict__ spec,
                                                            const c32* __restrict__ tw, c32* __restrict__ T, int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int P = 512, Q0 = P / 2 + 1, CPW = S == 2 ? 1 : 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    c32* sx = reinterpret_cast<c32*>(smem_raw) + warp * WX_SLOTS;
    const int c = blockIdx.x;
    const int b0 = (blockIdx.y * BW_WARPS + warp) * CPW;
    if (b0 >= ncol) return;                     // the whole warp leaves together
    c32* row[2];
    bool ok[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int b = S == 2 ? b0 : b0 + q, s = S == 2 ? q : 0;
        ok[q] = b < ncol;
        row[q] = T + (((int64_t)min(b, ncol - 1) * S + s) * P1 + c) * ldt;
    }
    c32 v[2][16];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int j = lane + 32 * r;
            v[q][r] = (ok[q] && j < n0) ? row[q][j] : zero<float>();
        }
    c32 u[32];
    fft512_fwd2<float, true>(v, u, sx, tw);
    const float* Kc = spec + (int64_t)min(c, P1 - c) * Q0 * S * S;
    const int k1 = lane & 15;
    if constexpr (S == 2) {
        const int s = lane >> 4;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2) {
            const int p = k1 + 16 * k2;
            const float2 kk = __ldg(reinterpret_cast<const float2*>(Kc + min(p, P - p) * 4 + 2 * s));
            c32 o;
            o.re = __shfl_xor_sync(0xffffffffu, u[k2].re, 16);
            o.im = __shfl_xor_sync(0xffffffffu, u[k2].im, 16);
            const c32 u0 = s ? o : u[k2], u1 = s ? u[k2] : o;
            u[k2] = mk<float>(kk.x * u0.re + kk.y * u1.re, kk.x * u0.im + kk.y * u1.im);
        }
    } else {
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2) {
            const int p = k1 + 16 * k2;
            const float kk = __ldg(Kc + min(p, P - p));
            u[k2] = kk * u[k2];
        }
    }
    fft512_inv2<float, true>(u, v, sx, tw);
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int j = lane + 32 * r;
            if (ok[q] && j < n0) row[q][j] = v[q][r];
        }
}

// Row passes for P1 = 512 in FP32 (n1 <= 256): a block of RW_WARPS warps takes RW_ROWS = 16 consecutive rows
// i0 .. i0+15 of one sheet of one column, two rows per warp (fftw.cuh).  The frequency columns pass through a
// shared tile [c][16] (rows padded to 17) so that each column c's 16 rows are one aligned 128-byte run of T
// (T's rows are ldt long, a multiple of 16: rows i >= n0 of the run are the transforms of zero rows, which no
// pass reads).  The tile takes the place of the warps' exchange tiles once every warp is done with its own.
constexpr int RW_WARPS = 8, RW_ROWS = 2 * RW_WARPS, RW_TS = RW_ROWS + 1;
#ifndef GT_RW_MINB
#define GT_RW_MINB 2        // blocks per SM the row passes' register budget is cut for
#endif
constexpr size_t RW_SMEM = (size_t)(RW_WARPS * WX_SLOTS > 512 * RW_TS ? RW_WARPS * WX_SLOTS : 512 * RW_TS) * sizeof(c32);

__global__ void __launch_bounds__(RW_WARPS * 32, GT_RW_MINB) lp_pass_aw(const c32* __restrict__ x, int64_t ldx, int64_t off, int S,
                                                               int n0, int n1, int ldt, const c32* __restrict__ tw,
                                                               c32* __restrict__ T, const int* __restrict__ col_list) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c32* sm = reinterpret_cast<c32*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * RW_ROWS, s = blockIdx.y;
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const c32* xs = x + (int64_t)col * ldx + off + (int64_t)s * n0 * n1;
    c32 v[2][16];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = i0 + 2 * warp + q;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int j = lane + 32 * r;
            v[q][r] = (i < n0 && j < n1) ? xs[(int64_t)i * n1 + j] : zero<float>();
        }
    }
    c32 u[32];
    fft512_fwd2<float, true>(v, u, sm + warp * WX_SLOTS, tw);
    __syncthreads();                               // every warp is past its exchange: the tile may reuse them
    {
        const int il = 2 * warp + (lane >> 4), k1 = lane & 15;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2) sm[(k1 + 16 * k2) * RW_TS + il] = u[k2];
    }
    __syncthreads();
    c32* Ts = T + ((int64_t)blockIdx.z * S + s) * 512 * ldt + i0;
    for (int idx = threadIdx.x; idx < 512 * (RW_ROWS / 2); idx += RW_WARPS * 32) {
        const int c = idx >> 3, m = idx & 7;
        const c32 a = sm[c * RW_TS + 2 * m], b = sm[c * RW_TS + 2 * m + 1];
        *reinterpret_cast<float4*>(Ts + (int64_t)c * ldt + 2 * m) = make_float4(a.re, a.im, b.re, b.im);
    }
}

// Pass C for P1 = 512 in FP32 (n1 <= 256): each warp takes two rows i, i+1 of one sheet of one column and
// reads them straight from T, with no block-wide staging: lane L loads the two rows' values at frequency
// columns c = L + 32 m (m < 16) as one 16-byte load each (rows i, i+1 are adjacent in T, i even), which gives it
// the k2 = L/16 + 2 m terms of k1 = L mod 16 (c = k1 + 16 k2) for both rows; one exchange with lane L ^ 16
// leaves lane 16 q + k1 holding row q at every k2, the inverse FFT's layout (fftw.cuh).  Warps are
// independent, so one warp's loads overlap another's transforms.
constexpr int CW_WARPS = 4;
#ifndef GT_CW_MINB
#define GT_CW_MINB 5        // blocks per SM the register budget is cut for (102 registers)
#endif
constexpr size_t CW_SMEM = (size_t)CW_WARPS * WX_SLOTS * sizeof(c32);

// mode 0: out = R_t x + j w L - (V[a] - V[b]); 1: out = rhs - (that); 2: out = L
__global__ void __launch_bounds__(CW_WARPS * 32, GT_CW_MINB) lp_pass_cw(const c32* __restrict__ T,
                                                               const c32* __restrict__ x,
                                                               const c32* __restrict__ rhs, c32* __restrict__ out,
                                                               int64_t ld, int64_t off, int64_t off_v, int S, int n0,
                                                               int n1, int nx, int ny, int di, int dj, int ldt,
                                                               const c32* __restrict__ tw, const uint8_t* __restrict__ mask,
                                                               const int* __restrict__ col_op,
                                                               const double* __restrict__ omega, const c64* __restrict__ zs,
                                                               int mode, const int* __restrict__ col_list,
                                                               const int* __restrict__ sheet_layer) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    c32* sm = reinterpret_cast<c32*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (blockIdx.x * CW_WARPS + warp) * 2, s = blockIdx.y;
    if (i >= n0) return;                           // the whole warp leaves together
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const c32* Ts = T + ((int64_t)blockIdx.z * S + s) * 512 * ldt + i;
    const int q = lane >> 4;
    c32 u[32];
    float4 f[16];                                  // every load in flight before the first exchange
#pragma unroll
    for (int m = 0; m < 16; ++m) f[m] = __ldg(reinterpret_cast<const float4*>(Ts + (int64_t)(lane + 32 * m) * ldt));
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        // mine: row q at k2 = q + 2m; the partner's: row q at k2 = 1 - q + 2m, for which it sends its row-q value
        const c32 r0 = mk<float>(f[m].x, f[m].y), r1 = mk<float>(f[m].z, f[m].w);
        const c32 mine = q ? r1 : r0, send = q ? r0 : r1;
        c32 got;
        got.re = __shfl_xor_sync(0xffffffffu, send.re, 16);
        got.im = __shfl_xor_sync(0xffffffffu, send.im, 16);
        u[2 * m] = q ? got : mine;
        u[2 * m + 1] = q ? mine : got;
    }
    c32 v[2][16];
    fft512_inv2<float, true>(u, v, sm + warp * WX_SLOTS, tw);
    const int op = col_op ? col_op[col] : 0;
    const float w = omega ? float(omega[op]) : 0.0f;
    const c32 z = zs ? cvt<float>(zs[(int64_t)op * S + s]) : zero<float>();
    const int64_t base = (int64_t)col * ld;
    const int layer = sheet_layer ? sheet_layer[s] : s;
#pragma unroll
    for (int qq = 0; qq < 2; ++qq) {
        const int ii = i + qq;
        if (ii >= n0) continue;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int j = lane + 32 * r;
            if (j >= n1) continue;
            const int64_t pos = off + ((int64_t)s * n0 + ii) * n1 + j;
            const c32 L = v[qq][r];
            c32 y;
            if (mode == 2) {
                y = mask[pos] ? L : zero<float>();
            } else if (!mask[pos]) {
                y = zero<float>();
            } else {
                const int64_t va = off_v + ((int64_t)layer * nx + ii) * ny + j;
                const int64_t vb = va + (int64_t)di * ny + dj;
                y = z * x[base + pos] + w * jmul(L) - (x[base + va] - x[base + vb]);
                if (mode == 1) y = rhs[base + pos] - y;
            }
            out[base + pos] = y;
        }
    }
}

// Pass C with its T tile brought in by TMA (P1 = 512, FP32).  A block of RW_WARPS warps takes 16 rows
// i0 .. i0+15 of one sheet of one column: one thread issues two cp.async.bulk.tensor loads of the tile
// [c = 0..511][16 rows] (two 256-row boxes of 128 bytes each, 128-byte swizzle) onto an mbarrier, so the whole
// 64 KB tile arrives as full 128-byte lines with no registers spent on it; each warp then reads its two rows'
// values at its lanes' frequency columns as 16-byte pieces (the swizzle puts the 8 columns a bank group
// serves on 8 different 16-byte chunks), and the tile's memory becomes the warps' FFT exchange tiles.
// T is viewed as a 2-D tensor of floats: x = 2 ldt (a row of T), y = (column slot x S + sheet) x 512 + c.
constexpr int CT_WARPS = RW_WARPS, CT_TILE_BYTES = 512 * 16 * 8;
constexpr size_t CT_SMEM = 1024 + (size_t)(CT_TILE_BYTES > RW_WARPS * WX_SLOTS * (int)sizeof(c32)
                                               ? CT_TILE_BYTES : RW_WARPS * WX_SLOTS * sizeof(c32));
constexpr uint64_t CT_WAIT_NS = 1000000000ull;     // a tile not in after a second counts as lost
constexpr uint32_t CT_SPIN_LIMIT = 1u << 26;        // and polls, should the timer not advance

__device__ unsigned int g_lp_wait_timeouts = 0;   // TMA waits that gave up (read and cleared by the host)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t wait_ns) {
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < CT_SPIN_LIMIT; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > wait_ns) return false;
    }
    return false;
}

__global__ void __launch_bounds__(CT_WARPS * 32, GT_RW_MINB) lp_pass_ct(const __grid_constant__ CUtensorMap tmap,
                                                                const c32* __restrict__ x,
                                                                const c32* __restrict__ rhs, c32* __restrict__ out,
                                                                int64_t ld, int64_t off, int64_t off_v, int S, int n0,
                                                                int n1, int nx, int ny, int di, int dj,
                                                                const c32* __restrict__ tw, const uint8_t* __restrict__ mask,
                                                                const int* __restrict__ col_op,
                                                                const double* __restrict__ omega, const c64* __restrict__ zs,
                                                                int mode, const int* __restrict__ col_list,
                                                                const int* __restrict__ sheet_layer,
                                                                uint32_t missing_bytes, uint64_t wait_ns) {
    // missing_bytes: 0, except when a test makes the wait run out (the barrier then expects bytes no load
    // brings; the loads themselves are the usual two)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    // the 128-byte swizzle repeats every 1024 bytes: the tile starts on a 1024-byte boundary
    unsigned char* tile = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * 16, s = blockIdx.y;
    const uint32_t b = smem_u32(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                     "r"(CT_TILE_BYTES + missing_bytes) : "memory");
        const int y0 = (blockIdx.z * S + s) * 512;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                         ::"r"(smem_u32(tile + h * (CT_TILE_BYTES / 2))), "l"(&tmap), "r"(2 * i0), "r"(y0 + 256 * h),
                         "r"(b) : "memory");
    }
    // while the tile is in flight: ask L2 for the lines the epilogue will read (the strips' x, the potentials
    // at both ends of each strip, the mask), so that they are on chip when the inverse FFT is done
    {
        const int ip = i0 + 2 * warp;
        const int colp = col_list ? col_list[blockIdx.z] : blockIdx.z;
        const int64_t basep = (int64_t)colp * ld;
        const int layerp = sheet_layer ? sheet_layer[s] : s;
#pragma unroll
        for (int qq = 0; qq < 2; ++qq) {
            const int ii = ip + qq;
            if (ii >= n0) continue;
            const int64_t row = off + ((int64_t)s * n0 + ii) * n1;
            const int j = 16 * lane;                         // lane L: the L-th 128-byte line (16 values) of a row
            if (j < n1) {
                const int64_t va = off_v + ((int64_t)layerp * nx + ii) * ny + j;
                if (mode != 2) {
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(x + basep + row + j));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(x + basep + va));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(x + basep + va + (int64_t)di * ny + dj));
                    if (mode == 1) asm volatile("prefetch.global.L2 [%0];" ::"l"(rhs + basep + row + j));
                }
            }
            if (128 * lane < n1) asm volatile("prefetch.global.L2 [%0];" ::"l"(mask + row + 128 * lane));
        }
    }
    if (!mbar_wait_bounded(b, 0, wait_ns)) {
        // the tile did not arrive: record it and leave once the copies in flight have landed (or given up on)
        if (threadIdx.x == 0) atomicAdd(&g_lp_wait_timeouts, 1u);
        mbar_wait_bounded(b, 0, wait_ns);
        return;
    }
    const int i = i0 + 2 * warp;
    const int q = lane >> 4;
    c32 u[32];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const int c = lane + 32 * m;
        // rows i, i+1 of column c: 16-byte chunk `warp` of the 128-byte line c, swizzled by c mod 8
        const float4 f = *reinterpret_cast<const float4*>(tile + c * 128 + ((warp ^ (c & 7)) << 4));
        const c32 r0 = mk<float>(f.x, f.y), r1 = mk<float>(f.z, f.w);
        const c32 mine = q ? r1 : r0, send = q ? r0 : r1;
        c32 got;
        got.re = __shfl_xor_sync(0xffffffffu, send.re, 16);
        got.im = __shfl_xor_sync(0xffffffffu, send.im, 16);
        u[2 * m] = q ? got : mine;
        u[2 * m + 1] = q ? mine : got;
    }
    __syncthreads();                               // every warp has its values: the tile becomes exchange tiles
    if (i >= n0) return;                           // the whole warp leaves together (no barrier follows)
    c32 v[2][16];
    fft512_inv2<float, true>(u, v, reinterpret_cast<c32*>(tile) + warp * WX_SLOTS, tw);
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const int op = col_op ? col_op[col] : 0;
    const float w = omega ? float(omega[op]) : 0.0f;
    const c32 z = zs ? cvt<float>(zs[(int64_t)op * S + s]) : zero<float>();
    const int64_t base = (int64_t)col * ld;
    const int layer = sheet_layer ? sheet_layer[s] : s;
#pragma unroll
    for (int qq = 0; qq < 2; ++qq) {
        const int ii = i + qq;
        if (ii >= n0) continue;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int j = lane + 32 * r;
            if (j >= n1) continue;
            const int64_t pos = off + ((int64_t)s * n0 + ii) * n1 + j;
            const c32 L = v[qq][r];
            c32 yv;
            if (mode == 2) {
                yv = mask[pos] ? L : zero<float>();
            } else if (!mask[pos]) {
                yv = zero<float>();
            } else {
                const int64_t va = off_v + ((int64_t)layer * nx + ii) * ny + j;
                const int64_t vb = va + (int64_t)di * ny + dj;
                yv = z * x[base + pos] + w * jmul(L) - (x[base + va] - x[base + vb]);
                if (mode == 1) yv = rhs[base + pos] - yv;
            }
            out[base + pos] = yv;
        }
    }
}

unsigned int lp_take_wait_timeouts() {
    unsigned int h = 0, zero_v = 0;
    GT_CUDA(cudaMemcpyFromSymbol(&h, g_lp_wait_timeouts, sizeof(h)));
    if (h) GT_CUDA(cudaMemcpyToSymbol(g_lp_wait_timeouts, &zero_v, sizeof(zero_v)));
    return h;
}

// Row passes for P a power of 8: the first stage of pass A reads the strip row straight from x, the last
// stage of pass C feeds the epilogue from registers; stages alternate two shared buffers.
template <typename R, int P>
__global__ void __launch_bounds__(1024) lp_pass_a8(const cx<R>* __restrict__ x, int64_t ldx, int64_t off, int S, int n0,
                                                   int n1, int rows, const cx<R>* __restrict__ tw, cx<R>* __restrict__ T,
                                                   const int* __restrict__ col_list, int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int TEAM = P / 8, NBF = P / 8, ST = lp_srow(P);
    cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
    const int i0 = blockIdx.x * rows;
    const int s = blockIdx.y;
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const int tr = threadIdx.x / TEAM, t = threadIdx.x % TEAM;
    const int i = i0 + tr;
    cx<R>* b0 = buf + tr * ST;
    cx<R>* b1 = buf + (rows + tr) * ST;
    const cx<R>* xrow = x + (int64_t)col * ldx + off + ((int64_t)s * n0 + min(i, n0 - 1)) * n1;
    {
        cx<R> v[8];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int j = t + r * NBF;
            v[r] = (i < n0 && j < n1) ? xrow[j] : zero<R>();
        }
        dft8_h<R, false>(v);
#pragma unroll
        for (int r = 0; r < 8; ++r) b0[spad(t * 8 + r)] = v[r];
    }
    __syncthreads();
    const int cur = b8_stages<R, false, P, 8, P / 8, 1>(b0, b1, 0, t, tw);
    // last stage: natural order into the other buffer, then the transposed store
    {
        const cx<R>* src = cur ? b1 : b0;
        cx<R>* dst = cur ? b0 : b1;
        cx<R> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = src[spad(t + r * NBF)];
        if (t) {
#pragma unroll
            for (int r = 1; r < 8; ++r) v[r] = v[r] * tw[t * r];
        }
        dft8<R, false>(v);
#pragma unroll
        for (int r = 0; r < 8; ++r) dst[spad(t + r * NBF)] = v[r];
    }
    __syncthreads();
    const cx<R>* res = buf + (cur ? 0 : rows) * ST;
    cx<R>* Ts = T + ((int64_t)blockIdx.z * S + s) * (int64_t)P * ldt;
    const int lr = __ffs(rows) - 1;
    for (int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
        const int c = idx >> lr, rr = idx & (rows - 1);
        if (i0 + rr < n0) Ts[(int64_t)c * ldt + i0 + rr] = res[rr * ST + spad(c)];
    }
}

template <typename R, int P>
__global__ void __launch_bounds__(1024) lp_pass_c8(const cx<R>* __restrict__ T, const cx<R>* __restrict__ x,
                                                   const cx<R>* __restrict__ rhs, cx<R>* __restrict__ out, int64_t ld,
                                                   int64_t off, int64_t off_v, int S, int n0, int n1, int nx, int ny,
                                                   int di, int dj, int rows, const cx<R>* __restrict__ tw,
                                                   const uint8_t* __restrict__ mask, const int* __restrict__ col_op,
                                                   const double* __restrict__ omega, const c64* __restrict__ zs, int mode,
                                                   const int* __restrict__ col_list, const int* __restrict__ sheet_layer,
                                                   int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int TEAM = P / 8, NBF = P / 8, ST = lp_srow(P);
    cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
    const int i0 = blockIdx.x * rows;
    const int s = blockIdx.y;
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const cx<R>* Ts = T + ((int64_t)blockIdx.z * S + s) * (int64_t)P * ldt;
    const int lr = __ffs(rows) - 1;
    for (int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
        const int c = idx >> lr, rr = idx & (rows - 1);
        const int i = i0 + rr;
        buf[rr * ST + spad(c)] = i < n0 ? Ts[(int64_t)c * ldt + i] : zero<R>();
    }
    __syncthreads();
    const int tr = threadIdx.x / TEAM, t = threadIdx.x % TEAM;
    cx<R>* b0 = buf + tr * ST;
    cx<R>* b1 = buf + (rows + tr) * ST;
    // first inverse stage (NS = 1) from the natural-order row into the second buffer
    {
        cx<R> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = b0[spad(t + r * NBF)];
        dft8<R, true>(v);
#pragma unroll
        for (int r = 0; r < 8; ++r) b1[spad(t * 8 + r)] = v[r];
    }
    __syncthreads();
    const int cur = b8_stages<R, true, P, 8, P / 8, 1>(b0, b1, 1, t, tw);
    cx<R> L[4];
    {
        const cx<R>* src = cur ? b1 : b0;
        cx<R> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = src[spad(t + r * NBF)];
        if (t) {
#pragma unroll
            for (int r = 1; r < 8; ++r) {
                cx<R> w = tw[t * r];
                w.im = -w.im;
                v[r] = v[r] * w;
            }
        }
        dft8<R, true>(v);
#pragma unroll
        for (int r = 0; r < 4; ++r) L[r] = v[r];
    }
    const int i = i0 + tr;
    if (tr >= rows || i >= n0) return;
    const int op = col_op ? col_op[col] : 0;
    const R w = omega ? R(omega[op]) : R(0);
    const cx<R> z = zs ? cvt<R>(zs[(int64_t)op * S + s]) : zero<R>();
    const int64_t base = (int64_t)col * ld;
    const int layer = sheet_layer ? sheet_layer[s] : s;     // the nodes a face sheet's strips join
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int j = t + r * NBF;
        if (j >= n1) continue;
        const int64_t pos = off + ((int64_t)s * n0 + i) * n1 + j;
        cx<R> y;
        if (mode == 2) {
            y = mask[pos] ? L[r] : zero<R>();
        } else if (!mask[pos]) {
            y = zero<R>();
        } else {
            const cx<R> xv = x[base + pos];
            const int64_t va = off_v + ((int64_t)layer * nx + i) * ny + j;
            const int64_t vb = va + (int64_t)di * ny + dj;
            const cx<R> dv = x[base + va] - x[base + vb];
            y = z * xv + w * jmul(L[r]) - dv;
            if (mode == 1) y = rhs[base + pos] - y;
        }
        out[base + pos] = y;
    }
}

// mode 0: out = R_t x + j w L - (V[a] - V[b]); 1: out = rhs - (that); 2: out = L
template <typename R, int PL>
__global__ void __launch_bounds__(1024) lp_pass_c(const cx<R>* __restrict__ T, const cx<R>* __restrict__ x, const cx<R>* __restrict__ rhs,
                          cx<R>* __restrict__ out, int64_t ld, int64_t off, int64_t off_v, int S, int n0, int n1,
                          int nx, int ny, int di, int dj, int P1, int rows, const cx<R>* __restrict__ tw,
                          const uint8_t* __restrict__ mask, const int* __restrict__ col_op,
                          const double* __restrict__ omega, const c64* __restrict__ zs, int mode,
                          const int* __restrict__ col_list, const int* __restrict__ sheet_layer, int ldt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
    const int P = PL ? PL : P1;                  // compile-time when specialised
    const int stride = srow(P);
    const int i0 = blockIdx.x * rows;
    const int s = blockIdx.y;
    const int col = col_list ? col_list[blockIdx.z] : blockIdx.z;
    const cx<R>* Ts = T + ((int64_t)blockIdx.z * S + s) * (int64_t)P * ldt;
    const int lr = __ffs(rows) - 1;
    for (int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
        const int c = idx >> lr, rr = idx & (rows - 1);
        const int i = i0 + rr;
        buf[rr * stride + spad(c)] = i < n0 ? Ts[(int64_t)c * ldt + i] : zero<R>();
    }
    __syncthreads();
    const int team = P / 8;
    const int r = threadIdx.x / team, t = threadIdx.x - r * team;
    fft_row_t<R, true, PL, false, true>(buf + r * stride, r < rows, P, tw, team, t);
    const int op = col_op ? col_op[col] : 0;
    const R w = omega ? R(omega[op]) : R(0);
    const cx<R> z = zs ? cvt<R>(zs[(int64_t)op * S + s]) : zero<R>();
    const int64_t base = (int64_t)col * ld;
    // each team finishes its own row
    const int i = i0 + r;
    if (r >= rows || i >= n0) return;
    const int layer = sheet_layer ? sheet_layer[s] : s;
    for (int j = t; j < n1; j += team) {
        int64_t pos = off + ((int64_t)s * n0 + i) * n1 + j;
        cx<R> L = buf[r * stride + spad(j)];
        cx<R> y;
        if (mode == 2) {
            y = mask[pos] ? L : zero<R>();
        } else if (!mask[pos]) {
            y = zero<R>();
        } else {
            cx<R> xv = x[base + pos];
            int64_t va = off_v + ((int64_t)layer * nx + i) * ny + j;
            int64_t vb = va + (int64_t)di * ny + dj;
            cx<R> dv = x[base + va] - x[base + vb];
            y = z * xv + w * jmul(L) - dv;
            if (mode == 1) y = rhs[base + pos] - y;
        }
        out[base + pos] = y;
    }
}

// ------------------------------------------------------------------------------------------ launchers
template <typename R> static int ldt_of(const LpArgs<R>& a) { return a.ldt > 0 ? a.ldt : a.n0; }
template <typename R> static bool b8_fits(const LpArgs<R>& a);
template <typename R>
static void set_smem(const void* fn, size_t bytes) { raise_smem(fn, bytes); }

template <typename R>
void lp_shapes(const LpArgs<R>& a, int* rows_out, int* bt_out) {
    const int teamA = a.P1 / 8, teamB = a.P0 / 8;
    int rows = a.rows > 0 ? a.rows : 4;
    while (rows & (rows - 1)) rows &= rows - 1;     // the row passes index rows by shifts: a power of two
    const size_t nbufA = (a.P1 == 64 || a.P1 == 512) ? 2 : 1;   // the power-of-8 row passes double-buffer
    while (rows > 1 && (rows * teamA > 1024 || nbufA * rows * srow(a.P1) * sizeof(cx<R>) > 160 * 1024)) rows /= 2;
    int bt = a.bt > 0 ? a.bt : 2;
    const size_t nbuf = b8_fits(a) ? 2 : 1;       // the fused column pass double-buffers its rows
    const int per_col = b8_fits(a) ? teamB : a.S * teamB;
    while (bt > 1 && (bt * per_col > 512 * (b8_fits(a) ? 1 : 2) ||
                      nbuf * bt * a.S * srow(a.P0) * sizeof(cx<R>) > 160 * 1024)) bt /= 2;
    *rows_out = rows;
    *bt_out = bt;
}

// the specialised lengths; others run the runtime-length kernels
#define GT_LP_LENGTHS(X) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(1536) X(2048)

// the warp row passes apply for P1 = 512 in FP32 with T's rows a multiple of 16
template <typename R> static bool rw_fits(const LpArgs<R>& a) {
    return std::is_same<R, float>::value && a.P1 == 512 && a.n1 <= 256 && a.ldt > 0 && a.ldt % 16 == 0;
}

template <typename R, int PA>
static void launch_a(const LpArgs<R>& a, int rows, cudaStream_t st) {
    if constexpr (PA == 512 && std::is_same<R, float>::value) {
        if (rw_fits(a)) {
            set_smem<float>((const void*)lp_pass_aw, RW_SMEM);
            lp_pass_aw<<<dim3(ceil_div(a.n0, RW_ROWS), a.S, a.ncol), RW_WARPS * 32, RW_SMEM, st>>>(
                a.x, a.ld, a.off, a.S, a.n0, a.n1, a.ldt, a.tw1, a.T, a.col_list);
            GT_LAUNCH_CHECK();
            return;
        }
    }
    if constexpr (PA == 64 || PA == 512) {
        const size_t sm = (size_t)2 * rows * lp_srow(PA) * sizeof(cx<R>);
        set_smem<R>((const void*)lp_pass_a8<R, PA>, sm);
        lp_pass_a8<R, PA><<<dim3(ceil_div(a.n0, rows), a.S, a.ncol), rows * (PA / 8), sm, st>>>(
            a.x, a.ld, a.off, a.S, a.n0, a.n1, rows, a.tw1, a.T, a.col_list, ldt_of(a));
        GT_LAUNCH_CHECK();
        return;
    }
    size_t smA = (size_t)rows * srow(a.P1) * sizeof(cx<R>);
    dim3 gA(ceil_div(a.n0, rows), a.S, a.ncol);
    set_smem<R>((const void*)lp_pass_a<R, PA>, smA);
    lp_pass_a<R, PA><<<gA, rows * (a.P1 / 8), smA, st>>>(a.x, a.ld, a.off, a.S, a.n0, a.n1, a.P1, rows, a.tw1, a.T,
                                                          a.col_list, ldt_of(a));
    GT_LAUNCH_CHECK();
}

template <typename R, int P, int S>
static void launch_b8(const LpArgs<R>& a, int bt, cudaStream_t st) {
    const size_t sm = (size_t)2 * bt * S * lp_srow(P) * sizeof(cx<R>);
    set_smem<R>((const void*)lp_pass_b8<R, P, S>, sm);
    lp_pass_b8<R, P, S><<<dim3(a.P1, ceil_div(a.ncol, bt)), bt * (P / 8), sm, st>>>(a.n0, a.P1, a.ncol, bt, a.spec, a.tw0,
                                                                                  a.T, ldt_of(a));
    GT_LAUNCH_CHECK();
}

// the fused column pass applies for these lengths and sheet counts
template <typename R> static bool b8_fits(const LpArgs<R>& a) { return (a.P0 == 64 || a.P0 == 512) && a.S >= 1 && a.S <= 4; }

template <int S>
static void launch_bw(const LpArgs<float>& a, cudaStream_t st) {
    constexpr int CPW = S == 2 ? 1 : 2;
    const size_t sm = (size_t)BW_WARPS * WX_SLOTS * sizeof(c32);
    set_smem<float>((const void*)lp_pass_bw<S>, sm);
    lp_pass_bw<S><<<dim3(a.P1, ceil_div(a.ncol, BW_WARPS * CPW)), BW_WARPS * 32, sm, st>>>(a.n0, a.P1, a.ncol, a.spec,
                                                                                         a.tw0, a.T, ldt_of(a));
    GT_LAUNCH_CHECK();
}

template <typename R, int PB>
static void launch_b(const LpArgs<R>& a, int bt, cudaStream_t st) {
    if constexpr (PB == 512 && std::is_same<R, float>::value) {
        if (a.n0 <= PB / 2 && a.S <= 2) {
            if (a.S == 2) launch_bw<2>(a, st);
            else launch_bw<1>(a, st);
            return;
        }
    }
    if constexpr (PB == 64 || PB == 512) {
        if (b8_fits(a)) {
            switch (a.S) {
                case 1: launch_b8<R, PB, 1>(a, bt, st); return;
                case 2: launch_b8<R, PB, 2>(a, bt, st); return;
                case 3: launch_b8<R, PB, 3>(a, bt, st); return;
                default: launch_b8<R, PB, 4>(a, bt, st); return;
            }
        }
    }
    size_t smB = (size_t)bt * a.S * srow(a.P0) * sizeof(cx<R>);
    dim3 gB(a.P1, ceil_div(a.ncol, bt));
    const int team = a.P0 / 8, threads = std::min(bt * a.S, 1024 / team) * team;
    set_smem<R>((const void*)lp_pass_b<R, PB>, smB);
    lp_pass_b<R, PB><<<gB, threads, smB, st>>>(a.S, a.n0, a.P0, a.P1, a.ncol, bt, a.spec, a.tw0, a.T, ldt_of(a));
    GT_LAUNCH_CHECK();
}

// cuTensorMapEncodeTiled from the driver (no link against libcuda: the runtime hands out its entry point)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// pass C through TMA tiles unless GT_LP_TMA=0 (the per-warp 16-byte loads of lp_pass_cw instead; both compute
// the same values in the same order)
static bool lp_tma_enabled() {
    const char* e = std::getenv("GT_LP_TMA");
    return !(e && e[0] == '0') && tensor_map_encoder() != nullptr;
}

// T as a 2-D float tensor: rows of 2 ldt floats, ncol x S x 512 of them; boxes of 16 complex values x 256
// frequency columns, 128-byte swizzle
static CUtensorMap t_tensor_map(const LpArgs<float>& a) {
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)2 * a.ldt, (cuuint64_t)a.ncol * a.S * 512};
    const cuuint64_t strides[1] = {(cuuint64_t)a.ldt * sizeof(c32)};
    const cuuint32_t box[2] = {32, 256}, estr[2] = {1, 1};
    const CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)a.T, dims, strides, box, estr,
                                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw CudaError{cudaErrorInvalidValue, "cuTensorMapEncodeTiled of the FFT grid T"};
    return m;
}

template <typename R, int PA>
static void launch_c(const LpArgs<R>& a, int rows, cudaStream_t st) {
    if constexpr (PA == 512 && std::is_same<R, float>::value) {
        // TMA wants T 16-byte aligned, its rows a multiple of 16 bytes (ldt % 16 == 0 gives 128) and each box's
        // first float at a multiple of 16 bytes (2 x 16 i0 floats)
        if (rw_fits(a) && lp_tma_enabled() && (reinterpret_cast<uintptr_t>(a.T) & 15) == 0) {
            const CUtensorMap m = t_tensor_map(a);
            // GT_LP_TMA_TEST_SHORTFALL=1 (tests only): the barrier waits for 16 bytes that never come, with a
            // 1 ms limit, so that the GT_TIMEOUT path runs without a lost load
            const char* t = std::getenv("GT_LP_TMA_TEST_SHORTFALL");
            const bool shortfall = t && t[0] == '1';
            set_smem<float>((const void*)lp_pass_ct, CT_SMEM);
            lp_pass_ct<<<dim3(ceil_div(a.n0, 16), a.S, a.ncol), CT_WARPS * 32, CT_SMEM, st>>>(
                m, a.x, a.rhs, a.out, a.ld, a.off, a.off_v, a.S, a.n0, a.n1, a.nx, a.ny, a.di, a.dj, a.tw1, a.mask,
                a.col_op, a.omega, a.zs, a.mode, a.col_list, a.sheet_layer, shortfall ? 16u : 0u,
                shortfall ? 1000000ull : CT_WAIT_NS);
            GT_LAUNCH_CHECK();
            return;
        }
        if (rw_fits(a)) {
            set_smem<float>((const void*)lp_pass_cw, CW_SMEM);
            lp_pass_cw<<<dim3(ceil_div(a.n0, 2 * CW_WARPS), a.S, a.ncol), CW_WARPS * 32, CW_SMEM, st>>>(
                a.T, a.x, a.rhs, a.out, a.ld, a.off, a.off_v, a.S, a.n0, a.n1, a.nx, a.ny, a.di, a.dj, a.ldt, a.tw1,
                a.mask, a.col_op, a.omega, a.zs, a.mode, a.col_list, a.sheet_layer);
            GT_LAUNCH_CHECK();
            return;
        }
    }
    if constexpr (PA == 64 || PA == 512) {
        const size_t sm = (size_t)2 * rows * lp_srow(PA) * sizeof(cx<R>);
        set_smem<R>((const void*)lp_pass_c8<R, PA>, sm);
        lp_pass_c8<R, PA><<<dim3(ceil_div(a.n0, rows), a.S, a.ncol), rows * (PA / 8), sm, st>>>(
            a.T, a.x, a.rhs, a.out, a.ld, a.off, a.off_v, a.S, a.n0, a.n1, a.nx, a.ny, a.di, a.dj, rows, a.tw1, a.mask,
            a.col_op, a.omega, a.zs, a.mode, a.col_list, a.sheet_layer, ldt_of(a));
        GT_LAUNCH_CHECK();
        return;
    }
    size_t smA = (size_t)rows * srow(a.P1) * sizeof(cx<R>);
    dim3 gA(ceil_div(a.n0, rows), a.S, a.ncol);
    set_smem<R>((const void*)lp_pass_c<R, PA>, smA);
    lp_pass_c<R, PA><<<gA, rows * (a.P1 / 8), smA, st>>>(a.T, a.x, a.rhs, a.out, a.ld, a.off, a.off_v, a.S, a.n0, a.n1,
                                                          a.nx, a.ny, a.di, a.dj, a.P1, rows, a.tw1, a.mask, a.col_op,
                                                          a.omega, a.zs, a.mode, a.col_list, a.sheet_layer, ldt_of(a));
    GT_LAUNCH_CHECK();
}

template <typename R>
void launch_lp_pass(const LpArgs<R>& a, int pass, cudaStream_t st) {
    int rows, bt;
    lp_shapes<R>(a, &rows, &bt);
    if (pass == 0) {
        switch (a.P1) {
#define GT_CASE(L) \
    case L: launch_a<R, L>(a, rows, st); break;
            GT_LP_LENGTHS(GT_CASE)
#undef GT_CASE
            default: launch_a<R, 0>(a, rows, st);
        }
    } else if (pass == 1) {
        switch (a.P0) {
#define GT_CASE(L) \
    case L: launch_b<R, L>(a, bt, st); break;
            GT_LP_LENGTHS(GT_CASE)
#undef GT_CASE
            default: launch_b<R, 0>(a, bt, st);
        }
    } else {
        switch (a.P1) {
#define GT_CASE(L) \
    case L: launch_c<R, L>(a, rows, st); break;
            GT_LP_LENGTHS(GT_CASE)
#undef GT_CASE
            default: launch_c<R, 0>(a, rows, st);
        }
    }
}

template <typename R>
void launch_lp(const LpArgs<R>& a, cudaStream_t st) {
    for (int pass = 0; pass < 3; ++pass) launch_lp_pass<R>(a, pass, st);
}

template void launch_lp<float>(const LpArgs<float>&, cudaStream_t);
template void launch_lp_pass<float>(const LpArgs<float>&, int, cudaStream_t);
template void launch_lp_pass<double>(const LpArgs<double>&, int, cudaStream_t);
template void launch_lp<double>(const LpArgs<double>&, cudaStream_t);
template void lp_shapes<float>(const LpArgs<float>&, int*, int*);
template void lp_shapes<double>(const LpArgs<double>&, int*, int*);

}  // namespace gt
