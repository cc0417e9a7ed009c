// Krylov vector work of the restarted GMRES (GroundTruth: _gmres, peec.py:3093-3224; the device twin of
// gpu.TorchVectors, gpu.py:409-462), batched over slots (one basis per column being solved).
//
// Classical Gram-Schmidt with one conditional re-orthogonalisation (DGKS: a second pass when the norm fell
// below 0.7 of the product's, peec.py:3156-3159).  Dot products are reduced per warp by shuffles, per block
// through shared memory in FP64, and across blocks by a second FP64 pass over per-block partials (fixed
// order: results are reproducible).  The Hessenberg column, its Givens rotations and the least-squares
// right-hand side live on the device in FP64 (peec.py:3160-3184); so does the decision that a slot's cycle
// has converged.
#include <type_traits>
#include "kernels.h"
#include "solver.h"

namespace gt {

template <typename R> __device__ __forceinline__ R shfl_sum(R v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// basis entries: loads and stores of cx<R> or of FP16 pairs
template <typename R> __device__ __forceinline__ cx<R> bload(const cx<R>* p) { return *p; }
__device__ __forceinline__ c32 bload(const h16c* p) {
    const float2 f = __half22float2(p->v);
    return mk<float>(f.x, f.y);
}
template <typename R> __device__ __forceinline__ void bstore(cx<R>* p, cx<R> v) { *p = v; }
__device__ __forceinline__ void bstore(h16c* p, c32 v) { p->v = __floats2half2_rn(v.re, v.im); }

constexpr int DOT_THREADS = 256;
constexpr int DOT_EPT = 8;
constexpr int DOT_CHUNK = DOT_THREADS * DOT_EPT;
// the update keeps fewer elements per thread (more blocks resident, several basis vectors in flight)
constexpr int UPD_EPT = 4;
constexpr int UPD_CHUNK = DOT_THREADS * UPD_EPT;

int update_chunks(int64_t n) { return (int)((n + UPD_CHUNK - 1) / UPD_CHUNK); }
constexpr int MAXV = 256;

// partial[(slot * nchunk + chunk) * (nv + 1) + i] = sum over the chunk of conj(V_i) w, i < nv; index nv: |w|^2
template <typename R, typename B>
__global__ void __launch_bounds__(DOT_THREADS) dots_kernel(const B* __restrict__ V, int64_t ldv, int64_t lds, int nv,
                                                           const cx<R>* __restrict__ w, int64_t ldw, int64_t n,
                                                           const int* __restrict__ active, c64* __restrict__ partial,
                                                           int nchunk, R vs) {
    __shared__ c64 red[DOT_THREADS / 32][MAXV + 1];
    const int slot = blockIdx.y;
    if (active && !active[slot]) return;
    const int chunk = blockIdx.x;
    const int64_t base = (int64_t)chunk * DOT_CHUNK;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    cx<R> wv[DOT_EPT];
    R nrm = 0;
#pragma unroll
    for (int e = 0; e < DOT_EPT; ++e) {
        int64_t q = base + e * DOT_THREADS + tid;
        wv[e] = q < n ? w[(int64_t)slot * ldw + q] : zero<R>();
        nrm += norm2(wv[e]);
    }
    const B* Vs = V + (int64_t)slot * lds;
    int i = 0;
    // full chunks: UN basis vectors' loads in flight together (FP32 arithmetic; FP64 keeps one)
    constexpr int UN = sizeof(R) == 4 ? 2 : 1;
    if (base + DOT_CHUNK <= n) {
        for (; i + UN <= nv; i += UN) {
            cx<R> v[UN][DOT_EPT];
#pragma unroll
            for (int u = 0; u < UN; ++u)
#pragma unroll
                for (int e = 0; e < DOT_EPT; ++e) v[u][e] = bload(Vs + (int64_t)(i + u) * ldv + base + e * DOT_THREADS + tid);
#pragma unroll
            for (int u = 0; u < UN; ++u) {
                R ar = 0, ai = 0;
#pragma unroll
                for (int e = 0; e < DOT_EPT; ++e) {
                    ar += v[u][e].re * wv[e].re + v[u][e].im * wv[e].im;
                    ai += v[u][e].re * wv[e].im - v[u][e].im * wv[e].re;
                }
                ar = shfl_sum(ar);
                ai = shfl_sum(ai);
                if (lane == 0) red[warp][i + u] = mk<double>((double)ar * vs, (double)ai * vs);
            }
        }
    }
    for (; i < nv; ++i) {
        const B* Vi = Vs + (int64_t)i * ldv;
        R ar = 0, ai = 0;
#pragma unroll
        for (int e = 0; e < DOT_EPT; ++e) {
            int64_t q = base + e * DOT_THREADS + tid;
            cx<R> v = q < n ? bload(Vi + q) : zero<R>();
            ar += v.re * wv[e].re + v.im * wv[e].im;
            ai += v.re * wv[e].im - v.im * wv[e].re;
        }
        ar = shfl_sum(ar);
        ai = shfl_sum(ai);
        if (lane == 0) red[warp][i] = mk<double>((double)ar * vs, (double)ai * vs);
    }
    nrm = shfl_sum(nrm);
    if (lane == 0) red[warp][nv] = mk<double>(nrm, 0.0);
    __syncthreads();
    for (int i = tid; i <= nv; i += DOT_THREADS) {
        c64 acc = zero<double>();
        for (int q = 0; q < DOT_THREADS / 32; ++q) acc += red[q][i];
        partial[((int64_t)slot * nchunk + chunk) * (nv + 1) + i] = acc;
    }
}

template <typename R, typename B>
void launch_dots(const B* V, int64_t ldv, int64_t lds, int nv, const cx<R>* w, int64_t ldw, int64_t n, int nslot,
                 const int* active, c64* partial, int nchunk, cudaStream_t st, R vs) {
    dots_kernel<R, B><<<dim3(nchunk, nslot), DOT_THREADS, 0, st>>>(V, ldv, lds, nv, w, ldw, n, active, partial, nchunk,
                                                                    vs);
    GT_LAUNCH_CHECK();
}

// out[slot * ldo + i] = sum over chunks of partial (i <= nv); mode 1 adds to out
__global__ void reduce_kernel(const c64* __restrict__ partial, int nchunk, int nv, const int* __restrict__ active,
                              c64* __restrict__ out, int ldo, int mode) {
    const int slot = blockIdx.x;
    if (active && !active[slot]) return;
    for (int i = threadIdx.x; i <= nv; i += blockDim.x) {
        c64 acc = zero<double>();
        for (int c = 0; c < nchunk; ++c) acc += partial[((int64_t)slot * nchunk + c) * (nv + 1) + i];
        if (mode == 1) out[(int64_t)slot * ldo + i] += acc;
        else out[(int64_t)slot * ldo + i] = acc;
    }
}

void launch_reduce(const c64* partial, int nchunk, int nv, int nslot, const int* active, c64* out, int ldo, int mode,
                   cudaStream_t st) {
    reduce_kernel<<<nslot, 128, 0, st>>>(partial, nchunk, nv, active, out, ldo, mode);
    GT_LAUNCH_CHECK();
}

// w += sign * sum_i h_i V_i (sign -1: Gram-Schmidt; +1: the cycle's combination); partial |w|^2 per chunk of
// UPD_CHUNK elements (nchunk = update_chunks(n))
template <typename R, typename B>
__global__ void __launch_bounds__(DOT_THREADS) update_kernel(const B* __restrict__ V, int64_t ldv, int64_t lds,
                                                             int nv, const c64* __restrict__ h, int ldh,
                                                             cx<R>* __restrict__ w, int64_t ldw, int64_t n,
                                                             const int* __restrict__ active, c64* __restrict__ partial,
                                                             int nchunk, int sign, R vs) {
    __shared__ cx<R> hs[MAXV];
    __shared__ double red[DOT_THREADS / 32];
    const int slot = blockIdx.y;
    if (active && !active[slot]) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < nv; i += DOT_THREADS) {
        c64 v = h[(int64_t)slot * ldh + i];
        hs[i] = mk<R>(R(sign * v.re * vs), R(sign * v.im * vs));
    }
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * UPD_CHUNK;
    cx<R> acc[UPD_EPT];
#pragma unroll
    for (int e = 0; e < UPD_EPT; ++e) {
        int64_t q = base + e * DOT_THREADS + tid;
        acc[e] = q < n ? w[(int64_t)slot * ldw + q] : zero<R>();
    }
    const B* Vs = V + (int64_t)slot * lds;
    int i = 0;
    // full chunks: UN basis vectors' loads in flight together (FP32 arithmetic; FP64 keeps one)
    constexpr int UN = sizeof(R) == 4 ? 4 : 1;
    if (base + UPD_CHUNK <= n) {
        for (; i + UN <= nv; i += UN) {
            cx<R> v[UN][UPD_EPT];
#pragma unroll
            for (int u = 0; u < UN; ++u)
#pragma unroll
                for (int e = 0; e < UPD_EPT; ++e) v[u][e] = bload(Vs + (int64_t)(i + u) * ldv + base + e * DOT_THREADS + tid);
#pragma unroll
            for (int u = 0; u < UN; ++u) {
                const cx<R> hi = hs[i + u];
#pragma unroll
                for (int e = 0; e < UPD_EPT; ++e) acc[e] += hi * v[u][e];
            }
        }
    }
    for (; i < nv; ++i) {
        const cx<R> hi = hs[i];
        const B* Vi = Vs + (int64_t)i * ldv;
#pragma unroll
        for (int e = 0; e < UPD_EPT; ++e) {
            int64_t q = base + e * DOT_THREADS + tid;
            if (q < n) acc[e] += hi * bload(Vi + q);
        }
    }
    R nrm = 0;
#pragma unroll
    for (int e = 0; e < UPD_EPT; ++e) {
        int64_t q = base + e * DOT_THREADS + tid;
        if (q < n) {
            w[(int64_t)slot * ldw + q] = acc[e];
            nrm += norm2(acc[e]);
        }
    }
    nrm = shfl_sum(nrm);
    if (lane == 0) red[warp] = nrm;
    __syncthreads();
    if (tid == 0 && partial) {
        double s = 0;
        for (int q = 0; q < DOT_THREADS / 32; ++q) s += red[q];
        partial[(int64_t)slot * nchunk + blockIdx.x] = mk<double>(s, 0.0);
    }
}

template <typename R, typename B>
void launch_update(const B* V, int64_t ldv, int64_t lds, int nv, const c64* h, int ldh, cx<R>* w, int64_t ldw,
                   int64_t n, int nslot, const int* active, c64* partial, int sign, cudaStream_t st, R vs) {
    const int nchunk = update_chunks(n);
    update_kernel<R, B><<<dim3(nchunk, nslot), DOT_THREADS, 0, st>>>(V, ldv, lds, nv, h, ldh, w, ldw, n, active,
                                                                      partial, nchunk, sign, vs);
    GT_LAUNCH_CHECK();
}

template void launch_dots<float, c32>(const c32*, int64_t, int64_t, int, const c32*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, float);
template void launch_dots<float, h16c>(const h16c*, int64_t, int64_t, int, const c32*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, float);
template void launch_dots<double, c64>(const c64*, int64_t, int64_t, int, const c64*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, double);
template void launch_update<float, c32>(const c32*, int64_t, int64_t, int, const c64*, int, c32*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, float);
template void launch_update<float, h16c>(const h16c*, int64_t, int64_t, int, const c64*, int, c32*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, float);
template void launch_update<double, c64>(const c64*, int64_t, int64_t, int, const c64*, int, c64*, int64_t, int64_t, int, const int*, c64*, int, cudaStream_t, double);

// ------------------------------------------------------------------------------------------ per-slot scalars
// After the first Gram-Schmidt pass: hvec[0..j] = h, hvec[j+1] = |w_before|^2; hn2 = |w_after|^2 (reduced
// from the update's partials).  Decide the re-orthogonalisation.
__global__ void dgks_kernel(GmresState s, int j) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s.nslot) return;
    int re = 0;
    if (s.active[slot]) {
        double before = sqrt(s.hvec[(int64_t)slot * s.ldh + j + 1].re);
        double after = sqrt(s.hn2[slot].re);
        re = after < s.reorth_ratio * before;
    }
    s.reorth[slot] = re;
}

// The Hessenberg column j of each active slot: rotate, new rotation, residual estimate, convergence.
__global__ void givens_kernel(GmresState s, int j) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s.nslot || !s.active[slot]) return;
    const int m = s.m;
    c64* H = s.H + (int64_t)slot * (m + 1) * m + (int64_t)j * (m + 1);
    const c64* h = s.hvec + (int64_t)slot * s.ldh;
    const c64* h2 = s.h2vec + (int64_t)slot * s.ldh;
    const bool re = s.reorth[slot];
    double hnorm2 = 0;
    for (int i = 0; i <= j; ++i) {
        c64 v = h[i];
        if (re) v += h2[i];
        H[i] = v;
        hnorm2 += norm2(v);
    }
    double hn = sqrt(re ? s.hn2b[slot].re : s.hn2[slot].re);
    double* cs = s.cs + (int64_t)slot * m;
    c64* sn = s.sn + (int64_t)slot * m;
    c64* g = s.g + (int64_t)slot * (m + 1);
    for (int i = 0; i < j; ++i) {
        c64 a = H[i], c = H[i + 1];
        H[i] = cs[i] * a + sn[i] * c;
        H[i + 1] = cs[i] * c - conj(sn[i]) * a;
    }
    c64 a = H[j];
    double aa = sqrt(norm2(a));
    double rho = hypot(aa, hn);
    if (rho == 0.0) {
        cs[j] = 1.0;
        sn[j] = zero<double>();
    } else if (aa == 0.0) {
        cs[j] = 0.0;
        sn[j] = mk<double>(1.0, 0.0);
        H[j] = mk<double>(hn, 0.0);
    } else {
        c64 ph = mk<double>(a.re / aa, a.im / aa);
        cs[j] = aa / rho;
        sn[j] = (hn / rho) * ph;
        H[j] = rho * ph;
    }
    H[j + 1] = zero<double>();
    c64 gj = g[j];
    g[j + 1] = mk<double>(-1.0, 0.0) * (conj(sn[j]) * gj);
    g[j] = cs[j] * gj;
    s.it[slot] = j + 1;
    s.its_total[slot] += 1;
    double res = sqrt(norm2(g[j + 1]));
    bool breakdown = hn <= 1e-14 * sqrt(hnorm2);
    bool done = res <= s.eta[slot] || breakdown || j + 1 >= m || s.its_total[slot] >= s.max_its;
    s.inv_hn[slot] = (hn > 0 && !breakdown) ? 1.0 / hn : 0.0;
    if (done) s.active[slot] = 0;
    s.resid_est[slot] = res;
}

// store v (a basis vector, unscaled) at p[q]; with a narrower basis type also the stored value, unscaled,
// to vc[q] (the vector the next product is applied to)
template <typename R, typename B>
__device__ __forceinline__ void put_basis(const GmresStateT<R, B>& s, B* p, cx<R>* vc, int64_t q, cx<R> v) {
    if constexpr (std::is_same<B, cx<R>>::value) {
        p[q] = v;
    } else {
        bstore(p + q, s.scale * v);
        vc[q] = (R(1) / s.scale) * bload(p + q);
    }
}

template <typename R, typename B>
__global__ void scale_kernel(GmresStateT<R, B> s, int j, int64_t n) {
    const int slot = blockIdx.y;
    if (!s.active[slot]) return;
    const R f = R(s.inv_hn[slot]);
    const cx<R>* w = s.w + (int64_t)slot * s.ldv;
    B* v = s.V + (int64_t)slot * s.lds + (int64_t)(j + 1) * s.ldv;
    cx<R>* vc = s.vcur ? s.vcur + (int64_t)slot * s.ldv : nullptr;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        put_basis(s, v, vc, q, f * w[q]);
}

// y = R^-1 g over the slot's k = it columns (back substitution, FP64)
__global__ void hsolve_kernel(GmresState s) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s.nslot) return;
    const int m = s.m, k = s.it[slot];
    const c64* H = s.H + (int64_t)slot * (m + 1) * m;
    const c64* g = s.g + (int64_t)slot * (m + 1);
    c64* y = s.y + (int64_t)slot * s.ldh;
    for (int i = k - 1; i >= 0; --i) {
        c64 acc = g[i];
        for (int q = i + 1; q < k; ++q) acc -= H[(int64_t)q * (m + 1) + i] * y[q];
        c64 d = H[(int64_t)i * (m + 1) + i];
        y[i] = (norm2(d) > 0) ? cdiv(acc, d) : zero<double>();
    }
    for (int i = k; i < m; ++i) y[i] = zero<double>();
}

// a slot's cycle starts from r / rho: V_0 = r / rho, g = (1, 0, ...), rotations cleared
template <typename R, typename B>
__global__ void init_cycle_kernel(GmresStateT<R, B> s, const c64* __restrict__ r, int64_t ldr, const int* __restrict__ slot_col,
                                  const double* __restrict__ rho, int64_t n) {
    const int slot = blockIdx.y;
    const int col = slot_col[slot];
    const double inv = rho[col] > 0 ? 1.0 / rho[col] : 0.0;
    B* v = s.V + (int64_t)slot * s.lds;
    cx<R>* vc = s.vcur ? s.vcur + (int64_t)slot * s.ldv : nullptr;
    const c64* rc = r + (int64_t)col * ldr;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        put_basis(s, v, vc, q, cvt<R>(inv * rc[q]));
}

__global__ void init_state_kernel(GmresState s, const int* __restrict__ slot_col, const double* __restrict__ rho,
                                  const double* __restrict__ bnorm, double tol, double inner_tol) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s.nslot) return;
    int col = slot_col[slot];
    c64* g = s.g + (int64_t)slot * (s.m + 1);
    g[0] = mk<double>(1.0, 0.0);
    for (int i = 1; i <= s.m; ++i) g[i] = zero<double>();
    s.it[slot] = 0;
    s.active[slot] = 1;
    // the cycle needs to reach the outer tolerance at most (half of it, as a margin), never below inner_tol
    double need = rho[col] > 0 ? 0.5 * tol * bnorm[col] / rho[col] : 1.0;
    s.eta[slot] = fmax(inner_tol, need);
}

// x[col] += rho[col] * e[slot] (FP64 accumulation of the cycle's correction)
template <typename R>
__global__ void refine_kernel(c64* __restrict__ x, int64_t ldx, const cx<R>* __restrict__ e, int64_t lde,
                              const int* __restrict__ slot_col, const double* __restrict__ rho, int64_t n) {
    const int slot = blockIdx.y;
    const int col = slot_col[slot];
    const double f = rho[col];
    const cx<R>* es = e + (int64_t)slot * lde;
    c64* xc = x + (int64_t)col * ldx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        xc[q] += f * cvt<double>(es[q]);
}

__global__ void any_active_kernel(const int* __restrict__ active, int n, int* __restrict__ flag) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (active[i]) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) *flag = any;
}

__global__ void sqrt_norms_kernel(const c64* __restrict__ nrm2, int ld, int n, double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sqrt(nrm2[(int64_t)i * ld].re);
}

template <typename R>
__global__ void to64_kernel(c64* __restrict__ dst, int64_t ldd, const cx<R>* __restrict__ src, int64_t lds,
                            const int* __restrict__ slot_col, int64_t n) {
    const int s = blockIdx.y;
    c64* d = dst + (int64_t)slot_col[s] * ldd;
    const cx<R>* x = src + (int64_t)s * lds;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        d[q] = cvt<double>(x[q]);
}

// dst slot c = src slot c converted to D, for the listed slots (all nslot when list is null): the FP32 inner
// solve's vectors into and out of an FP64 preconditioner apply
template <typename D, typename S>
__global__ void recast_kernel(cx<D>* __restrict__ dst, int64_t ldd, const cx<S>* __restrict__ src, int64_t lds,
                              const int* __restrict__ list, int64_t n) {
    const int c = list ? list[blockIdx.y] : (int)blockIdx.y;
    cx<D>* d = dst + (int64_t)c * ldd;
    const cx<S>* x = src + (int64_t)c * lds;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        d[q] = cvt<D>(x[q]);
}

__global__ void gcr_scale_kernel(c64* __restrict__ p, c64* __restrict__ q, int64_t ld, const c64* __restrict__ nu2,
                                 const int* __restrict__ active, int64_t n) {
    const int c = blockIdx.y;
    if (active && !active[c]) return;
    const double nu = sqrt(nu2[c].re);
    const double f = nu > 0 ? 1.0 / nu : 0.0;
    c64* pc = p + (int64_t)c * ld;
    c64* qc = q + (int64_t)c * ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        pc[i] = f * pc[i];
        qc[i] = f * qc[i];
    }
}

// ------------------------------------------------------------------------------------------ launchers
template <typename R>
void launch_to64(c64* dst, int64_t ldd, const cx<R>* src, int64_t lds, const int* slot_col, int64_t n, int nslot,
                 cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    to64_kernel<R><<<dim3(blocks, nslot), 256, 0, st>>>(dst, ldd, src, lds, slot_col, n);
    GT_LAUNCH_CHECK();
}
template void launch_to64<float>(c64*, int64_t, const c32*, int64_t, const int*, int64_t, int, cudaStream_t);
template void launch_to64<double>(c64*, int64_t, const c64*, int64_t, const int*, int64_t, int, cudaStream_t);

template <typename D, typename S>
void launch_recast(cx<D>* dst, int64_t ldd, const cx<S>* src, int64_t lds, const int* list, int64_t n, int nslot,
                   cudaStream_t st) {
    if (nslot <= 0) return;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    recast_kernel<D, S><<<dim3(blocks, nslot), 256, 0, st>>>(dst, ldd, src, lds, list, n);
    GT_LAUNCH_CHECK();
}
template void launch_recast<double, float>(c64*, int64_t, const c32*, int64_t, const int*, int64_t, int, cudaStream_t);
template void launch_recast<float, double>(c32*, int64_t, const c64*, int64_t, const int*, int64_t, int, cudaStream_t);

void launch_gcr_scale(c64* p, c64* q, int64_t ld, const c64* nu2, const int* active, int64_t n, int ncol,
                      cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    gcr_scale_kernel<<<dim3(blocks, ncol), 256, 0, st>>>(p, q, ld, nu2, active, n);
    GT_LAUNCH_CHECK();
}

void launch_dgks(const GmresState& s, int j, cudaStream_t st) {
    dgks_kernel<<<ceil_div(s.nslot, 128), 128, 0, st>>>(s, j);
    GT_LAUNCH_CHECK();
}
void launch_givens(const GmresState& s, int j, cudaStream_t st) {
    givens_kernel<<<ceil_div(s.nslot, 64), 64, 0, st>>>(s, j);
    GT_LAUNCH_CHECK();
}
template <typename R, typename B>
void launch_scale(const GmresStateT<R, B>& s, int j, int64_t n, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    scale_kernel<R, B><<<dim3(blocks, s.nslot), 256, 0, st>>>(s, j, n);
    GT_LAUNCH_CHECK();
}
void launch_hsolve(const GmresState& s, cudaStream_t st) {
    hsolve_kernel<<<ceil_div(s.nslot, 64), 64, 0, st>>>(s);
    GT_LAUNCH_CHECK();
}
template <typename R, typename B>
void launch_init_cycle(const GmresStateT<R, B>& s, const c64* r, int64_t ldr, const int* slot_col, const double* rho,
                       int64_t n, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    init_cycle_kernel<R, B><<<dim3(blocks, s.nslot), 256, 0, st>>>(s, r, ldr, slot_col, rho, n);
    GT_LAUNCH_CHECK();
}
void launch_init_state(const GmresState& s, const int* slot_col, const double* rho, const double* bnorm, double tol,
                       double inner_tol, cudaStream_t st) {
    init_state_kernel<<<ceil_div(s.nslot, 64), 64, 0, st>>>(s, slot_col, rho, bnorm, tol, inner_tol);
    GT_LAUNCH_CHECK();
}
template <typename R>
void launch_refine(c64* x, int64_t ldx, const cx<R>* e, int64_t lde, const int* slot_col, const double* rho, int64_t n,
                   int nslot, cudaStream_t st) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    refine_kernel<R><<<dim3(blocks, nslot), 256, 0, st>>>(x, ldx, e, lde, slot_col, rho, n);
    GT_LAUNCH_CHECK();
}
void launch_any_active(const int* active, int n, int* flag, cudaStream_t st) {
    any_active_kernel<<<1, 256, 0, st>>>(active, n, flag);
    GT_LAUNCH_CHECK();
}
__global__ void sqrt_norms_active_kernel(const c64* __restrict__ nrm2, int ld, int n, const int* __restrict__ active,
                                         double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && active[i]) out[i] = sqrt(nrm2[(int64_t)i * ld].re);
}

void launch_sqrt_norms_active(const c64* nrm2, int ld, int n, const int* active, double* out, cudaStream_t st) {
    sqrt_norms_active_kernel<<<ceil_div(n, 128), 128, 0, st>>>(nrm2, ld, n, active, out);
    GT_LAUNCH_CHECK();
}

void launch_sqrt_norms(const c64* nrm2, int ld, int n, double* out, cudaStream_t st) {
    sqrt_norms_kernel<<<ceil_div(n, 128), 128, 0, st>>>(nrm2, ld, n, out);
    GT_LAUNCH_CHECK();
}

template void launch_scale<float, c32>(const GmresStateT<float, c32>&, int, int64_t, cudaStream_t);
template void launch_scale<float, h16c>(const GmresStateT<float, h16c>&, int, int64_t, cudaStream_t);
template void launch_scale<double, c64>(const GmresStateT<double, c64>&, int, int64_t, cudaStream_t);
template void launch_init_cycle<float, c32>(const GmresStateT<float, c32>&, const c64*, int64_t, const int*, const double*, int64_t, cudaStream_t);
template void launch_init_cycle<float, h16c>(const GmresStateT<float, h16c>&, const c64*, int64_t, const int*, const double*, int64_t, cudaStream_t);
template void launch_init_cycle<double, c64>(const GmresStateT<double, c64>&, const c64*, int64_t, const int*, const double*, int64_t, cudaStream_t);
template void launch_refine<float>(c64*, int64_t, const c32*, int64_t, const int*, const double*, int64_t, int, cudaStream_t);
template void launch_refine<double>(c64*, int64_t, const c64*, int64_t, const int*, const double*, int64_t, int, cudaStream_t);

}  // namespace gt
