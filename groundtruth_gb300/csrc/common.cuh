// Shared device helpers of the GB300 PEEC solver: complex arithmetic templated on the real type
// (float for the inner iterations, double for residuals and factorisation), error plumbing.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <atomic>
#include <string>

namespace gt {

template <typename R> struct alignas(2 * sizeof(R)) cx { R re, im; };
using c32 = cx<float>;
using c64 = cx<double>;

template <typename R> __host__ __device__ __forceinline__ cx<R> mk(R a, R b) { cx<R> z; z.re = a; z.im = b; return z; }
template <typename R> __host__ __device__ __forceinline__ cx<R> zero() { return mk<R>(R(0), R(0)); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return mk<R>(a.re + b.re, a.im + b.im); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return mk<R>(a.re - b.re, a.im - b.im); }
template <typename R> __host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
    return mk<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename R> __host__ __device__ __forceinline__ cx<R> operator*(R s, cx<R> a) { return mk<R>(s * a.re, s * a.im); }
template <typename R> __host__ __device__ __forceinline__ cx<R>& operator+=(cx<R>& a, cx<R> b) { a.re += b.re; a.im += b.im; return a; }
template <typename R> __host__ __device__ __forceinline__ cx<R>& operator-=(cx<R>& a, cx<R> b) { a.re -= b.re; a.im -= b.im; return a; }
template <typename R> __host__ __device__ __forceinline__ cx<R> conj(cx<R> a) { return mk<R>(a.re, -a.im); }
// conj(a) * b
template <typename R> __host__ __device__ __forceinline__ cx<R> cmulc(cx<R> a, cx<R> b) {
    return mk<R>(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
template <typename R> __host__ __device__ __forceinline__ R norm2(cx<R> a) { return a.re * a.re + a.im * a.im; }
template <typename R> __host__ __device__ __forceinline__ cx<R> jmul(cx<R> a) { return mk<R>(-a.im, a.re); }  // j * a
// a / b
template <typename R> __host__ __device__ __forceinline__ cx<R> cdiv(cx<R> a, cx<R> b) {
    R d = b.re * b.re + b.im * b.im;
    return mk<R>((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
template <typename D, typename S> __host__ __device__ __forceinline__ cx<D> cvt(cx<S> a) { return mk<D>(D(a.re), D(a.im)); }

inline int ceil_div(int64_t a, int64_t b) { return int((a + b - 1) / b); }

// The failure text of the calling host thread (gt_last_error).
void set_error(const std::string& s);

struct CudaError {
    cudaError_t code;
    std::string where;
};

#define GT_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e__ = (call);                                                          \
        if (e__ != cudaSuccess) throw ::gt::CudaError{e__, std::string(#call) + " at " +   \
                                                    __FILE__ + ":" + std::to_string(__LINE__)}; \
    } while (0)

// kernels launched by the library (gt_launch_count)
extern std::atomic<long long> g_launches;

// Let `fn` take `bytes` of dynamic shared memory on the current device.  The cap only ever rises: host
// threads that launch the same kernel with different sizes on their own streams must not lower it between
// another thread's raise and its launch.
void raise_smem(const void* fn, size_t bytes);

#define GT_LAUNCH_CHECK()               \
    do {                                \
        ::gt::g_launches.fetch_add(1);  \
        GT_CUDA(cudaGetLastError());    \
    } while (0)

}  // namespace gt
