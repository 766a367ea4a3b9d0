// Common definitions for the dedalus GB300 kernels: status codes, error
// capture, complex arithmetic on a generic real type, launch helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "dd_gb300.h"
#include "timing.cuh"
#include <atomic>
#include <string>

namespace dd {

// ---------------------------------------------------------------- errors
// Last error message, thread-local so concurrent contexts on different host
// threads do not clobber each other.
void set_error(const char* fmt, ...);
const char* last_error();

#define DD_CHECK_ARG(cond, ...)                                      \
    do {                                                             \
        if (!(cond)) {                                               \
            ::dd::set_error(__VA_ARGS__);                            \
            return DD_ERR_INVALID;                                   \
        }                                                            \
    } while (0)

#define DD_CHECK_SUPPORTED(cond, ...)                                \
    do {                                                             \
        if (!(cond)) {                                               \
            ::dd::set_error(__VA_ARGS__);                            \
            return DD_ERR_UNSUPPORTED;                               \
        }                                                            \
    } while (0)

#define DD_CUDA(call)                                                \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            ::dd::set_error("%s failed: %s (%s:%d)", #call,          \
                            cudaGetErrorString(e_), __FILE__, __LINE__); \
            return DD_ERR_CUDA;                                      \
        }                                                            \
    } while (0)

// Check the launch just issued (configuration errors surface here).
#define DD_LAUNCH_CHECK()  DD_CUDA(cudaGetLastError())

#define DD_TRY(expr)                                                 \
    do {                                                             \
        int s_ = (expr);                                             \
        if (s_ != DD_OK) return s_;                                  \
    } while (0)

// Raise a kernel's dynamic shared-memory limit once per device (the attribute
// belongs to the device current at the call); `done` holds one bit per device.
inline int ensure_smem(const void* fn, size_t bytes, std::atomic<unsigned long long>& done) {
    int dev = 0;
    DD_CUDA(cudaGetDevice(&dev));
    const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return DD_OK;
    DD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    done.fetch_or(bit, std::memory_order_release);
    return DD_OK;
}

// ---------------------------------------------------------------- complex
template <typename T>
struct C {
    T x, y;
};

template <typename T>
__host__ __device__ __forceinline__ C<T> mk(T x, T y) { C<T> r; r.x = x; r.y = y; return r; }
template <typename T>
__device__ __forceinline__ C<T> operator+(C<T> a, C<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T>
__device__ __forceinline__ C<T> operator-(C<T> a, C<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T>
__device__ __forceinline__ C<T> cmul(C<T> a, C<T> w) {
    return mk<T>(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
// a * conj(w)
template <typename T>
__device__ __forceinline__ C<T> cmulc(C<T> a, C<T> w) {
    return mk<T>(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
template <typename T>
__device__ __forceinline__ C<T> conj(C<T> a) { return mk<T>(a.x, -a.y); }
template <typename T>
__device__ __forceinline__ C<T> scale(C<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// multiply by -i (forward sign) or +i (inverse sign)
template <bool INV, typename T>
__device__ __forceinline__ C<T> mul_mi(C<T> a) {
    return INV ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}
template <typename T>
__device__ __forceinline__ C<T> zero() { return mk<T>(T(0), T(0)); }

// Global-memory element types for each real type.
template <typename T> struct Vec2;
template <> struct Vec2<double> { typedef double2 type; };
template <> struct Vec2<float>  { typedef float2 type; };

template <typename T>
__device__ __forceinline__ C<T> ldc(const typename Vec2<T>::type* p) {
    typename Vec2<T>::type v = *p;
    return mk<T>(v.x, v.y);
}
template <typename T>
__device__ __forceinline__ void stc(typename Vec2<T>::type* p, C<T> a) {
    typename Vec2<T>::type v; v.x = a.x; v.y = a.y; *p = v;
}

// Short precision tag for labels: f64, f32, df64.
template <typename T> struct PrecName;
template <> struct PrecName<double> { static constexpr const char* s = "_f64"; };
template <> struct PrecName<float> { static constexpr const char* s = "_f32"; };

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace dd
