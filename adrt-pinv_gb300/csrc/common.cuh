// Shared device/host helpers for the sm_103a kernels of the ADRT oblique inverses.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "adrt_pinv_gb300.h"

namespace adrt {

// ------------------------------------------------------------------ complex arithmetic on interleaved pairs
template <typename real> struct cx;
template <> struct cx<float> { using t = float2; };
template <> struct cx<double> { using t = double2; };
template <typename real> using cplx = typename cx<real>::t;

template <typename real> __host__ __device__ __forceinline__ cplx<real> mk(real re, real im) {
    cplx<real> r; r.x = re; r.y = im; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// a + w * b (complex multiply-add, 4 FMAs)
template <typename C> __device__ __forceinline__ C cfma(C w, C b, C a) {
    C r;
    r.x = fma(w.x, b.x, fma(-w.y, b.y, a.x));
    r.y = fma(w.x, b.y, fma(w.y, b.x, a.y));
    return r;
}
// w * b
template <typename C> __device__ __forceinline__ C cmul(C w, C b) {
    C r;
    r.x = fma(w.x, b.x, -w.y * b.y);
    r.y = fma(w.x, b.y, w.y * b.x);
    return r;
}
// conj(w) * b
template <typename C> __device__ __forceinline__ C cmulc(C w, C b) {
    C r;
    r.x = fma(w.x, b.x, w.y * b.y);
    r.y = fma(w.x, b.y, -w.y * b.x);
    return r;
}
// conj(w0) * a + conj(w1) * b
template <typename C> __device__ __forceinline__ C cdot2c(C w0, C a, C w1, C b) {
    C r;
    r.x = fma(w0.x, a.x, fma(w0.y, a.y, fma(w1.x, b.x, w1.y * b.y)));
    r.y = fma(w0.x, a.y, fma(-w0.y, a.x, fma(w1.x, b.y, -w1.y * b.x)));
    return r;
}
template <typename C, typename S> __device__ __forceinline__ C cscale(S s, C a) { C r; r.x = s * a.x; r.y = s * a.y; return r; }

// ------------------------------------------------------------------ bit utilities (usable in constant expressions)
__host__ __device__ constexpr int brev(int x, int bits) {
    int r = 0;
    for (int i = 0; i < bits; ++i) r |= ((x >> i) & 1) << (bits - 1 - i);
    return r;
}
__host__ __device__ constexpr int imax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int imin(int a, int b) { return a < b ? a : b; }

// ------------------------------------------------------------------ error reporting shared by the C ABI
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);
int launch_status(const char* where);
// the status of a cudaLaunchKernelEx call: its own return value (cluster launches can be refused there), then the
// launch error state
int launch_ex_status(cudaError_t launched, const char* where);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// number of kernels this library has launched (all threads), for launch accounting
void count_launch();

}  // namespace adrt
