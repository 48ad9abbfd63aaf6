// common.cuh -- shared types, error handling and small helpers of the GB300 IC library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/mitos_gb300.h"

namespace mitos {

// ---- complex type of either precision -------------------------------------------------
template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <typename T> using cplx = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T re, T im) {
    cplx<T> c;
    c.x = re;
    c.y = im;
    return c;
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
    return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
    return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cscale(cplx<T> a, T s) {
    return mk<T>(a.x * s, a.y * s);
}
// multiply by i*s (s real): (a + ib) * i s = -b s + i a s
template <typename T> __host__ __device__ __forceinline__ cplx<T> cmul_is(cplx<T> a, T s) {
    return mk<T>(-a.y * s, a.x * s);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cconj(cplx<T> a) {
    return mk<T>(a.x, -a.y);
}
// FP32 complex add and subtract as one packed instruction on both lanes (sm_100 and later: the
// FP32x2 add and fused multiply-add).  Each lane rounds as the scalar operation: a - b is
// fma(b, -1, a), whose product is exact.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(MITOS_NO_FP32X2)
#define MITOS_FP32X2 1
#endif
template <> __host__ __device__ __forceinline__ float2 cadd<float>(float2 a, float2 b) {
#ifdef MITOS_FP32X2
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
template <> __host__ __device__ __forceinline__ float2 csub<float>(float2 a, float2 b) {
#ifdef MITOS_FP32X2
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}

// ---- error state ----------------------------------------------------------------------
void set_error(int code, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);

// prefetch the 32-byte sector at p into L2 (no register is written; p must lie in an allocation)
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

#define MITOS_CUDA(call)                                                                  \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess) return check_cuda(_e, #call);                              \
    } while (0)

#define MITOS_LAUNCH_CHECK(what)                                                          \
    do {                                                                                  \
        cudaError_t _e = cudaGetLastError();                                              \
        if (_e != cudaSuccess) return check_cuda(_e, what);                               \
    } while (0)

// the library's stream (created on first use) and kernel-launch counter
cudaStream_t stream();
int library_device();                 // the device the library stream was created on
void set_stream(cudaStream_t s);      // this thread's launches go to s (nullptr: the library stream)
void set_async(bool on);              // this thread's entry points return without synchronising
bool async_mode();
void set_workspace_set(int s);        // this thread's workspace() buffers come from set s
void count_launch(int n = 1);
void launch_begin(const char *name);  // pairs with count_launch for per-launch timing

// integer wavevector component of index i on an N grid, with +N/2 at the Nyquist index
// (src/fft.c:31-33: i > N/2 maps to i - N)
__host__ __device__ __forceinline__ int kint(int i, int N) { return i > N / 2 ? i - N : i; }

}  // namespace mitos
