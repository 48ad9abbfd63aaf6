// noalloc.cu -- calc_cross_powerspec_noalloc: the P(k) binning without any device allocation.
//
// Who needs it: callers that must not allocate device memory from inside their loop.  Two
// common cases: a process whose device memory budget is already handed to another allocator
// (a framework's caching pool that holds nearly all of the GPU), where a fresh cudaMalloc fails;
// and streaming analysis loops where cudaMalloc / cudaFree would synchronise the device and stall
// the copies and kernels overlapping with the binning.  The regular calc_cross_powerspec caches
// its accumulators and bin table in library workspace, allocated on first use; this variant
// keeps its accumulators in a fixed file-scope device array instead, and computes bins on the fly.
//
// Limits: at most MITOS_NOALLOC_MAX_BINS bins; the inputs must already be device pointers.
// The scratch array is shared by every call on a device and keeps the last call's contents;
// each call clears it before use.  Calls whose GPU work overlaps (two host threads, or calls on
// different streams) race on the array; issue them one after another.
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that first call before
// any stream capture.
#include <math.h>
#include <string.h>

#include "common.cuh"

#define MITOS_NOALLOC_MAX_BINS 4096
#define MITOS_NOALLOC_MAX_DEVICES 64

namespace mitos {

// [0, B): sum of mult * k, [B, 2B): sum of mult * Re(X conj Y), [2B, 3B): counts (as uint64)
static __device__ __align__(256) double g_noalloc_scratch[3 * MITOS_NOALLOC_MAX_BINS];
static double *g_noalloc_ptr[MITOS_NOALLOC_MAX_DEVICES];

// bin of a mode of squared integer wavevector norm n2: linear shells of width k_Nyq / bins
// (isqrt(n2 bins^2) / (N/2)) or the reference log bins (src/calc_powerspec.c:61-63)
__device__ __forceinline__ int noalloc_bin(long n2, int N, int bins, int linear, double dk,
                                           double log_min_k, double inv_span) {
    if (linear) {
        const long a = n2 * (long)bins * bins;
        long r = (long)sqrt((double)a);
        while (r * r > a) r--;
        while ((r + 1) * (r + 1) <= a) r++;
        const int b = (int)(r / (N / 2));
        return b < bins ? b : -1;
    }
    const double k = sqrt((double)n2) * dk;
    const float u = (log(k) - log_min_k) * inv_span;
    const int b = (int)floor((bins - 1) * u);
    return (b >= 0 && b < bins) ? b : -1;
}

template <typename T>
__global__ void k_bin_cross_noalloc(int N, double dk, int bins, int linear, double log_min_k, double inv_span,
                                    const cplx<T> *__restrict__ f1, const cplx<T> *__restrict__ f2,
                                    double *__restrict__ acc) {
    const int H = N / 2 + 1;
    const long total = (long)N * N * H;
    double *bk = acc, *bp = acc + bins;
    unsigned long long *bn = reinterpret_cast<unsigned long long *>(acc + 2 * bins);
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int jy = kint((int)(xy % N), N), jx = kint((int)(xy / N), N);
        const long n2 = (long)jx * jx + (long)jy * jy + (long)z * z;
        if (n2 == 0) continue;
        const int b = noalloc_bin(n2, N, bins, linear, dk, log_min_k, inv_span);
        if (b < 0) continue;
        const cplx<T> a = f1[id], c = f2[id];
        const int mult = (z == 0 || z == N / 2) ? 1 : 2;
        const double kx = __dmul_rn((double)jx, dk), ky = __dmul_rn((double)jy, dk), kz = __dmul_rn((double)z, dk);
        const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
        atomicAdd(bk + b, mult * k);
        atomicAdd(bp + b, mult * ((double)a.x * (double)c.x + (double)a.y * (double)c.y));
        atomicAdd(bn + b, (unsigned long long)mult);
    }
}

// set-up, once per device with that device current: the device address of the scratch array
static double *noalloc_scratch() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MITOS_NOALLOC_MAX_DEVICES) {
        set_error(4, "calc_cross_powerspec_noalloc: no usable current device");
        return nullptr;
    }
    if (!g_noalloc_ptr[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(4, "calc_cross_powerspec_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return nullptr;
        }
        g_noalloc_ptr[dev] = p;
    }
    return g_noalloc_ptr[dev];
}

}  // namespace mitos

// No counterpart in the reference (see include/mitos_gb300.h).
extern "C" int calc_cross_powerspec_noalloc(int N, double boxlen, const void *dev_box1, const void *dev_box2,
                                            int precision, int bins, int linear, double *k_in_bins,
                                            double *power_in_bins, long *obs_in_bins) {
    using namespace mitos;
    if (bins < 1 || bins > MITOS_NOALLOC_MAX_BINS) {
        set_error(3, "calc_cross_powerspec_noalloc: %d bins requested, at most %d are supported", bins,
                  MITOS_NOALLOC_MAX_BINS);
        return 3;
    }
    if (N < 2 || (N & 1) || !dev_box1 || !dev_box2 || boxlen <= 0 ||
        (precision != MITOS_FP32 && precision != MITOS_FP64)) {
        set_error(1, "calc_cross_powerspec_noalloc: invalid arguments");
        return 1;
    }
    double *acc = noalloc_scratch();
    if (!acc) return 4;
    cudaStream_t s = stream();
    // the array keeps the previous call's sums: clear what must start at zero
    MITOS_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * bins, s));
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2, min_k = dk;
    const double lmin = log(min_k), inv_span = 1.0 / (log(max_k) - lmin);
    const long total = (long)N * N * (N / 2 + 1);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    launch_begin("bin_cross_noalloc");
    if (precision == MITOS_FP32)
        k_bin_cross_noalloc<float><<<blocks, 256, 0, s>>>(N, dk, bins, linear, lmin, inv_span,
                                                          (const float2 *)dev_box1, (const float2 *)dev_box2, acc);
    else
        k_bin_cross_noalloc<double><<<blocks, 256, 0, s>>>(N, dk, bins, linear, lmin, inv_span,
                                                           (const double2 *)dev_box1, (const double2 *)dev_box2, acc);
    count_launch();
    MITOS_LAUNCH_CHECK("calc_cross_powerspec_noalloc");
    // results straight into the caller's host arrays: k and P sums first, counts after
    MITOS_CUDA(cudaMemcpyAsync(k_in_bins, acc, sizeof(double) * bins, cudaMemcpyDeviceToHost, s));
    MITOS_CUDA(cudaMemcpyAsync(power_in_bins, acc + bins, sizeof(double) * bins, cudaMemcpyDeviceToHost, s));
    MITOS_CUDA(cudaMemcpyAsync(obs_in_bins, acc + 2 * bins, sizeof(long) * bins, cudaMemcpyDeviceToHost, s));
    MITOS_CUDA(cudaStreamSynchronize(s));
    const double boxvol = boxlen * boxlen * boxlen;
    for (int i = 0; i < bins; i++) {
        k_in_bins[i] /= (double)obs_in_bins[i];
        power_in_bins[i] /= (double)obs_in_bins[i];
        power_in_bins[i] /= boxvol;
    }
    return 0;
}
