// noalloc.cu -- calc_cross_powerspec_noalloc: the P(k) binning without any device allocation.
//
// Who needs it: callers that must not allocate device memory from inside their loop.  Two
// common cases: a process whose device memory budget is already handed to another allocator
// (a framework's caching pool that holds nearly all of the GPU), where a fresh cudaMalloc fails;
// and streaming analysis loops where cudaMalloc / cudaFree would synchronise the device and stall
// the copies and kernels overlapping with the binning.  The regular calc_cross_powerspec caches
// its accumulators and a bin table per |n|^2 in library workspace, allocated on first use; this
// variant keeps its accumulators and the bins' |n|^2 edges in a fixed file-scope device array.
//
// Bins: the host finds, for every bin, the first |n|^2 that falls in it, with the same rule the
// regular entry point tabulates (pk_bin_of_n2: the reference's float-u log bins of
// src/calc_powerspec.c:61-63, or linear shells); the rule is non-decreasing in |n|^2, so these
// edges give every mode the regular table's bin.  The kernel finds a mode's bin by binary search
// over the edges, sums per block in shared memory and flushes each block's sums once.
//
// Limits: at most MITOS_NOALLOC_MAX_BINS bins; the inputs must already be device pointers on the
// library's device (the device current at the library's first call).  The scratch array is shared
// by every call and keeps the last call's contents; each call clears its accumulators before use.
// Calls whose GPU work overlaps (two host threads, or a call overlapping another process's use of
// the same library copy) race on the array; issue them one after another.
// Set-up: the first call looks up the array's device address with cudaGetSymbolAddress (with the
// device current) and caches it.  With CUDA's lazy module loading (the default) the array is also
// reserved at that moment, so make the first call -- a set-up-only call with N = 0 and null grids
// is enough -- before another allocator takes the device's memory, and before any stream capture.
#include <math.h>
#include <string.h>

#include <mutex>

#include "common.cuh"
#include "context.cuh"

#define MITOS_NOALLOC_MAX_BINS 4096
#define MITOS_NOALLOC_THREADS 512

namespace mitos {

// [0, B): sum of mult * k, [B, 2B): sum of mult * Re(X conj Y), [2B, 3B): counts (as uint64),
// [3B, 4B + 1): the bins' first |n|^2 (as int64; entry B: the first |n|^2 beyond the last bin)
static __device__ __align__(256) double g_noalloc_scratch[4 * MITOS_NOALLOC_MAX_BINS + 8];
static double *g_noalloc_ptr = nullptr;
static std::mutex g_noalloc_mu;

template <typename T>
__global__ void __launch_bounds__(MITOS_NOALLOC_THREADS)
k_bin_cross_noalloc(int N, double dk, int bins, const cplx<T> *__restrict__ f1, const cplx<T> *__restrict__ f2,
                    double *__restrict__ acc) {
    extern __shared__ double sh[];
    double *sk = sh, *sp = sh + bins;
    unsigned long long *sn = reinterpret_cast<unsigned long long *>(sh + 2 * bins);
    long long *se = reinterpret_cast<long long *>(sh + 3 * bins);
    const long long *edges = reinterpret_cast<const long long *>(acc + 3 * bins);
    for (int i = threadIdx.x; i < bins; i += blockDim.x) {
        sk[i] = 0;
        sp[i] = 0;
        sn[i] = 0;
    }
    for (int i = threadIdx.x; i <= bins; i += blockDim.x) se[i] = edges[i];
    __syncthreads();
    const int H = N / 2 + 1;
    const long total = (long)N * N * H;
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int jy = kint((int)(xy % N), N), jx = kint((int)(xy / N), N);
        const long long n2 = (long long)jx * jx + (long long)jy * jy + (long long)z * z;
        if (n2 < se[0]) continue;  // the DC mode (se[0] = 1)
        // the last bin whose first |n|^2 is <= n2; bin `bins` holds the modes beyond the last bin
        int lo = 0, hi = bins;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (se[mid] <= n2) lo = mid;
            else hi = mid - 1;
        }
        if (lo >= bins) continue;
        const cplx<T> a = f1[id], c = f2[id];
        const int mult = (z == 0 || z == N / 2) ? 1 : 2;
        const double kx = __dmul_rn((double)jx, dk), ky = __dmul_rn((double)jy, dk), kz = __dmul_rn((double)z, dk);
        const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
        atomicAdd(sk + lo, mult * k);
        atomicAdd(sp + lo, mult * ((double)a.x * (double)c.x + (double)a.y * (double)c.y));
        atomicAdd(sn + lo, (unsigned long long)mult);
    }
    __syncthreads();
    unsigned long long *bn = reinterpret_cast<unsigned long long *>(acc + 2 * bins);
    for (int i = threadIdx.x; i < bins; i += blockDim.x) {
        if (sn[i]) {
            atomicAdd(acc + i, sk[i]);
            atomicAdd(acc + bins + i, sp[i]);
            atomicAdd(bn + i, sn[i]);
        }
    }
}

// set-up, once, with the library's device current: the device address of the scratch array
static double *noalloc_scratch(int *status) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    int dev = -1;
    *status = 4;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_error(4, "calc_cross_powerspec_noalloc: no usable current device");
        return nullptr;
    }
    const int libdev = library_device();
    if (dev != libdev) {
        set_error(3, "calc_cross_powerspec_noalloc: device %d is current, the library runs on device %d", dev, libdev);
        *status = 3;
        return nullptr;
    }
    if (!g_noalloc_ptr) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(4, "calc_cross_powerspec_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return nullptr;
        }
        g_noalloc_ptr = p;
    }
    *status = 0;
    return g_noalloc_ptr;
}

// edges[b] = the first n2 >= 1 whose bin is >= b (b = 0 .. bins), by bisection on the
// non-decreasing bin rule; modes beyond the last bin count as bin `bins`
static void bin_edges(int N, int bins, int linear, double boxlen, long long *edges) {
    const long n2max = 3L * (N / 2) * (N / 2);
    const double dk = 2 * M_PI / boxlen;
    const double lmin = log(dk), lmax = log(sqrt(3) * dk * N / 2);
    auto key = [&](long n2) -> int {
        if (n2 > n2max) return bins;
        const int b = pk_bin_of_n2(n2, N, bins, linear, dk, lmin, lmax);
        return b < 0 ? bins : b;
    };
    for (int b = 0; b <= bins; b++) {
        long lo = b == 0 ? 1 : edges[b - 1], hi = n2max + 1;  // key(hi) >= b
        while (lo < hi) {
            const long mid = lo + (hi - lo) / 2;
            if (key(mid) >= b) hi = mid;
            else lo = mid + 1;
        }
        edges[b] = lo;
    }
}

}  // namespace mitos

// No counterpart in the reference (see include/mitos_gb300.h).
extern "C" int calc_cross_powerspec_noalloc(int N, double boxlen, const void *dev_box1, const void *dev_box2,
                                            int precision, int bins, int linear, double *k_in_bins,
                                            double *power_in_bins, long *obs_in_bins) {
    using namespace mitos;
    int st = 0;
    if (N == 0 && !dev_box1 && !dev_box2) return noalloc_scratch(&st) ? 0 : st;  // set-up only
    if (bins < 1 || bins > MITOS_NOALLOC_MAX_BINS) {
        set_error(3, "calc_cross_powerspec_noalloc: %d bins requested, at most %d are supported", bins,
                  MITOS_NOALLOC_MAX_BINS);
        return 3;
    }
    if (N < 2 || N > 4096 || (N & 1) || !dev_box1 || !dev_box2 || !(boxlen > 0) || !k_in_bins ||
        !power_in_bins || !obs_in_bins || (precision != MITOS_FP32 && precision != MITOS_FP64)) {
        set_error(1, "calc_cross_powerspec_noalloc: invalid arguments");
        return 1;
    }
    double *acc = noalloc_scratch(&st);
    if (!acc) return st;
    long long edges[MITOS_NOALLOC_MAX_BINS + 1];
    bin_edges(N, bins, linear, boxlen, edges);
    cudaStream_t s = stream();
    // the array keeps the previous call's sums: clear what must start at zero
    MITOS_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * bins, s));
    MITOS_CUDA(cudaMemcpyAsync(acc + 3 * bins, edges, sizeof(long long) * (bins + 1), cudaMemcpyHostToDevice, s));
    const size_t smem = sizeof(double) * (4 * (size_t)bins + 1);
    const double dk = 2 * M_PI / boxlen;
    const long total = (long)N * N * (N / 2 + 1);
    int blocks = (int)((total + MITOS_NOALLOC_THREADS - 1) / MITOS_NOALLOC_THREADS);
    if (blocks > 152 * 4) blocks = 152 * 4;
    launch_begin("bin_cross_noalloc");
    if (precision == MITOS_FP32) {
        MITOS_CUDA(cudaFuncSetAttribute(k_bin_cross_noalloc<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_bin_cross_noalloc<float><<<blocks, MITOS_NOALLOC_THREADS, smem, s>>>(N, dk, bins, (const float2 *)dev_box1,
                                                                                (const float2 *)dev_box2, acc);
    } else {
        MITOS_CUDA(cudaFuncSetAttribute(k_bin_cross_noalloc<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_bin_cross_noalloc<double><<<blocks, MITOS_NOALLOC_THREADS, smem, s>>>(N, dk, bins, (const double2 *)dev_box1,
                                                                                 (const double2 *)dev_box2, acc);
    }
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
