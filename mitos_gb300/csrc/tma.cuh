// tma.cuh -- tensor-memory-accelerator tile loads (cp.async.bulk.tensor) completing on a shared
// memory mbarrier, with bounded waits, and the host encoding of 3D tiled tensor maps.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

namespace mitos {

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// the barriers' initialisation visible to the tensor copies (async proxy)
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// generic-proxy accesses of shared memory ordered before later tensor copies into it
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// box of a 3D tiled tensor map at element coordinates (c0 innermost) into shared memory
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// untiled bulk copy of `bytes` (a multiple of 16) from global src to shared dst (both 16-byte
// aligned), completing on bar
__device__ __forceinline__ void bulk_load_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// wait for the phase of the given parity to complete, at most about 2^22 polls (a suspended poll
// plus a short sleep each: well under a few seconds); false if it never did
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    for (int i = 0; i < (1 << 22); i++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

// host: cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda);
// null where the driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// 3D tiled map of a grid [n2][n1][pitch] of elements (FLOAT32 or FLOAT64), box {b0, b1, b2}
// (b0 innermost); false where it cannot be encoded
bool encode_grid_map(CUtensorMap *m, const void *base, bool f64, long n2, long n1, long pitch, unsigned b0,
                     unsigned b1, unsigned b2);

}  // namespace mitos
