// rng.cuh -- the reference's xoshiro256** stream on the GPU: one step (include/random_xorshift.h:15-29),
// sampleNorm in FP64 and FP32 (src/random.c:34-49), and jump-ahead by GF(2) polynomials.
//
// xoshiro256** is linear over GF(2) on its 256-bit state: the state after J steps is q_J(A) s0,
// with A the one-step map and q_J(x) = x^J mod p(x), p the characteristic polynomial of A.  The
// host computes the polynomials (noise.cu); a block tabulates A^i s0 (i < 256) in shared memory
// and a thread's start state is the XOR of the entries its polynomial's bits select.
#pragma once
#include <stdint.h>

#include "context.cuh"
#include "crmath.cuh"

namespace mitos {

struct RngState {
    uint64_t s[4];
};

__device__ __forceinline__ uint64_t drotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

__device__ __forceinline__ uint64_t dnext(uint64_t &s0, uint64_t &s1, uint64_t &s2, uint64_t &s3) {
    const uint64_t result = drotl(s1 * 5, 7) * 9;  // include/random_xorshift.h:17
    const uint64_t t = s1 << 17;
    s2 ^= s0;
    s3 ^= s1;
    s1 ^= s2;
    s0 ^= s3;
    s2 ^= t;
    s3 = drotl(s3, 45);
    return result;
}

// sampleNorm in FP64: src/random.c:34-49 (2^64 = (double)UINT64_MAX + 1), with the correctly
// rounded log and cos of crmath.cuh: the reference formula's exactly rounded value, which the host
// libm gives too except where it misrounds by an ulp
__device__ __forceinline__ double gauss64(uint64_t A, uint64_t B) { return crm::box_muller(A, B); }

// the same with the device libm's log and cos (within an ulp or two): for the thermal normals,
// whose float outputs absorb such differences
__device__ __forceinline__ double gauss64_libm(uint64_t A, uint64_t B) {
    const double RMax = 18446744073709551616.0;
    const double u = (__ull2double_rn(A) + 0.5) / RMax;
    const double v = (__ull2double_rn(B) + 0.5) / RMax;
    return sqrt(-2 * log(u)) * cos(2 * 3.14159265358979323846 * v);
}

// the same Box-Muller transform in FP32, without divergence: t = u or 1 - u (the exact complement
// ~A), t in (0, 1/2]; ln u = ln t for u < 1/2 (|ln t| >= ln 2, so the hardware log2 keeps full
// relative precision) and ln u = ln(1 - t) = -2 atanh(s), s = t / (2 - t) <= 1/3, for u >= 1/2
// (the atanh series through s^15; the next term is below 4e-9 relative)
//
// No 64-bit integer -> float conversions (they run on the FP64 pipe, a small fraction of the FP32
// rate on this part): the uniform is hi 2^32 + lo from the two 32-bit halves (one FMA: within an
// ulp of the rounded 64-bit value, 2^-24 relative at every magnitude), the cosine argument the
// top 32 bits (absolute error below 2^-32).
//
// -2 ln u of the uniform of draw A
__device__ __forceinline__ float gauss32_r2(uint64_t A) {
    const float inv64 = 5.42101086242752217e-20f;  // 2^-64
    const bool hi = (A >> 63) != 0;
    const uint64_t a = hi ? ~A : A;
    const float af = fmaf((float)(unsigned)(a >> 32), 4294967296.f, (float)(unsigned)a);
    const float t = (af + 0.5f) * inv64;
    const float s = __fdividef(t, 2.f - t), s2 = s * s;
    float p = 1.f / 15.f;
    p = fmaf(p, s2, 1.f / 13.f);
    p = fmaf(p, s2, 1.f / 11.f);
    p = fmaf(p, s2, 1.f / 9.f);
    p = fmaf(p, s2, 1.f / 7.f);
    p = fmaf(p, s2, 1.f / 5.f);
    p = fmaf(p, s2, 1.f / 3.f);
    p = fmaf(p, s2, 1.f);
    const float lnu = hi ? -2.f * s * p : __logf(t);
    return -2.f * lnu;  // > 0
}
__device__ __forceinline__ float gauss32(uint64_t A, uint64_t B) {
    const float x = gauss32_r2(A);
    // cos(2 pi v) = -cos(2 pi (v - 1/2)), argument in (-pi, pi) for the hardware cosine
    const float w = ((float)(int)((unsigned)(B >> 32) ^ 0x80000000u) + 0.5f) * 2.3283064365386963e-10f;  // 2^-32
    return -(x * rsqrtf(x)) * __cosf(6.28318530717958647692f * w);
}

// gauss32 with cospif for the cosine: within an ulp or two of the result even where the cosine
// is near zero (__cosf's error is absolute, 2^-21.4), for uses that normalise a triple of normals,
// where a small length would magnify that absolute error
__device__ __forceinline__ float gauss32_cospi(uint64_t A, uint64_t B) {
    const float x = gauss32_r2(A);
    // cos(2 pi v) = -cos(pi (2 v - 1)), 2 v - 1 in (-1, 1) from the top 32 bits of B
    const float w2 = ((float)(int)((unsigned)(B >> 32) ^ 0x80000000u) + 0.5f) * 4.6566128730773926e-10f;  // 2^-31
    return -(x * rsqrtf(x)) * cospif(w2);
}

template <typename T> __device__ __forceinline__ T gauss(uint64_t A, uint64_t B);
template <> __device__ __forceinline__ float gauss<float>(uint64_t A, uint64_t B) { return gauss32(A, B); }
template <> __device__ __forceinline__ double gauss<double>(uint64_t A, uint64_t B) { return gauss64(A, B); }

// Start states.  A thread's state is sum_i q_i A^i s0 over the bits q_i of its jump polynomial
// (A: one xoshiro256** step, sums in GF(2)).  Each block tabulates A^i s0 for i = 0..255 in
// shared memory once; a thread's state is then the XOR of the entries its bits select
// (a broadcast load and an and-xor per word and bit, against a full state step per bit for
// Horner's rule).
__device__ __forceinline__ void noise_state_table(const RngState &s0, ulonglong4 *tab) {
    if (threadIdx.x == 0) {
        uint64_t a0 = s0.s[0], a1 = s0.s[1], a2 = s0.s[2], a3 = s0.s[3];
        for (int i = 0; i < 256; i++) {
            tab[i] = make_ulonglong4(a0, a1, a2, a3);
            dnext(a0, a1, a2, a3);
        }
    }
    __syncthreads();
}

// the state q(A) s0 for the polynomial q (four words) from the block's table of A^i s0
__device__ __forceinline__ void jump_state(const ulonglong4 *tab, const uint64_t *__restrict__ q, uint64_t &r0,
                                           uint64_t &r1, uint64_t &r2, uint64_t &r3) {
#pragma unroll 1
    for (int wq = 0; wq < 4; wq++) {
        const unsigned long long w = q[wq];
        const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
#pragma unroll 8
        for (int bit = 0; bit < 64; bit++) {
            const unsigned m = 0u - (((bit < 32 ? lo : hi) >> (bit & 31)) & 1u);
            const uint64_t mm = ((uint64_t)m << 32) | m;
            const ulonglong4 e = tab[wq * 64 + bit];
            r0 ^= e.x & mm;
            r1 ^= e.y & mm;
            r2 ^= e.z & mm;
            r3 ^= e.w & mm;
        }
    }
}

// device table of the polynomials x^(first + stride c) mod p, c < count (four words each); cached
// per (first, stride, count) until mitos_release_all
const uint64_t *affine_jump_polys(unsigned long long first, unsigned long long stride, long count);

}  // namespace mitos
