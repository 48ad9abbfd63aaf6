// ngenic.cu -- generate_ngeniclike_grf (src/grf_ngeniclike.c:28-203): the N-GenIC-style white
// noise field, one thread per (x, y) column.
//
// The reference draws from GSL's gsl_rng_ranlxd1: one generator seeded with Seed fills an N x N
// seed table in a mirrored order (:68-88); every column then reseeds the generator from its table
// entry (:108) and draws, for kz < N/2, a phase 2 pi U and an amplitude U != 0 (:111-114), so the
// columns are independent and run in parallel here.  delta = Box^(3/2) sqrt(-ln ampl) (:60-62,
// :145-148); (re, im) = delta (sin phase, cos phase); the kz = 0 plane writes the conjugate at
// (-x, -y) (:157-195); the Nyquist modes and kz = N/2 stay zero.  The reference repeats the fill
// for three axes with identical results (:90); it is done once.
//
// The generator is double-precision RANLUX at luxury level 1 (M. Luscher's ranlxd; GSL's
// ranlxd1): twelve 48-bit words, subtract with borrow x_n = x_{n-5} - x_{n-12} - c_{n-1}
// (mod 2^48), blocks of 202 steps of which the last 12 words are delivered, x / 2^48; seeding by
// a 31-bit shift register (tap 18) over the low 32 bits of the seed, 0 -> 1.  On the device the
// words live in shared memory, word-major ([word][thread]), so a warp's accesses are
// consecutive 8-byte words; every lane follows the same block and delivery schedule.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "context.cuh"

namespace mitos {

#define NG_THREADS 128
#define NG_LUX 202
static constexpr uint64_t NG_W48 = 1ULL << 48;

// ---- host generator (the seed table) ---------------------------------------------------------
struct HostRanlxd {
    uint64_t x[12];
    int carry = 0, i = 0, left = 0;
    explicit HostRanlxd(unsigned long seed) {
        if (seed == 0) seed = 1;
        uint32_t reg = (uint32_t)(seed & 0x7FFFFFFFUL);  // b[p] at bit p, p = 0..30
        int p = 0;
        for (int k = 0; k < 12; k++) {
            uint64_t v = 0;
            for (int l = 0; l < 48; l++) {
                const int b = (reg >> p) & 1, q = (reg >> ((p + 18) % 31)) & 1;
                v = 2 * v + (uint64_t)(1 - b);
                reg = (reg & ~(1u << p)) | ((uint32_t)(b ^ q) << p);
                p = (p + 1) % 31;
            }
            x[k] = v;
        }
    }
    double uniform() {
        if (left == 0) {
            for (int s = 0; s < NG_LUX; s++) {
                const int j = i + 7 < 12 ? i + 7 : i - 5;
                int64_t y = (int64_t)x[j] - (int64_t)x[i] - carry;
                carry = y < 0;
                if (y < 0) y += (int64_t)NG_W48;
                x[i] = (uint64_t)y;
                i = i + 1 < 12 ? i + 1 : 0;
            }
            left = 12;
        }
        int k = i + (12 - left);
        if (k >= 12) k -= 12;
        left--;
        return (double)x[k] / (double)NG_W48;
    }
};

static void seed_table(int N, unsigned long seed, std::vector<unsigned> &t) {
    HostRanlxd r(seed);
    t.assign((size_t)N * N, 0u);
    auto U = [&r]() { return (unsigned)(0x7fffffff * r.uniform()); };
    for (int i = 0; i < N / 2; i++) {
        for (int j = 0; j < i; j++) t[i * N + j] = U();
        for (int j = 0; j < i + 1; j++) t[j * N + i] = U();
        for (int j = 0; j < i; j++) t[(N - 1 - i) * N + j] = U();
        for (int j = 0; j < i + 1; j++) t[(N - 1 - j) * N + i] = U();
        for (int j = 0; j < i; j++) t[i * N + (N - 1 - j)] = U();
        for (int j = 0; j < i + 1; j++) t[j * N + (N - 1 - i)] = U();
        for (int j = 0; j < i; j++) t[(N - 1 - i) * N + (N - 1 - j)] = U();
        for (int j = 0; j < i + 1; j++) t[(N - 1 - j) * N + (N - 1 - i)] = U();
    }
}

// ---- device generator --------------------------------------------------------------------------
struct DevRanlxd {
    uint64_t (*x)[NG_THREADS];  // shared words, [word][thread]
    int t, carry, i, left;
    __device__ void seed(unsigned long s) {
        if (s == 0) s = 1;
        uint32_t reg = (uint32_t)(s & 0x7FFFFFFFUL);
        // rotating frame: bit 0 of reg is b[p], bit 18 is b[p + 18 mod 31]
        for (int k = 0; k < 12; k++) {
            uint64_t v = 0;
            for (int l = 0; l < 48; l++) {
                const uint32_t b = reg & 1u, q = (reg >> 18) & 1u;
                v = 2 * v + (uint64_t)(1u - b);
                reg = (reg >> 1) | ((b ^ q) << 30);
            }
            x[k][t] = v;
        }
        carry = 0;
        i = 0;
        left = 0;
    }
    __device__ double uniform() {
        if (left == 0) {
#pragma unroll 1
            for (int s = 0; s < NG_LUX; s++) {
                const int j = i + 7 < 12 ? i + 7 : i - 5;
                long long y = (long long)x[j][t] - (long long)x[i][t] - carry;
                carry = y < 0;
                if (y < 0) y += (long long)NG_W48;
                x[i][t] = (uint64_t)y;
                i = i + 1 < 12 ? i + 1 : 0;
            }
            left = 12;
        }
        int k = i + (12 - left);
        if (k >= 12) k -= 12;
        left--;
        return (double)x[k][t] * (1.0 / (double)NG_W48);
    }
};

template <typename T> __device__ __forceinline__ void amp_phase(double fac, double ampl, double u_phase, T &re, T &im);
template <> __device__ __forceinline__ void amp_phase<double>(double fac, double ampl, double u_phase, double &re, double &im) {
    const double phase = u_phase * 2 * M_PI;
    const double delta = fac * sqrt(-log(ampl));
    double s, c;
    sincos(phase, &s, &c);
    re = delta * s;
    im = delta * c;
}
// FP32 grids: the same arithmetic in single precision; ln of an amplitude near 1 goes through
// log1pf of the exact complement
template <> __device__ __forceinline__ void amp_phase<float>(double fac, double ampl, double u_phase, float &re, float &im) {
    const float lnu = ampl > 0.5 ? log1pf(-(float)(1.0 - ampl)) : logf((float)ampl);
    const float delta = (float)fac * sqrtf(-lnu);
    float s, c;
    sincospif((float)(2.0 * u_phase), &s, &c);
    re = delta * s;
    im = delta * c;
}

template <typename T>
__global__ void __launch_bounds__(NG_THREADS)
k_ngenic(int N, int NX, int X0, const unsigned *__restrict__ table, double fac, cplx<T> *__restrict__ out) {
    __shared__ uint64_t words[12][NG_THREADS];
    const long col = (long)blockIdx.x * NG_THREADS + threadIdx.x;
    if (col >= (long)N * N) return;
    const int i = (int)(col / N), j = (int)(col % N);
    const int ii = i == 0 ? 0 : N - i;
    const bool mine = i >= X0 && i < X0 + NX, partner = ii >= X0 && ii < X0 + NX;
    if (!mine && !partner) return;  // :104-105
    const int H = N / 2 + 1;
    DevRanlxd r{words, (int)threadIdx.x, 0, 0, 0};
    r.seed(table[col]);
#pragma unroll 1
    for (int k = 0; k < N / 2; k++) {
        const double up = r.uniform();
        double ampl;
        do ampl = r.uniform();
        while (ampl == 0);
        if (i == N / 2 || j == N / 2 || k == N / 2) continue;
        if (i == 0 && j == 0 && k == 0) continue;
        T re, im;
        amp_phase<T>(fac, ampl, up, re, im);
        if (k > 0) {
            if (mine) out[((long)(i - X0) * N + j) * H + k] = mk<T>(re, im);
        } else if (i == 0) {
            if (j >= N / 2) continue;
            if (mine) {
                out[(long)j * H] = mk<T>(re, im);
                out[(long)(N - j) * H] = mk<T>(re, -im);
            }
        } else {
            if (i >= N / 2) continue;
            const int jj = j == 0 ? 0 : N - j;
            if (mine) out[((long)(i - X0) * N + j) * H] = mk<T>(re, im);
            if (partner) out[((long)(ii - X0) * N + jj) * H] = mk<T>(re, -im);
        }
    }
}

static int ngenic_launch(int N, int NX, int X0, double boxlen, long seed, int precision, void *fbox) {
    if (N < 2 || N % 2 || NX < 1 || X0 < 0 || X0 + NX > N || boxlen <= 0) {
        set_error(1, "invalid grid for generate_ngeniclike_grf");
        return 1;
    }
    std::vector<unsigned> t;
    seed_table(N, (unsigned long)seed, t);
    unsigned *dt = (unsigned *)workspace(sizeof(unsigned) * (size_t)N * N, 140);
    if (!dt) return 4;  // :68-69 returns 4 when the seed table cannot be allocated
    MITOS_CUDA(cudaMemcpyAsync(dt, t.data(), sizeof(unsigned) * t.size(), cudaMemcpyHostToDevice, stream()));
    const size_t cs = precision == MITOS_FP32 ? 8 : 16;
    MITOS_CUDA(cudaMemsetAsync(fbox, 0, cs * (size_t)NX * N * (N / 2 + 1), stream()));  // :92-99
    double fac = pow(boxlen, 1.5) / sqrt(2.0);  // :60
    fac *= sqrt(2.0);                            // :62
    const unsigned blocks = (unsigned)(((long)N * N + NG_THREADS - 1) / NG_THREADS);
    launch_begin("ngenic");
    if (precision == MITOS_FP32)
        k_ngenic<float><<<blocks, NG_THREADS, 0, stream()>>>(N, NX, X0, dt, fac, (cplx<float> *)fbox);
    else
        k_ngenic<double><<<blocks, NG_THREADS, 0, stream()>>>(N, NX, X0, dt, fac, (cplx<double> *)fbox);
    count_launch();
    MITOS_LAUNCH_CHECK("N-GenIC-like noise");
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    return 0;
}

}  // namespace mitos

using namespace mitos;

extern "C" int generate_ngeniclike_grf(mitos_c128 *fbox, int N, int NX, int X0, long block_size, double boxlen,
                                       long seed) {
    (void)block_size;  // unused by the reference too
    if (!fbox) return 1;
    return ngenic_launch(N, NX, X0, boxlen, seed, MITOS_FP64, fbox);
}

extern "C" int generate_ngeniclike_grf_dg(struct distributed_grid *grf, long seed) {
    if (!grf || !grf->fbox) return 1;
    const int e = ngenic_launch(grf->N, (int)grf->NX, (int)grf->X0, grf->boxlen, seed, grf->precision, grf->fbox);
    if (!e) grf->momentum_space = 1;
    return e;
}

extern "C" int mitos_ranlxd1_uniforms(unsigned long seed, long n, double *out) {
    if (!out || n < 0) return 1;
    HostRanlxd r(seed);
    for (long i = 0; i < n; i++) out[i] = r.uniform();
    return 0;
}
