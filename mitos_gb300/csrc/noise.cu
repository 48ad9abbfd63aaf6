// noise.cu -- white noise with the reference's sequential xoshiro256** stream, generated one
// (x, y) column per thread on the GPU.
//
// src/grf.c:47-63 draws, on one rank, the modes in x -> y -> z order (z fastest) from one
// stream; each mode with k > 0 takes two sampleNorm calls (four 64-bit draws, real part
// first, src/random.c:34-49) and the DC mode takes none.  Column c = x N + y therefore starts
// at draw offset 0 (c = 0) or 4 (c (N/2+1) - 1) (c > 0).
//
// xoshiro256** is linear over GF(2) on its 256-bit state, so the state after J steps is
// q_J(A) s0, with A the one-step transition and q_J(x) = x^J mod p(x), p the characteristic
// polynomial of A.  p is recovered once with Berlekamp-Massey from 512 output bits; the
// polynomials of all column offsets are computed on the host (cached per N); on the GPU each
// block tabulates A^i s0 (i < 256) and a thread's start state q_c(A) s0 is the XOR of the entries
// selected by the bits of q_c.
#include <math.h>
#include <string.h>

#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "context.cuh"
#include "rng.cuh"

namespace mitos {

// ---- GF(2) polynomial arithmetic modulo p(x) = x^256 + plow(x) ------------------------------
struct Poly {
    uint64_t w[4];
};
static Poly g_plow;
static bool g_pready = false;
static std::mutex g_nmu;

static inline uint64_t rotl64h(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline void xo_step(uint64_t s[4]) {
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64h(s[3], 45);
}

static void pmulmod(const Poly &a, const Poly &b, Poly &out) {
    uint64_t r[9] = {0};
    for (int i = 0; i < 256; i++) {
        if (!((a.w[i >> 6] >> (i & 63)) & 1)) continue;
        const int ws = i >> 6, bs = i & 63;
        for (int j = 0; j < 4; j++) {
            r[j + ws] ^= b.w[j] << bs;
            if (bs) r[j + ws + 1] ^= b.w[j] >> (64 - bs);
        }
    }
    for (int i = 511; i >= 256; i--) {
        if (!((r[i >> 6] >> (i & 63)) & 1)) continue;
        r[i >> 6] ^= 1ULL << (i & 63);
        const int sh = i - 256, ws = sh >> 6, bs = sh & 63;
        for (int j = 0; j < 4; j++) {
            r[j + ws] ^= g_plow.w[j] << bs;
            if (bs) r[j + ws + 1] ^= g_plow.w[j] >> (64 - bs);
        }
    }
    memcpy(out.w, r, sizeof out.w);
}

static void pmulx(Poly &a) {
    const uint64_t top = a.w[3] >> 63;
    a.w[3] = (a.w[3] << 1) | (a.w[2] >> 63);
    a.w[2] = (a.w[2] << 1) | (a.w[1] >> 63);
    a.w[1] = (a.w[1] << 1) | (a.w[0] >> 63);
    a.w[0] <<= 1;
    if (top)
        for (int j = 0; j < 4; j++) a.w[j] ^= g_plow.w[j];
}

static Poly ppow_x(unsigned long long e) {  // x^e mod p
    Poly r = {{1, 0, 0, 0}};
    Poly b = {{2, 0, 0, 0}};  // x
    while (e) {
        if (e & 1) pmulmod(r, b, r);
        e >>= 1;
        if (e) pmulmod(b, b, b);
    }
    return r;
}

// Horner evaluation q(A) s0 on the host
static void horner(const Poly &q, const uint64_t s0[4], uint64_t out[4]) {
    uint64_t r[4] = {0, 0, 0, 0};
    for (int i = 255; i >= 0; i--) {
        xo_step(r);
        if ((q.w[i >> 6] >> (i & 63)) & 1)
            for (int j = 0; j < 4; j++) r[j] ^= s0[j];
    }
    memcpy(out, r, 4 * sizeof(uint64_t));
}

// Berlekamp-Massey on bit 0 of s[0]; p(x) is the reciprocal of the connection polynomial
static bool charpoly_init() {
    if (g_pready) return true;
    uint64_t s[4] = {0x9E3779B97f4A7C15ULL, 0xBF58476D1CE4E5B9ULL, 0x94D049BB133111EBULL, 1ULL};
    const int NB = 512;
    std::vector<uint8_t> b(NB);
    for (int n = 0; n < NB; n++) {
        b[n] = (uint8_t)(s[0] & 1);
        xo_step(s);
    }
    std::vector<uint8_t> C(NB + 1, 0), B(NB + 1, 0), T;
    C[0] = B[0] = 1;
    int L = 0, m = 1;
    for (int n = 0; n < NB; n++) {
        uint8_t d = b[n];
        for (int i = 1; i <= L; i++) d ^= C[i] & b[n - i];
        if (!d) {
            m++;
        } else if (2 * L <= n) {
            T = C;
            for (int i = 0; i + m <= NB; i++) C[i + m] ^= B[i];
            L = n + 1 - L;
            B = T;
            m = 1;
        } else {
            for (int i = 0; i + m <= NB; i++) C[i + m] ^= B[i];
            m++;
        }
    }
    if (L != 256) return false;
    memset(&g_plow, 0, sizeof g_plow);
    for (int j = 0; j < 256; j++)
        if (C[256 - j]) g_plow.w[j >> 6] |= 1ULL << (j & 63);
    // self-check: a jump of 1000 steps must equal 1000 sequential steps
    uint64_t s0[4] = {1, 2, 3, 4}, seq[4] = {1, 2, 3, 4}, jmp[4];
    for (int i = 0; i < 1000; i++) xo_step(seq);
    g_pready = true;
    horner(ppow_x(1000), s0, jmp);
    if (memcmp(seq, jmp, sizeof seq) != 0) {
        g_pready = false;
        return false;
    }
    return true;
}

void rng_jump(uint64_t st[4], unsigned long long n) {
    std::lock_guard<std::mutex> lk(g_nmu);
    if (!charpoly_init()) return;
    uint64_t out[4];
    horner(ppow_x(n), st, out);
    memcpy(st, out, sizeof out);
}

// x^(first + stride c) mod p for c < count into tab (four words each), on the host's threads:
// each step multiplies by x^stride through the table MT[i] = x^(stride + i) mod p
static void fill_affine(uint64_t *tab, unsigned long long first, unsigned long long stride, long count) {
    std::vector<Poly> MT(256);
    MT[0] = ppow_x(stride);
    for (int i = 1; i < 256; i++) {
        MT[i] = MT[i - 1];
        pmulx(MT[i]);
    }
    unsigned nth = std::thread::hardware_concurrency();
    if (nth < 1) nth = 1;
    if (nth > 32) nth = 32;
    if (count < 4096) nth = 1;
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nth; w++) {
        th.emplace_back([&, w]() {
            const long c0 = count * w / nth, c1 = count * (w + 1) / nth;
            Poly q;
            for (long c = c0; c < c1; c++) {
                if (c == c0) {
                    q = ppow_x(first + stride * (unsigned long long)c);
                } else {
                    Poly r = {{0, 0, 0, 0}};
                    for (int i = 0; i < 256; i++)
                        if ((q.w[i >> 6] >> (i & 63)) & 1)
                            for (int j = 0; j < 4; j++) r.w[j] ^= MT[i].w[j];
                    q = r;
                }
                memcpy(&tab[4 * c], q.w, sizeof q.w);
            }
        });
    }
    for (auto &t : th) t.join();
}

static uint64_t *upload_polys(const std::vector<uint64_t> &tab, const char *what) {
    uint64_t *d = nullptr;
    if (cudaMalloc(&d, sizeof(uint64_t) * tab.size()) != cudaSuccess) {
        cudaGetLastError();
        set_error(5, what);
        return nullptr;
    }
    cudaMemcpy(d, tab.data(), sizeof(uint64_t) * tab.size(), cudaMemcpyHostToDevice);
    return d;
}

// per-N table of column polynomials (device), 4 x uint64 per column: column 0 starts at draw 0,
// column c > 0 at T c - 4 (T = 4 (N/2 + 1) draws a column, none for the DC mode)
static std::map<int, uint64_t *> g_ptabs;
static const uint64_t *column_polys(int N) {
    std::lock_guard<std::mutex> lk(g_nmu);
    auto it = g_ptabs.find(N);
    if (it != g_ptabs.end()) return it->second;
    if (!charpoly_init()) {
        set_error(4, "xoshiro256** characteristic polynomial check failed");
        return nullptr;
    }
    const long ncol = (long)N * N;
    const unsigned long long T = 4ULL * (N / 2 + 1);
    std::vector<uint64_t> tab(4 * ncol, 0);
    tab[0] = 1;
    if (ncol > 1) fill_affine(tab.data() + 4, T - 4, T, ncol - 1);
    uint64_t *d = upload_polys(tab, "out of device memory for the noise column table");
    if (d) g_ptabs[N] = d;
    return d;
}

struct AffineKey {
    unsigned long long first, stride;
    long count;
    bool operator<(const AffineKey &o) const {
        if (first != o.first) return first < o.first;
        if (stride != o.stride) return stride < o.stride;
        return count < o.count;
    }
};
static std::map<AffineKey, uint64_t *> g_atabs;
const uint64_t *affine_jump_polys(unsigned long long first, unsigned long long stride, long count) {
    std::lock_guard<std::mutex> lk(g_nmu);
    const AffineKey key{first, stride, count};
    auto it = g_atabs.find(key);
    if (it != g_atabs.end()) return it->second;
    if (!charpoly_init()) {
        set_error(4, "xoshiro256** characteristic polynomial check failed");
        return nullptr;
    }
    std::vector<uint64_t> tab(4 * (size_t)count);
    fill_affine(tab.data(), first, stride, count);
    uint64_t *d = upload_polys(tab, "out of device memory for a jump table");
    if (d) g_atabs[key] = d;
    return d;
}

void release_jump_tables() {
    std::lock_guard<std::mutex> lk(g_nmu);
    for (auto &kv : g_ptabs) cudaFree(kv.second);
    g_ptabs.clear();
    for (auto &kv : g_atabs) cudaFree(kv.second);
    g_atabs.clear();
}

#define NOISE_THREADS 128
#define NOISE_CHUNK 16

// One thread generates one column (x, y) of the half-complex grid, z fastest, from its jumped
// state.  (Two consecutive columns a thread, the second continuing the first's stream without a
// jump, measured slower at 512^3: 0.678 against 0.660 ms, with half the warps to hide the
// xoshiro dependency chains.)  Values are staged per chunk of z and written as rows.
// A^i s0 (i < 256) of each realisation's start state, once per launch: the table every block of
// k_noise reads (a single thread stepping 256 times in each block left the block's other threads
// waiting at its barrier)
__global__ void k_state_tables(RngState s0, const RngState *__restrict__ states, int nb, ulonglong4 *__restrict__ tab) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const RngState s = states ? states[b] : s0;
    uint64_t a0 = s.s[0], a1 = s.s[1], a2 = s.s[2], a3 = s.s[3];
    for (int i = 0; i < 256; i++) {
        tab[(size_t)b * 256 + i] = make_ulonglong4(a0, a1, a2, a3);
        dnext(a0, a1, a2, a3);
    }
}

template <typename T>
__global__ void __launch_bounds__(NOISE_THREADS)
k_noise(int N, const uint64_t *__restrict__ polys, const ulonglong4 *__restrict__ gtab, T factor,
        const T *__restrict__ filt, cplx<T> *__restrict__ out, size_t ostride, uint4 *__restrict__ zero,
        size_t zero_n16) {
    // the optional buffer to clear, 16 bytes a streaming store, strided over the whole grid of
    // threads and spread over the z chunks below, so the stores drain while the generator's integer
    // work runs.  (At 512^3 the clearing adds about 0.1 ms to the kernel, what the separate memset
    // took: 8.81-8.84 ms an IC either way.)
    const size_t zstep = (size_t)gridDim.x * gridDim.y * blockDim.x;
    size_t zi = ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
    const int H0 = N / 2 + 1, nchunks = (H0 + NOISE_CHUNK - 1) / NOISE_CHUNK;
    const int zper = zero ? (int)((zero_n16 / zstep + 1 + nchunks - 1) / nchunks) : 0;
    // batched launches: realisation blockIdx.y has its own state table and output grid
    out = bat<cplx<T>>(out, (size_t)blockIdx.y * ostride);
    __shared__ cplx<T> stage[NOISE_THREADS][NOISE_CHUNK + 1];
    __shared__ ulonglong4 tab[256];
    for (int i = threadIdx.x; i < 256; i += NOISE_THREADS) tab[i] = gtab[(size_t)blockIdx.y * 256 + i];
    __syncthreads();
    const int H = N / 2 + 1;
    const long ncol = (long)N * N;
    const long cblock = (long)blockIdx.x * NOISE_THREADS;  // first column of the block
    const long c0 = cblock + threadIdx.x;
    const bool valid = c0 < ncol;
    uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    if (valid) jump_state(tab, polys + 4 * c0, r0, r1, r2, r3);
    {
        const long c = c0;
        const int kx = valid ? kint((int)(c / N), N) : 0;
        const int ky = valid ? kint((int)(c % N), N) : 0;
        for (int z0 = 0; z0 < H; z0 += NOISE_CHUNK) {
            for (int k = 0; k < zper && zi < zero_n16; k++, zi += zstep) __stcs(zero + zi, make_uint4(0, 0, 0, 0));
            const int cz = (H - z0) < NOISE_CHUNK ? (H - z0) : NOISE_CHUNK;
            if (valid) {
                for (int j = 0; j < cz; j++) {
                    const int z = z0 + j;
                    cplx<T> val = mk<T>(0, 0);
                    const int n2 = kx * kx + ky * ky + z * z;
                    if (n2 > 0) {
                        const uint64_t A = dnext(r0, r1, r2, r3), B = dnext(r0, r1, r2, r3);
                        const uint64_t C2 = dnext(r0, r1, r2, r3), D = dnext(r0, r1, r2, r3);
                        T a = gauss<T>(A, B) * factor;
                        T b = gauss<T>(C2, D) * factor;
                        if (filt) {
                            const T f = filt[n2];
                            a *= f;
                            b *= f;
                        }
                        val = mk<T>(a, b);
                    }
                    stage[threadIdx.x][j] = val;
                }
            }
            __syncthreads();
            // write-out: row of thread rr is column cblock + rr
            if (cz == NOISE_CHUNK) {
                static_assert((NOISE_CHUNK & (NOISE_CHUNK - 1)) == 0, "chunk is a power of two");
                constexpr int SH = __builtin_ctz(NOISE_CHUNK);
#pragma unroll 4
                for (int idx = threadIdx.x; idx < NOISE_THREADS * NOISE_CHUNK; idx += NOISE_THREADS) {
                    const int rr = idx >> SH, j = idx & (NOISE_CHUNK - 1);
                    const long cc = cblock + rr;
                    if (cc < ncol) __stcs(out + cc * H + z0 + j, stage[rr][j]);
                }
            } else {
                for (int idx = threadIdx.x; idx < NOISE_THREADS * cz; idx += NOISE_THREADS) {
                    const int rr = idx / cz, j = idx % cz;
                    const long cc = cblock + rr;
                    if (cc < ncol) __stcs(out + cc * H + z0 + j, stage[rr][j]);
                }
            }
            __syncthreads();
        }
    }
    for (; zero && zi < zero_n16; zi += zstep) __stcs(zero + zi, make_uint4(0, 0, 0, 0));
}

// enforce_hermiticity on the kz = 0 and kz = N/2 planes (src/grf.c:103-137): targets are never
// sources, so the planes are fixed in place
template <typename T>
__global__ void k_hermitian(int N, cplx<T> *fbox, size_t bstride) {
    const int H = N / 2 + 1;
    const int x = blockIdx.y;  // 0 .. N/2
    const int zsel = blockIdx.z & 1;
    fbox = bat<cplx<T>>(fbox, (size_t)(blockIdx.z >> 1) * bstride);  // realisation of a batch
    const int z = zsel ? N / 2 : 0;
    for (int y = blockIdx.x * blockDim.x + threadIdx.x; y < N; y += gridDim.x * blockDim.x) {
        if ((x == 0 || x == N / 2) && y > N / 2) continue;
        const int invx = (x > 0) ? N - x : 0;
        const int invy = (y > 0) ? N - y : 0;
        const long id = ((long)x * N + y) * H + z;
        if (invx == x && invy == y) {
            fbox[id].y = 0;
        } else {
            const cplx<T> s = fbox[((long)invx * N + invy) * H + z];
            fbox[id] = mk<T>(s.x, -s.y);
        }
    }
}

int noise_generate(const GridGeom &g, int precision, double boxlen, uint64_t st[4],
                   const void *filter_by_n2, void *fbox, const void *states, int batch, size_t bstride,
                   void *zero, size_t zero_bytes) {
    if (zero && (((uintptr_t)zero & 15) || (zero_bytes & 15))) {
        set_error(3, "noise: the buffer to clear must be 16-byte aligned and sized");
        return 3;
    }
    const uint64_t *polys = column_polys(g.N);
    if (!polys) return 5;
    RngState s0;
    memcpy(s0.s, st, sizeof s0.s);
    const double boxvol = boxlen * boxlen * boxlen;
    const double factor = sqrt(boxvol / 2);  // src/grf.c:33
    const long ncol = (long)g.N * g.N;
    const int nb = states && batch > 1 ? batch : 1;
    const unsigned blocks = (unsigned)((ncol + NOISE_THREADS - 1) / NOISE_THREADS);
    const dim3 grid(blocks, nb);
    const RngState *sts = (const RngState *)states;
    ulonglong4 *tab = (ulonglong4 *)workspace(sizeof(ulonglong4) * 256 * (size_t)nb, 160);
    if (!tab) return 5;
    launch_begin("state_tables");
    k_state_tables<<<(nb + 31) / 32, 32, 0, stream()>>>(s0, sts, nb, tab);
    count_launch();
    MITOS_LAUNCH_CHECK("noise state tables");
    const size_t ost = sts ? bstride : 0;
    launch_begin("noise");
    if (precision == MITOS_FP32) {
        k_noise<float><<<grid, NOISE_THREADS, 0, stream()>>>(g.N, polys, tab, (float)factor, (const float *)filter_by_n2,
                                                             (float2 *)fbox, ost, (uint4 *)zero, zero_bytes / 16);
    } else {
        k_noise<double><<<grid, NOISE_THREADS, 0, stream()>>>(g.N, polys, tab, factor, (const double *)filter_by_n2,
                                                              (double2 *)fbox, ost, (uint4 *)zero, zero_bytes / 16);
    }
    count_launch();
    MITOS_LAUNCH_CHECK("noise");
    return 0;
}

int hermitian_planes(const GridGeom &g, int precision, void *fbox, int batch, size_t bstride) {
    dim3 grid((g.N + 255) / 256, g.N / 2 + 1, 2 * (batch > 1 ? batch : 1));
    launch_begin("hermitian");
    if (precision == MITOS_FP32) k_hermitian<float><<<grid, 256, 0, stream()>>>(g.N, (float2 *)fbox, bstride);
    else k_hermitian<double><<<grid, 256, 0, stream()>>>(g.N, (double2 *)fbox, bstride);
    count_launch();
    MITOS_LAUNCH_CHECK("hermitian planes");
    return 0;
}

}  // namespace mitos

// ---- host-only entry points for checking the jump-ahead without a GPU ---------------------
// state after n draws from s0 (polynomial jump)
extern "C" int mitos_rng_jump(uint64_t s[4], unsigned long long n) {
    mitos::rng_jump(s, n);
    return 0;
}
// start state of noise column c of an N grid (the state the GPU thread of column c uses)
extern "C" int mitos_noise_column_state(int N, long c, const uint64_t s0[4], uint64_t out[4]) {
    uint64_t s[4] = {s0[0], s0[1], s0[2], s0[3]};
    const unsigned long long T = 4ULL * (N / 2 + 1);
    mitos::rng_jump(s, c == 0 ? 0ULL : T * (unsigned long long)c - 4ULL);
    for (int i = 0; i < 4; i++) out[i] = s[i];
    return 0;
}

// ---- host copies of the FP64 Box-Muller transform and its correctly rounded log and cos ------
// (the device's operation sequence on the host; for checks without a GPU)
extern "C" double mitos_cr_log(double x) { return crm::cr_log(x); }
extern "C" double mitos_cr_cos(double y) { return crm::cr_cos(y); }
extern "C" double mitos_sample_norm_cr(uint64_t A, uint64_t B) { return crm::box_muller(A, B); }
// the fast step's rounding (NaN when its error interval straddles a rounding boundary) and the
// accurate step's, separately
extern "C" int mitos_cr_steps(int fn, double x, double *fast, double *accurate) {
    if (fn == 0) {
        const crm::LogArg a = crm::log_reduce(x);
        *fast = crm::ziv_round(crm::log_fast(a), crm::kZivEps);
        *accurate = crm::round_td(crm::log_accurate(a));
    } else {
        crm::CosArg ca;
        *fast = crm::ziv_round(crm::cos_fast(x, ca), crm::kZivEps);
        *accurate = crm::round_td(crm::cos_accurate(x));
    }
    return 0;
}
