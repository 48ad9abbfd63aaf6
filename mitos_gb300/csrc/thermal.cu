// thermal.cu -- thermal motion of a particle species on the GPU: the loop of src/mitos.c:928-965 and
// :1054-1062 (the branch without Firebolt, where every draw is accepted).  Particle i of the species
// (in id order) takes seven draws of the run's one xoshiro256** stream: a momentum from the
// inverse-CDF sampler of src/random.c:261-289, then three sampleNorm for a direction; its velocity
// gains n^ p / (a_ini M) c.
//
// Parallel form.  The draw count per particle is fixed, so particle i starts at draw 7 i of the
// species: a thread takes a run of R consecutive particles from its jumped start state (rng.cuh),
// stages its velocity increments in shared memory, and the block adds them to the velocities with
// consecutive threads on consecutive addresses.
//
// The sampler's piece choice compares u = (double)w / 2^64 (w the 64-bit draw; (double)UINT64_MAX
// is 2^64) with the pieces' CDF values.  Each comparison is exact in integers: the host finds, per
// piece, the largest w with u <= Fr, and a 1024-bucket table over the top bits of w gives the piece
// to start from.  Both precisions therefore pick the reference's piece for every draw.  The FP64
// build then evaluates the cubic, the momentum, the directions (GPU libm) and the float update with
// the reference's operations and rounding; the FP32 build evaluates them in float from the same
// piece (u - Fl taken exactly in integers first, so the cancellation costs no precision), with
// normals whose cosine is accurate near its zeros (a normalised triple of small normals would
// magnify an absolute error).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <vector>

#include "../../include/mitos_gb300.h"
#include "context.cuh"
#include "rng.cuh"

namespace mitos {

// ---- host: the sampler of src/random.c:87-209 for fd_pdf / be_pdf --------------------------------
// (the constants of include/random.h:35-39: 1000 midpoint cells, a 1000-entry search table, the
// momentum range [1e-10, 15] kT)
namespace {
constexpr int kCdfCells = 1000;
constexpr int kTableLen = 1000;

struct ThermalPdf {
    int kind;  // 1 Fermi-Dirac, 2 Bose-Einstein (src/random.c:52-71)
    double T, mu;
    double operator()(double x) const {
        if (x <= 0) return 0;
        return x * x / (exp((x - mu) / T) + (kind == 2 ? -1. : 1.));
    }
};

// Pieces of the inverse CDF, built by recursive halving.  A piece is halved while it holds more
// than 5% of the probability; then while its cubic Hermite interpolant of x(F) is not monotone or
// misses the CDF by more than 1e-6 at its middle.  Whether a piece is halved depends only on its
// own ends, so the recursion gives the reference's pieces, already in order.
struct PieceBuilder {
    ThermalPdf f;
    double xl, norm;
    std::vector<struct interval> out;
    bool overflow = false;

    double integral(double b) const {  // midpoint rule on [xl, b]
        const double h = (b - xl) / kCdfCells;
        double s = 0;
        for (int i = 0; i < kCdfCells; i++) s += h * f(xl + (i + 0.5) * h);
        return s;
    }
    double cdf(double x) const { return norm * integral(x); }

    void by_mass(double l, double r, double Fl, double Fr, int depth) {
        if (Fr - Fl > 0.05 && depth < 200) {
            const double m = l + 0.5 * (r - l), Fm = cdf(m);
            by_mass(l, m, Fl, Fm, depth + 1);
            by_mass(m, r, Fm, Fr, depth + 1);
        } else {
            overflow |= depth >= 200;
            by_fit(l, r, Fl, Fr, depth);
        }
    }
    void by_fit(double l, double r, double Fl, double Fr, int depth) {
        const double pl = norm * f(l), pr = norm * f(r), dF = Fr - Fl;
        struct interval iv;
        memset(&iv, 0, sizeof iv);
        iv.l = l;
        iv.r = r;
        iv.Fl = Fl;
        iv.Fr = Fr;
        iv.a0 = l;
        iv.a1 = dF / pl;
        iv.a2 = 3 * (r - l) - dF * (2. / pl + 1. / pr);
        iv.a3 = 2 * (l - r) + dF * (1. / pl + 1. / pr);
        const double xmid = iv.a0 + iv.a1 * 0.5 + iv.a2 * 0.25 + iv.a3 * 0.125;
        iv.error = fabs(cdf(xmid) - 0.5 * (Fr + Fl));
        const double slope = dF / (r - l);
        const bool monotone = slope <= 3 * pl && slope <= 3 * pr;
        if ((iv.error > 1e-6 || !monotone) && depth < 200) {
            const double m = l + 0.5 * (r - l), Fm = cdf(m);
            by_fit(l, m, Fl, Fm, depth + 1);
            by_fit(m, r, Fm, Fr, depth + 1);
        } else {
            overflow |= depth >= 200;
            out.push_back(iv);
        }
    }
};
}  // namespace

// ---- device table ------------------------------------------------------------------------------
// The reference's scan (src/random.c:270-280) starts at a search-table piece whose Fr is below
// u (or at piece 0) and steps on while Fr < u, so the piece it ends on is the last one with Fr < u,
// or piece 0 when there is none: the search table only makes the scan short.  With "Fr_j < u"
// exact as "w > le_j" (le_j below), the kernel starts from the last piece whose le lies below the
// start of w's bucket (top 10 bits of w) and steps on while w > le of the next piece: one table
// load, then usually one threshold compare.  The host checks that the sampler's search table is
// the one initSampler builds, which that argument assumes.
constexpr int kBucketBits = 10;
constexpr int kBuckets = 1 << kBucketBits;

struct ThermPiece {
    unsigned long long le;     // largest draw w with (double)w 2^-64 <= Fr: "Fr < u" is w > le
    unsigned long long flfix;  // floor(Fl 2^64)
    double Fl, Fr, a0, a1, a2, a3;
    float invw;                // FP32: 2^-64 / (Fr - Fl)
    float b0, b1, b2, b3;      // FP32 copies of a0..a3
    float pad;
};
static_assert(sizeof(ThermPiece) == 88, "piece layout");

// FP32 part of a piece, as kept in shared memory
struct PieceF {
    unsigned long long flfix;
    float invw, b0, b1, b2, b3, pad;
};
static_assert(sizeof(PieceF) == 32, "shared piece layout");

struct ThermTable {
    int n;
    const ThermPiece *piece;
    const unsigned short *bucket;  // [kBuckets]: piece to start from for the draws of each bucket
};

static unsigned long long largest_not_above(double Fr) {
    auto below = [&](unsigned long long w) { return (double)w * 0x1p-64 <= Fr; };
    if (below(~0ULL)) return ~0ULL;
    unsigned long long lo = 0, hi = ~0ULL;  // below(lo), !below(hi)
    while (hi - lo > 1) {
        const unsigned long long mid = lo + (hi - lo) / 2;
        if (below(mid)) lo = mid;
        else hi = mid;
    }
    return lo;
}

// host image of the device table of a sampler; 0 or status 3 for a sampler this kernel cannot take
static int table_image(const struct sampler *s, std::vector<unsigned char> &img, int &n) {
    n = s ? s->intervalNum : 0;
    if (!s || n < 1 || n > 65535 || s->I_max < 1 || !s->intervals || !s->index) {
        set_error(3, "thermal sampler: no pieces or no search table");
        return 3;
    }
    for (int j = 0; j < n; j++) {
        const struct interval &iv = s->intervals[j];
        // the reference scan also requires r > (the previous piece's r); with pieces in order and
        // increasing right ends that holds for every consecutive piece
        if (!(iv.r > 0) || !(iv.Fr >= 0) || !(iv.Fr - iv.Fl > 0) ||
            (j > 0 && (!(iv.r > s->intervals[j - 1].r) || !(iv.Fr > s->intervals[j - 1].Fr)))) {
            set_error(3, "thermal sampler: pieces not in order of increasing right end");
            return 3;
        }
    }
    // the search table must be initSampler's (src/random.c:191-206)
    for (int i = 0; i < s->I_max; i++) {
        const double u = (double)i / s->I_max;
        double rmax = 0;
        int want = 0;
        for (int j = 0; j < n; j++)
            if (s->intervals[j].Fr < u && s->intervals[j].r > rmax) {
                rmax = s->intervals[j].r;
                want = j;
            }
        if (s->index[i] != (double)want) {
            set_error(3, "thermal sampler: search table is not the one initSampler builds");
            return 3;
        }
    }
    const size_t pb = sizeof(ThermPiece) * n;
    img.assign(pb + sizeof(unsigned short) * kBuckets, 0);
    ThermPiece *pc = (ThermPiece *)img.data();
    for (int j = 0; j < n; j++) {
        const struct interval &iv = s->intervals[j];
        ThermPiece &p = pc[j];
        p.le = largest_not_above(iv.Fr);
        const double fl = iv.Fl * 0x1p64;
        p.flfix = fl <= 0 ? 0ULL : (fl >= 0x1p64 ? ~0ULL : (unsigned long long)fl);
        p.Fl = iv.Fl;
        p.Fr = iv.Fr;
        p.a0 = iv.a0;
        p.a1 = iv.a1;
        p.a2 = iv.a2;
        p.a3 = iv.a3;
        p.invw = (float)(0x1p-64 / (iv.Fr - iv.Fl));
        p.b0 = (float)iv.a0;
        p.b1 = (float)iv.a1;
        p.b2 = (float)iv.a2;
        p.b3 = (float)iv.a3;
    }
    // bucket b holds the draws w >> (64 - kBucketBits) == b; its start piece is the pick of its
    // smallest draw: (number of pieces with le < w) - 1, at least 0
    unsigned short *bucket = (unsigned short *)(img.data() + pb);
    int c = 0;
    for (int b = 0; b < kBuckets; b++) {
        const unsigned long long w0 = (unsigned long long)b << (64 - kBucketBits);
        while (c < n && pc[c].le < w0) c++;
        bucket[b] = (unsigned short)(c > 0 ? c - 1 : 0);
    }
    return 0;
}

static ThermTable table_view(const void *dev, int n) {
    ThermTable t;
    t.n = n;
    t.piece = (const ThermPiece *)dev;
    t.bucket = (const unsigned short *)((const char *)dev + sizeof(ThermPiece) * n);
    return t;
}

// ---- kernel ------------------------------------------------------------------------------------
#define THERMAL_THREADS 128
#define THERMAL_CHUNK 8

// Shared memory: the block's table of A^i s0 (8 KB) while the threads jump to their start states,
// then, in the same bytes, the bucket table, the thresholds and (FP32) the pieces.
__host__ __device__ constexpr size_t thermal_smem(int n) {
    const size_t tables = sizeof(unsigned short) * kBuckets + (sizeof(unsigned long long) + sizeof(PieceF)) * (size_t)n;
    return tables > 256 * sizeof(ulonglong4) ? tables : 256 * sizeof(ulonglong4);
}

// PACKED: velocities at stride 3 from a 16-byte aligned base and runs of a multiple of 4 particles,
// so each thread adds its increments itself, three float4 a group of 4 particles (loaded before the
// group computes); otherwise increments are staged in shared memory and the block adds them with
// consecutive threads on consecutive addresses
template <typename T, bool PACKED>
__global__ void __launch_bounds__(THERMAL_THREADS, sizeof(T) == 4 ? 10 : 6)
k_thermal(long n, int R, RngState s0, const uint64_t *__restrict__ polys, ThermTable tt, double a_ini, double M_eV,
          double c, float vfac, float *__restrict__ vel, long stride, int *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    ulonglong4 *tab = (ulonglong4 *)smem;
    noise_state_table(s0, tab);
    const long g = (long)blockIdx.x * THERMAL_THREADS + threadIdx.x;
    const long first = g * R;
    uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    if (first < n) jump_state(tab, polys + 4 * g, r0, r1, r2, r3);
    __syncthreads();
    // the sampler tables over the jump table
    PieceF *spf = (PieceF *)smem;
    unsigned long long *sle = (unsigned long long *)(spf + tt.n);
    unsigned short *sbk = (unsigned short *)(sle + tt.n);
    for (int i = threadIdx.x; i < tt.n; i += THERMAL_THREADS) {
        const ThermPiece &P = tt.piece[i];
        sle[i] = P.le;
        spf[i] = PieceF{P.flfix, P.invw, P.b0, P.b1, P.b2, P.b3, 0.f};
    }
    for (int i = threadIdx.x; i < kBuckets; i += THERMAL_THREADS) sbk[i] = tt.bucket[i];
    __syncthreads();
    const long block_first = (long)blockIdx.x * THERMAL_THREADS * R;
    bool bad = false;
    // one particle: its seven draws, momentum and direction; d = its velocity increment
    auto one = [&](T *d) {
        const uint64_t w = dnext(r0, r1, r2, r3);
        int pk = sbk[w >> (64 - kBucketBits)];
        while (pk + 1 < tt.n && w > sle[pk + 1]) pk++;
        if constexpr (sizeof(T) == 8) {
            // src/random.c:284-286, src/mitos.c:935-965 with the reference's rounding
            const ThermPiece &P = tt.piece[pk];
            const double u = __dmul_rn(__ull2double_rn(w), 0x1p-64);
            const double v = __ddiv_rn(__dsub_rn(u, P.Fl), __dsub_rn(P.Fr, P.Fl));
            const double H = __dadd_rn(__dadd_rn(__dadd_rn(P.a0, __dmul_rn(P.a1, v)), __dmul_rn(__dmul_rn(P.a2, v), v)),
                                       __dmul_rn(__dmul_rn(__dmul_rn(P.a3, v), v), v));
            const double p = __ddiv_rn(H, a_ini);
            bad |= isnan(p) || p <= 0;
            const double V = __dmul_rn(__ddiv_rn(p, M_eV), c);
            double e[3];
            for (int m = 0; m < 3; m++) {
                const uint64_t A = dnext(r0, r1, r2, r3), B = dnext(r0, r1, r2, r3);
                e[m] = gauss64_libm(A, B);
            }
            const double len = hypot(e[0], hypot(e[1], e[2]));
            if (len > 0)
                for (int m = 0; m < 3; m++) e[m] = __ddiv_rn(e[m], len);
            for (int m = 0; m < 3; m++) d[m] = __dmul_rn(e[m], V);
        } else {
            const PieceF P = spf[pk];
            const long long diff = (long long)(w - P.flfix);  // (u - Fl) 2^64, exact
            const float dv = fmaf((float)(int)(diff >> 32), 4294967296.f, (float)(unsigned)diff);
            const float v = dv * P.invw;
            const float H = fmaf(fmaf(fmaf(P.b3, v, P.b2), v, P.b1), v, P.b0);
            bad |= !(H > 0.f);
            const float V = H * vfac;
            float e[3];
            for (int m = 0; m < 3; m++) {
                const uint64_t A = dnext(r0, r1, r2, r3), B = dnext(r0, r1, r2, r3);
                e[m] = gauss32_cospi(A, B);
            }
            const float l2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
            const float sc = l2 > 0.f ? rsqrtf(l2) * V : V;
            for (int m = 0; m < 3; m++) d[m] = e[m] * sc;
        }
    };
    // v + d in the reference's arithmetic: float + double rounded once (FP64), float (FP32)
    auto addv = [](float v, T d) -> float {
        if constexpr (sizeof(T) == 8) return __double2float_rn(__dadd_rn((double)v, d));
        else return v + d;
    };
    if constexpr (PACKED) {
        for (int k0 = 0; k0 < R; k0 += 4) {
            const long p0 = first + k0;
            if (p0 >= n) break;
            const int cnt = n - p0 < 4 ? (int)(n - p0) : 4;
            float *q = vel + 3 * p0;
            float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0;
            if (cnt == 4) {
                q0 = reinterpret_cast<const float4 *>(q)[0];
                q1 = reinterpret_cast<const float4 *>(q)[1];
                q2 = reinterpret_cast<const float4 *>(q)[2];
            }
            T d[12];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (j < cnt) one(d + 3 * j);
                else d[3 * j] = d[3 * j + 1] = d[3 * j + 2] = 0;
            }
            if (cnt == 4) {
                q0 = make_float4(addv(q0.x, d[0]), addv(q0.y, d[1]), addv(q0.z, d[2]), addv(q0.w, d[3]));
                q1 = make_float4(addv(q1.x, d[4]), addv(q1.y, d[5]), addv(q1.z, d[6]), addv(q1.w, d[7]));
                q2 = make_float4(addv(q2.x, d[8]), addv(q2.y, d[9]), addv(q2.z, d[10]), addv(q2.w, d[11]));
                reinterpret_cast<float4 *>(q)[0] = q0;
                reinterpret_cast<float4 *>(q)[1] = q1;
                reinterpret_cast<float4 *>(q)[2] = q2;
            } else {
#pragma unroll
                for (int i = 0; i < 12; i++)
                    if (i < 3 * cnt) q[i] = addv(q[i], d[i]);
            }
        }
    } else {
        __shared__ T stage[THERMAL_THREADS][3 * THERMAL_CHUNK + 1];
        for (int k0 = 0; k0 < R; k0 += THERMAL_CHUNK) {
            // the velocities this chunk adds to, on their way to L2 while the chunk computes
            if (first + k0 < n) {
                const long last = min(first + k0 + THERMAL_CHUNK, min(first + R, n)) - 1;
                prefetch_l2(vel + (first + k0) * stride);
                prefetch_l2(vel + last * stride + 2);
            }
            for (int j = 0; j < THERMAL_CHUNK; j++) {
                T d[3] = {0, 0, 0};
                if (k0 + j < R && first + k0 + j < n) one(d);
                for (int m = 0; m < 3; m++) stage[threadIdx.x][3 * j + m] = d[m];
            }
            __syncthreads();
            // add the block's increments: thread t's run starts at particle block_first + t R
            for (int idx = threadIdx.x; idx < THERMAL_THREADS * 3 * THERMAL_CHUNK; idx += THERMAL_THREADS) {
                const int t = idx / (3 * THERMAL_CHUNK), f = idx - t * (3 * THERMAL_CHUNK);
                const int j = f / 3, m = f - 3 * j;
                const long p = block_first + (long)t * R + k0 + j;
                if (k0 + j < R && p < n) {
                    float *a = vel + p * stride + m;
                    *a = addv(*a, stage[t][f]);
                }
            }
            __syncthreads();
        }
    }
    if (bad) atomicOr(err, 1);
}

// one species: n particles from state s0 advanced by `skip` draws; vel (device) n x stride floats.
// The grid is one wave of resident blocks (every thread a run of R particles, the same work), so no
// partial second wave idles most SMs.
static int thermal_launch(int prec, long n, const uint64_t s0[4], unsigned long long skip, const ThermTable &tt,
                          double a_ini, double M_eV, double c, float *vel, long stride, int *err) {
    if (n <= 0) return 0;
    const size_t smem = thermal_smem(tt.n);
    const bool packed = stride == 3 && ((uintptr_t)vel & 15) == 0;
    int dev = 0, sms = 0, per_sm = 0;
    MITOS_CUDA(cudaGetDevice(&dev));
    MITOS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto occupancy = [&](auto kern) -> int {
        if (smem > 48 * 1024) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        MITOS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THERMAL_THREADS, smem));
        return 0;
    };
    int e = prec == MITOS_FP32 ? (packed ? occupancy(k_thermal<float, true>) : occupancy(k_thermal<float, false>))
                               : (packed ? occupancy(k_thermal<double, true>) : occupancy(k_thermal<double, false>));
    if (e) return e;
    if (per_sm < 1) {
        set_error(3, "thermal sampler of %d pieces does not fit the kernel's shared memory", tt.n);
        return 3;
    }
    const long wave = (long)sms * per_sm * THERMAL_THREADS;
    int R = (int)((n + wave - 1) / wave);
    if (packed) R = (R + 3) & ~3;  // runs of whole float4 groups: 16-byte aligned starts
    const long G = (n + R - 1) / R;
    const uint64_t *polys = affine_jump_polys(skip, 7ULL * (unsigned long long)R, G);
    if (!polys) return 5;
    RngState st;
    memcpy(st.s, s0, sizeof st.s);
    const unsigned blocks = (unsigned)((G + THERMAL_THREADS - 1) / THERMAL_THREADS);
    const float vfac = (float)(c / (a_ini * M_eV));
    launch_begin("thermal");
    if (prec == MITOS_FP32) {
        if (packed)
            k_thermal<float, true><<<blocks, THERMAL_THREADS, smem, stream()>>>(n, R, st, polys, tt, a_ini, M_eV, c,
                                                                               vfac, vel, stride, err);
        else
            k_thermal<float, false><<<blocks, THERMAL_THREADS, smem, stream()>>>(n, R, st, polys, tt, a_ini, M_eV, c,
                                                                                vfac, vel, stride, err);
    } else {
        if (packed)
            k_thermal<double, true><<<blocks, THERMAL_THREADS, smem, stream()>>>(n, R, st, polys, tt, a_ini, M_eV, c,
                                                                                vfac, vel, stride, err);
        else
            k_thermal<double, false><<<blocks, THERMAL_THREADS, smem, stream()>>>(n, R, st, polys, tt, a_ini, M_eV, c,
                                                                                 vfac, vel, stride, err);
    }
    count_launch();
    MITOS_LAUNCH_CHECK("thermal velocities");
    return 0;
}

// sampler tables of the pipeline's species, per (kind, T): device copies kept until mitos_release_all
struct CachedTable {
    void *dev;
    int n;
};
static std::mutex g_tmu;
static std::map<std::pair<int, double>, CachedTable> g_tables;

static int sampler_build(struct sampler *s, int kind, double T_eV);

void release_thermal_tables() {
    std::lock_guard<std::mutex> lk(g_tmu);
    for (auto &kv : g_tables) cudaFree(kv.second.dev);
    g_tables.clear();
}

int thermal_add(int prec, long n, const uint64_t seed_state[4], unsigned long long skip, int kind, double T_eV,
                double M_eV, double a_ini, double c, float *dvel, long stride, int *derr) {
    CachedTable ct;
    {
        std::lock_guard<std::mutex> lk(g_tmu);
        auto it = g_tables.find({kind, T_eV});
        if (it == g_tables.end()) {
            struct sampler s;
            int e = sampler_build(&s, kind, T_eV);
            std::vector<unsigned char> img;
            int nn = 0;
            if (!e) e = table_image(&s, img, nn);
            free(s.intervals);
            free(s.index);
            if (e) return e;
            void *d = nullptr;
            if (cudaMalloc(&d, img.size()) != cudaSuccess) {
                cudaGetLastError();
                set_error(5, "out of device memory for a thermal sampler table");
                return 5;
            }
            MITOS_CUDA(cudaMemcpy(d, img.data(), img.size(), cudaMemcpyHostToDevice));
            it = g_tables.emplace(std::make_pair(kind, T_eV), CachedTable{d, nn}).first;
        }
        ct = it->second;
    }
    return thermal_launch(prec, n, seed_state, skip, table_view(ct.dev, ct.n), a_ini, M_eV, c, dvel, stride,
                          derr);
}

static int sampler_build(struct sampler *s, int kind, double T_eV) {
    memset(s, 0, sizeof *s);
    if ((kind != 1 && kind != 2) || !(T_eV > 0)) {
        set_error(1, "thermal sampler: kind 1 (fermion) or 2 (boson) and T_eV > 0");
        return 1;
    }
    // src/mitos.c:645-668: the domain [1e-10, 15] kT in eV, mu = 0
    PieceBuilder b;
    b.f = ThermalPdf{kind, T_eV, 0.0};
    b.xl = 1e-10 * T_eV;
    const double xr = 15.0 * T_eV;
    b.norm = 1.0;
    b.norm = 1.0 / b.integral(xr);
    b.by_mass(b.xl, xr, 0.0, 1.0, 0);
    if (b.overflow) {
        set_error(7, "thermal sampler: pieces did not converge");
        return 7;
    }
    const int n = (int)b.out.size();
    s->intervals = (struct interval *)malloc(sizeof(struct interval) * n);
    s->index = (double *)malloc(sizeof(double) * kTableLen);
    if (!s->intervals || !s->index) {
        free(s->intervals);
        free(s->index);
        memset(s, 0, sizeof *s);
        set_error(5, "thermal sampler: out of host memory");
        return 5;
    }
    for (int j = 0; j < n; j++) {
        s->intervals[j] = b.out[j];
        s->intervals[j].id = j;
        s->intervals[j].nid = j + 1 < n ? j + 1 : -1;
    }
    // search table: per u = i / 1000 the piece with the largest right end among those with Fr < u;
    // pieces are in order, so that is the last one with Fr < u (piece 0 when there is none)
    int last = 0;
    for (int i = 0; i < kTableLen; i++) {
        const double u = (double)i / kTableLen;
        while (last + 1 < n && s->intervals[last + 1].Fr < u) last++;
        s->index[i] = (s->intervals[last].Fr < u) ? last : 0;
    }
    s->norm = b.norm;
    s->xl = b.xl;
    s->xr = xr;
    s->f = nullptr;
    s->params = nullptr;
    s->intervalNum = n;
    s->I_max = kTableLen;
    return 0;
}

}  // namespace mitos

// ==== C ABI ===================================================================================
extern "C" int thermal_sampler_init(struct sampler *s, int kind, double T_eV) {
    if (!s) {
        mitos::set_error(1, "thermal_sampler_init: no sampler");
        return 1;
    }
    return mitos::sampler_build(s, kind, T_eV);
}

extern "C" int thermal_sampler_free(struct sampler *s) {
    if (!s) return 0;
    free(s->intervals);
    free(s->index);
    s->intervals = nullptr;
    s->index = nullptr;
    s->intervalNum = 0;
    return 0;
}

// the kernel's piece choice for n draws w, on the host from the same table image (no GPU): the
// threshold compares and bucket table the kernel reads
extern "C" int mitos_thermal_pieces(const struct sampler *s, const uint64_t *w, long n, int *piece) {
    using namespace mitos;
    std::vector<unsigned char> img;
    int nn = 0;
    const int e = table_image(s, img, nn);
    if (e) return e;
    const ThermPiece *pc = (const ThermPiece *)img.data();
    const unsigned short *bucket = (const unsigned short *)(img.data() + sizeof(ThermPiece) * nn);
    for (long i = 0; i < n; i++) {
        int pk = bucket[w[i] >> (64 - kBucketBits)];
        while (pk + 1 < nn && w[i] > pc[pk + 1].le) pk++;
        piece[i] = pk;
    }
    return 0;
}

extern "C" int thermal_velocities(const struct sampler *s, rng_state *state, long n, double M_eV, double a_ini,
                                  double speed_of_light, float *vel, long stride) {
    using namespace mitos;
    if (!state || !vel || n < 0 || stride < 3 || !(M_eV > 0) || !(a_ini > 0)) {
        set_error(1, "thermal_velocities: state, vel, n >= 0, stride >= 3, M_eV > 0 and a_ini > 0 needed");
        return 1;
    }
    if (n == 0) return 0;
    std::vector<unsigned char> img;
    int nn = 0;
    int e = table_image(s, img, nn);
    if (e) return e;
    void *dtab = workspace(img.size(), 150);
    int *derr = (int *)workspace(sizeof(int), 151);
    if (!dtab || !derr) return 5;
    MITOS_CUDA(cudaMemcpyAsync(dtab, img.data(), img.size(), cudaMemcpyHostToDevice, stream()));
    MITOS_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), stream()));
    const size_t vbytes = sizeof(float) * (size_t)((n - 1) * stride + 3);
    float *dvel = vel;
    cudaPointerAttributes at;
    const bool dev = cudaPointerGetAttributes(&at, vel) == cudaSuccess &&
                     (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
    if (!dev) {
        cudaGetLastError();
        dvel = (float *)workspace(vbytes, 152);
        if (!dvel) return 5;
        MITOS_CUDA(cudaMemcpyAsync(dvel, vel, vbytes, cudaMemcpyHostToDevice, stream()));
    }
    e = thermal_launch(mitos_get_precision(), n, state->s, 0, table_view(dtab, nn), a_ini, M_eV,
                       speed_of_light, dvel, stride, derr);
    if (e) return e;
    if (!dev) MITOS_CUDA(cudaMemcpyAsync(vel, dvel, vbytes, cudaMemcpyDeviceToHost, stream()));
    int herr = 0;
    MITOS_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    // the caller's stream continues after the species' 7 n draws, as the reference loop leaves it
    rng_jump(state->s, 7ULL * (unsigned long long)n);
    if (herr) {
        set_error(8, "thermal_velocities: invalid thermal momentum drawn");
        return 8;
    }
    return 0;
}
