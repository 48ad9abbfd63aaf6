// particles.cu -- lattice particles displaced by TSC-gathered displacement grids, then CIC mass
// assignment onto a grid.
//
// Follows src/particle.c:87-129 (float lattice positions), src/mitos.c:843-862 (one TSC gather
// per direction; the gather of direction d sees the displacements of directions < d already
// applied), src/mitos.c:1072-1077 (periodic wrap) and analyse/src/mitos_read.c:280-334 (CIC).
// The deposit is accumulated in units of the mean density: each particle adds (N/M)^3 split
// over its 8 cells, so the overdensity is the deposited value minus one.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "context.cuh"
#include "particles.cuh"
#include "tma.cuh"

namespace mitos {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

bool encode_grid_map(CUtensorMap *m, const void *base, bool f64, long n2, long n1, long pitch, unsigned b0,
                     unsigned b1, unsigned b2) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
    if (!fn) return false;
    const cuuint64_t es = f64 ? 8 : 4;
    const cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[2] = {(cuuint64_t)pitch * es, (cuuint64_t)(pitch * n1) * es};
    const cuuint32_t box[3] = {b0, b1, b2};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims,
              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// set by a deposit kernel whose tile copies did not complete (it then stops; see lattice_fault)
__device__ int g_lattice_fault;

template <typename T> __device__ __forceinline__ T dfloor(T x);
template <> __device__ __forceinline__ float dfloor<float>(float x) { return floorf(x); }
template <> __device__ __forceinline__ double dfloor<double>(double x) { return floor(x); }
template <typename T> __device__ __forceinline__ int ifloor(T x);
template <> __device__ __forceinline__ int ifloor<float>(float x) { return __float2int_rd(x); }
template <> __device__ __forceinline__ int ifloor<double>(double x) { return __double2int_rd(x); }

// floor of x as an int and as a real.  FP32: one round-down add of 1.5 * 2^23 (the sum's unit bit
// is floor(x)'s for |x| < 2^22; the lattice path's grid coordinates stay far inside that), which
// replaces a float -> int and an int -> float conversion (quarter-rate or slower) by full-rate
// adds; identical results to __float2int_rd and its cast back.
template <typename T> __device__ __forceinline__ int floor_split(T x, T &f);
template <> __device__ __forceinline__ int floor_split<float>(float x, float &f) {
    const float m = __fadd_rd(x, 12582912.f);
    f = m - 12582912.f;
    return __float_as_int(m) - 0x4B400000;
}
template <> __device__ __forceinline__ int floor_split<double>(double x, double &f) {
    const int i = __double2int_rd(x);
    f = (double)i;
    return i;
}
// (float)i for 0 <= i < 2^23, without a conversion
__device__ __forceinline__ float small_int_to_float(int i) { return __int_as_float(0x4B000000 + i) - 8388608.f; }

// CIC region accumulators: 32-bit fixed point with 2^23 per mean density in FP32 (native
// integer shared atomics; exact, order independent), doubles in FP64
template <typename T> struct RegAcc;
template <> struct RegAcc<float> {
    using type = unsigned int;
    // w in [0, 1]: round-to-nearest-even of w 2^23 as the low bits of w 2^23 + 2^23 (one FMA; the
    // same integer as __float2uint_rn(w * 2^23), without the conversion)
    static __device__ __forceinline__ void add(unsigned int *c, float w) {
        atomicAdd(c, __float_as_uint(fmaf(w, 8388608.f, 8388608.f)) - 0x4B000000u);
    }
    static __device__ __forceinline__ float value(unsigned int c) { return (float)c * (1.f / 8388608.f); }
};
template <> struct RegAcc<double> {
    using type = double;
    static __device__ __forceinline__ void add(double *c, double w) { atomicAdd(c, w); }
    static __device__ __forceinline__ double value(double c) { return c; }
};

__device__ __forceinline__ int wrapi(int i, int N) {
    i %= N;
    return i < 0 ? i + N : i;
}

// periodic index for the small offsets of the interpolation stencils, with the general
// modulo kept for anything further out (non-finite positions included)
__device__ __forceinline__ int wrapn(int i, int N) {
    i += (i < 0) ? N : 0;
    i -= (i >= N) ? N : 0;
    if ((unsigned)i >= (unsigned)N) i = wrapi(i, N);
    return i;
}

// TSC interpolation at grid coordinates (Xg, Yg, Zg) of a padded real grid:
// src/grids_interp.c:267-309 written over the three nearest nodes of each axis
template <typename T>
__device__ __forceinline__ T tsc_gather(const T *__restrict__ box, int N, T Xg, T Yg, T Zg) {
    const T half = (T)0.5;
    const int nx = (int)dfloor<T>(Xg + half), ny = (int)dfloor<T>(Yg + half), nz = (int)dfloor<T>(Zg + half);
    const T dx = Xg - (T)nx, dy = Yg - (T)ny, dz = Zg - (T)nz;
    T wx[3], wy[3], wz[3];
    wx[0] = half * (half - dx) * (half - dx); wx[1] = (T)0.75 - dx * dx; wx[2] = half * (half + dx) * (half + dx);
    wy[0] = half * (half - dy) * (half - dy); wy[1] = (T)0.75 - dy * dy; wy[2] = half * (half + dy) * (half + dy);
    wz[0] = half * (half - dz) * (half - dz); wz[1] = (T)0.75 - dz * dz; wz[2] = half * (half + dz) * (half + dz);
    int zi[3], yi[3], xi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        zi[k] = wrapn(nz - 1 + k, N);
        yi[k] = wrapn(ny - 1 + k, N);
        xi[k] = wrapn(nx - 1 + k, N);
    }
    const long rp = N + 2;
    T sum = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const long xo = (long)xi[i] * N;
        T sy = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const T *row = box + (xo + yi[j]) * rp;
            const T sz = wz[0] * __ldg(row + zi[0]) + wz[1] * __ldg(row + zi[1]) + wz[2] * __ldg(row + zi[2]);
            sy += wy[j] * sz;
        }
        sum += wx[i] * sy;
    }
    return sum;
}

// fwrap of a float position (double fmod in the reference; exact for |x| < 2L with L a float)
__device__ __forceinline__ float fwrapf(float x, float L) {
    if (x < 0.f) x += L;
    if (x >= L) x -= L;
    return x;
}

template <typename T> __device__ __forceinline__ T fwrapT(T x, T L);
template <> __device__ __forceinline__ float fwrapT<float>(float x, float L) { return fmodf(fmodf(x, L) + L, L); }
template <> __device__ __forceinline__ double fwrapT<double>(double x, double L) { return fmod(fmod(x, L) + L, L); }

// Grid coordinate x N / L of a position.  FP32: N / L as the unevaluated sum g + g_lo of two floats
// and one FMA, so the coordinate is the exactly scaled position rounded once.  A rounded N / L (or
// L / N) alone scales every coordinate by its relative rounding error (up to 6e-8): the particle
// distribution stretched against the periodic grid, which moved the power of the box-scale modes
// along the axes by up to 4e-4 (1024^3 and 256^3, L = 2000 Mpc/h).  FP64: the product (g_lo = 0).
template <typename T> __device__ __forceinline__ T grid_coord(T p, T g, T g_lo) {
    if constexpr (sizeof(T) == 4) return fmaf(p, g, p * g_lo);
    else return p * g;
}
// host: N / L split for grid_coord (g_lo = 0 in FP64)
template <typename T> static void grid_scale(int N, double boxlen, T &g, T &g_lo) {
    const double s = N / boxlen;
    g = (T)s;
    g_lo = sizeof(T) == 4 ? (T)(s - (double)g) : (T)0;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_displace_cic(int N, int M, float spacing, T boxlen, T gfac, T g, T g_lo, T val,
               const T *__restrict__ d0, const T *__restrict__ d1, const T *__restrict__ d2,
               T *__restrict__ rho, float *__restrict__ pos_out, float *__restrict__ posraw_out) {
    const long np = (long)M * M * M;
    const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    const int z = (int)(id % M);
    const long xy = id / M;
    const int y = (int)(xy % M), x = (int)(xy / M);
    float p[3] = {x * spacing, y * spacing, z * spacing};  // src/particle.c:114-116
    const T *dd[3] = {d0, d1, d2};
    const T Nf = (T)N;
#pragma unroll
    for (int dir = 0; dir < 3; dir++) {
        // X = x N / boxlen (src/grids_interp.c:269-271); FP32 through grid_coord
        T disp;
        if constexpr (sizeof(T) == 4)
            disp = tsc_gather<T>(dd[dir], N, grid_coord<T>(p[0], g, g_lo), grid_coord<T>(p[1], g, g_lo),
                                 grid_coord<T>(p[2], g, g_lo));
        else
            disp = tsc_gather<T>(dd[dir], N, (T)p[0] * Nf / boxlen, (T)p[1] * Nf / boxlen, (T)p[2] * Nf / boxlen);
        p[dir] = (float)((T)p[dir] - disp);
    }
    if (posraw_out) {  // before the wrap: the velocity gather's positions (src/mitos.c:865-908)
        posraw_out[3 * id] = p[0];
        posraw_out[3 * id + 1] = p[1];
        posraw_out[3 * id + 2] = p[2];
    }
    const float Lf = (float)boxlen;
#pragma unroll
    for (int c = 0; c < 3; c++) p[c] = fwrapf(p[c], Lf);
    if (pos_out) {
        pos_out[3 * id] = p[0];
        pos_out[3 * id + 1] = p[1];
        pos_out[3 * id + 2] = p[2];
    }
    // CIC: X = x / (L / N) (analyse/src/mitos_read.c:288-333); FP32 through grid_coord
    T X, Y, Z;
    if constexpr (sizeof(T) == 4) {
        X = grid_coord<T>(p[0], g, g_lo);
        Y = grid_coord<T>(p[1], g, g_lo);
        Z = grid_coord<T>(p[2], g, g_lo);
    } else {
        X = (T)p[0] / gfac;
        Y = (T)p[1] / gfac;
        Z = (T)p[2] / gfac;
    }
    const int iX = (int)dfloor<T>(X), iY = (int)dfloor<T>(Y), iZ = (int)dfloor<T>(Z);
    const T dx = X - iX, dy = Y - iY, dz = Z - iZ;
    const T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
    const long rp = N + 2;
    const int x0 = wrapn(iX, N), x1 = wrapn(iX + 1, N);
    const int y0 = wrapn(iY, N), y1 = wrapn(iY + 1, N);
    const int z0 = wrapn(iZ, N), z1 = wrapn(iZ + 1, N);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z0, val * tx * ty * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z0, val * dx * ty * tz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z0, val * tx * dy * tz);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z1, val * tx * ty * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z0, val * dx * dy * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z1, val * dx * ty * dz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z1, val * tx * dy * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z1, val * dx * dy * dz);
}

// ---- lattice-aligned fast path ------------------------------------------------------------
// When M = N and every lattice coordinate i * spacing maps exactly onto grid node i, the TSC
// gather of direction 0 sits on nodes in x, y, z; direction 1 on nodes in y, z; direction 2 on
// nodes in z.  The displacement passes fold the stencil of those axes into the grids (exact in
// exact arithmetic), so the gathers read 1, 3 and 9 values.  The CIC deposit of a brick of
// particles accumulates in shared memory (one halo cell each side) and is flushed with
// atomics; deposits that land outside the brick's region go straight to global memory.
#define LB_X 8
#define LB_Y 8
#define LB_Z 32
#define LB_THREADS 512
#define LR_X (LB_X + 2)
#define LR_Y (LB_Y + 2)
#define LR_Z (LB_Z + 8)   // z halo of 4 each side keeps the flushed rows 16-byte aligned
#define LR_Z0 4           // region z index of the brick's first cell

template <typename T>
__device__ __forceinline__ void tsc_w(T d, T *w) {
    const T half = (T)0.5;
    w[0] = half * (half - d) * (half - d);
    w[1] = (T)0.75 - d * d;
    w[2] = half * (half + d) * (half + d);
}

// deposit of one particle outside its brick's shared region (rare): straight to global memory
template <typename T>
__device__ __noinline__ void cic_global(T *rho, int N, int rp, int iX, int iY, int iZ, T dx, T dy, T dz) {
    const T wx[2] = {1 - dx, dx}, wy[2] = {1 - dy, dy}, wz[2] = {1 - dz, dz};
#pragma unroll 1
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
            for (int c = 0; c < 2; c++)
                atomicAdd(rho + ((long)wrapn(iX + a, N) * N + wrapn(iY + b, N)) * rp + wrapn(iZ + c, N),
                          wx[a] * wy[b] * wz[c]);
}

// red.global.add.v4.f32: four consecutive floats in one reduction (sm_90 and later)
__device__ __forceinline__ void red_add_v4(float *p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// gather of the three displacement grids from global memory for a particle that moved too far
// for the brick's shared tiles (rare); same arithmetic as the tiled path.  rpd: row pitch of
// the displacement grids.
template <typename T>
__device__ __noinline__ void displace_global(int N, int rpd, T ginv, const T *d1, const T *d2, int y, int z,
                                             float &p0, float &p1, float &p2) {
    const long yz = (long)y * rpd + z;
    const T Xg = (T)p0 * ginv;
    const int nx = ifloor<T>(Xg + (T)0.5);
    T wx[3];
    tsc_w<T>(Xg - (T)nx, wx);
    long xo[3];
    for (int i = 0; i < 3; i++) xo[i] = (long)wrapn(nx - 1 + i, N) * N * rpd;
    p1 = (float)((T)p1 - (wx[0] * d1[xo[0] + yz] + wx[1] * d1[xo[1] + yz] + wx[2] * d1[xo[2] + yz]));
    const T Yg = (T)p1 * ginv;
    const int ny = ifloor<T>(Yg + (T)0.5);
    T wy[3];
    tsc_w<T>(Yg - (T)ny, wy);
    T sv = 0;
    for (int j = 0; j < 3; j++) {
        const long yo = (long)wrapn(ny - 1 + j, N) * rpd + z;
        sv += wy[j] * (wx[0] * d2[xo[0] + yo] + wx[1] * d2[xo[1] + yo] + wx[2] * d2[xo[2] + yo]);
    }
    p2 = (float)((T)p2 - sv);
}

// unsigned division n / d for n < 2^31 by a multiply-high and a shift (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994): m = floor(2^32 (2^s - d) / d) + 1
// with s = ceil(log2 d), q = (umulhi(n, m) + n) >> s.  The brick decode of the persistent deposit
// ran three runtime divisions per brick.
struct FastDiv {
    unsigned m;
    int s;
};
static FastDiv make_fastdiv(unsigned d) {
    FastDiv f;
    f.s = 0;
    while ((1u << f.s) < d) f.s++;
    f.m = (unsigned)(((1ULL << 32) * ((1ULL << f.s) - d)) / d + 1);
    return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned n, FastDiv f) { return (__umulhi(n, f.m) + n) >> f.s; }

// tiles of the brick: d0 on the brick, d1 with an x halo of TH, d2 with x and y halos of TH.  A
// particle displaced by under half a cell in x (and y) gathers inside them; one displaced farther
// (a few in 10^5 at z = 31 with 2 Mpc/h cells) takes the global-memory gather.  (A halo of 2:
// 1.263 ms at 512^3; 1: 1.219 ms.  d0 read from global memory instead of staged: 1.439 ms, the
// load at the head of each particle's chain exposed.)
#define TH 1
#define T1X (LB_X + 2 * TH)
#define T2Y (LB_Y + 2 * TH)
#define TILE_ELEMS (LB_X * LB_Y * LB_Z + T1X * LB_Y * LB_Z + T1X * T2Y * LB_Z)

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// stage the three displacement tiles of brick (x0, y0, z0) into shared memory: rows of LB_Z
// elements in 16-byte pieces (row pitch rpd * sizeof(T) and z0 are multiples of 16 bytes)
template <typename T>
__device__ __forceinline__ void stage_tiles(T *tiles, int N, int rpd, int x0, int y0, int z0, const T *__restrict__ d0,
                                            const T *__restrict__ d1, const T *__restrict__ d2) {
    constexpr int CH = 16 / sizeof(T);
    constexpr int RC = LB_Z / CH;
    constexpr int C0 = LB_X * LB_Y * RC, C1 = T1X * LB_Y * RC, C2 = T1X * T2Y * RC;
#pragma unroll
    for (int c = threadIdx.x; c < C0 + C1 + C2; c += LB_THREADS) {
        const T *src;
        if (c < C0) {
            const int r = c / RC, lx = r / LB_Y, ly = r % LB_Y;
            src = d0 + ((long)(x0 + lx) * N + y0 + ly) * rpd;
        } else if (c < C0 + C1) {
            const int r = (c - C0) / RC, lx = r / LB_Y, ly = r % LB_Y;
            src = d1 + ((long)wrapn(x0 - TH + lx, N) * N + y0 + ly) * rpd;
        } else {
            const int r = (c - C0 - C1) / RC, lx = r / T2Y, ly = r % T2Y;
            src = d2 + ((long)wrapn(x0 - TH + lx, N) * N + wrapn(y0 - TH + ly, N)) * rpd;
        }
        // the three tiles are contiguous in shared memory, each a sequence of LB_Z-element rows
        cp_async16(tiles + (long)c * CH, src + z0 + (c % RC) * CH);
    }
}

// tensor maps of the three displacement grids, boxes of the brick tiles: d0 {LB_Z, LB_Y, LB_X}, d1
// {LB_Z, LB_Y, T1X}, d2 {LB_Z, T2Y, T1X} (z innermost)
struct LatticeMaps {
    CUtensorMap m0, m1, m2;
};

// Persistent: each block walks bricks b = blockIdx.x, blockIdx.x + gridDim.x, ..., staging the
// next brick's tiles (second buffer) while it displaces and deposits the current one.  Bricks whose
// halos stay inside the box (not on an x or y face) are staged by three tensor copies issued by one
// thread, completing on the buffer's mbarrier; face bricks, whose halos wrap, by 16-byte cp.async.
template <typename T>
__global__ void __launch_bounds__(LB_THREADS, 2)
k_lattice_cic(int N, int rpd, int rpo, float spacing, float Lf, T ginv, T ginv_lo, const T *__restrict__ d0, const T *__restrict__ d1,
              const T *__restrict__ d2, T *__restrict__ rho, float *__restrict__ pos_out, size_t bstride, FastDiv div_bx,
              FastDiv div_by, float *__restrict__ posraw_out, const __grid_constant__ LatticeMaps maps, int use_tma,
              int region) {
    // batched launches: realisation blockIdx.y (its grids bstride bytes apart)
    if (gridDim.y > 1) {
        const size_t bo = (size_t)blockIdx.y * bstride;
        d0 = bat<const T>(d0, bo);
        d1 = bat<const T>(d1, bo);
        d2 = bat<const T>(d2, bo);
        rho = bat<T>(rho, bo);
    }
    using A = typename RegAcc<T>::type;
    extern __shared__ __align__(16) unsigned char smraw[];
    A *reg = reinterpret_cast<A *>(smraw);                                      // LR_X * LR_Y * LR_Z
    T *tbuf = reinterpret_cast<T *>(smraw + sizeof(A) * LR_X * LR_Y * LR_Z);    // 2 x TILE_ELEMS
    // brick order: x fastest, then y, then z, so the x and y neighbours whose planes the tile halos
    // read are in flight at the same time (their halo rows come from L2, not DRAM)
    const int bx_n = N / LB_X, by_n = N / LB_Y;
    const int nbricks = bx_n * by_n * (N / LB_Z);
    for (int i = threadIdx.x; i < LR_X * LR_Y * LR_Z; i += LB_THREADS) reg[i] = 0;
    // brick b -> (bx, by, bz), x fastest
    auto decode = [&](int b, int &bx, int &by, int &bz) {
        if (region) {
            // regions of 8 x 8 x 4 bricks (64 x 64 x 128 cells), x fastest inside a region and
            // across regions: the bricks in flight (about one region) share their halo rows and
            // flushed sectors in every direction while those are still in L2
            const int w = b & 255, r = b >> 8;
            const int rq = (int)fdiv((unsigned)r, div_bx);  // div_bx: regions along x
            const int rx = r - rq * (bx_n >> 3);
            const int rz = (int)fdiv((unsigned)rq, div_by);  // div_by: regions along y
            const int ry = rq - rz * (by_n >> 3);
            bx = (rx << 3) + (w & 7);
            by = (ry << 3) + ((w >> 3) & 7);
            bz = (rz << 2) + (w >> 6);
            return;
        }
        const int q = (int)fdiv((unsigned)b, div_bx);
        bx = b - q * bx_n;
        bz = (int)fdiv((unsigned)q, div_by);
        by = q - bz * by_n;
    };
    // tensor-copy staging: two mbarriers behind the tile buffers, one per buffer; bit b of `phase`
    // is the parity of buffer b's next completion (uniform in the block, as the brick sequence is)
    uint64_t *bars = reinterpret_cast<uint64_t *>(tbuf + 2 * TILE_ELEMS);
    const bool tma = use_tma && gridDim.y == 1 && (smem_u32(tbuf) & 127) == 0;
    if (tma && threadIdx.x == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        mbar_init_fence();
    }
    __syncthreads();
    unsigned phase = 0;
    auto by_tma = [&](int bx, int by) { return tma && bx > 0 && bx < bx_n - 1 && by > 0 && by < by_n - 1; };
    auto stage = [&](int bx, int by, int bz, int bi) {
        T *dst = tbuf + bi * TILE_ELEMS;
        const int x0 = bx * LB_X, y0 = by * LB_Y, z0 = bz * LB_Z;
        if (by_tma(bx, by)) {
            if (threadIdx.x == 0) {
                fence_proxy_async();
                mbar_expect_tx(bars + bi, (unsigned)(TILE_ELEMS * sizeof(T)));
                tma_load_3d(dst, &maps.m0, z0, y0, x0, bars + bi);
                tma_load_3d(dst + LB_X * LB_Y * LB_Z, &maps.m1, z0, y0, x0 - TH, bars + bi);
                tma_load_3d(dst + LB_X * LB_Y * LB_Z + T1X * LB_Y * LB_Z, &maps.m2, z0, y0 - TH, x0 - TH, bars + bi);
            }
        } else {
            stage_tiles<T>(dst, N, rpd, x0, y0, z0, d0, d1, d2);
        }
    };
    int b = blockIdx.x;
    if (b < nbricks) {
        int bx, by, bz;
        decode(b, bx, by, bz);
        stage(bx, by, bz, 0);
    }
    cp_async_commit();
    const int lz = threadIdx.x % LB_Z, ly = (threadIdx.x / LB_Z) % LB_Y, lxb = threadIdx.x / (LB_Z * LB_Y);
#pragma unroll 1
    for (int buf = 0; b < nbricks; b += gridDim.x, buf ^= 1) {
        int bx, by, bz;
        decode(b, bx, by, bz);
        const int x0 = bx * LB_X, y0 = by * LB_Y, z0 = bz * LB_Z;
        const int bn = b + gridDim.x;
        bool next_tma = false;
        if (bn < nbricks) {
            int nx, ny, nz;
            decode(bn, nx, ny, nz);
            stage(nx, ny, nz, buf ^ 1);
            next_tma = by_tma(nx, ny);
        }
        cp_async_commit();
        cp_async_wait_prev();
        bool ok = true;
        if (by_tma(bx, by)) {
            ok = mbar_wait(bars + buf, (phase >> buf) & 1u);
            phase ^= 1u << buf;
        }
        // this brick's tiles have landed; the accumulators are zero
        if (__syncthreads_or(!ok)) {
            // a tensor copy that never completed: flag it, let the next brick's copy finish (bounded)
            // and stop
            if (threadIdx.x == 0) atomicExch(&g_lattice_fault, 1);
            if (by_tma(bx, by)) mbar_wait(bars + buf, ((phase >> buf) & 1u) ^ 1u);  // once more, bounded
            if (next_tma) mbar_wait(bars + (buf ^ 1), (phase >> (buf ^ 1)) & 1u);
            cp_async_wait_all();
            return;
        }
        const T *t0 = tbuf + buf * TILE_ELEMS;
        const T *t1 = t0 + LB_X * LB_Y * LB_Z;
        const T *t2 = t1 + T1X * LB_Y * LB_Z;
#pragma unroll 1
        for (int rep = 0; rep < (LB_X * LB_Y * LB_Z) / LB_THREADS; rep++) {
            const int lx = lxb + rep * (LB_THREADS / (LB_Z * LB_Y));
            const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
            // src/particle.c:114-116
            float p0 = small_int_to_float(x) * spacing, p1 = small_int_to_float(y) * spacing,
                  p2 = small_int_to_float(z) * spacing;
            // direction 0: on nodes (stencil folded into d0)
            p0 = (float)((T)p0 - t0[(lx * LB_Y + ly) * LB_Z + lz]);
            // direction 1: x off node (src/grids_interp.c:269-306), y and z on nodes (folded into d1).
            // (The stencil coordinates take the plain product: N / L's rounding shifts where the
            // displacement is read by at most 6e-8 of the coordinate, far below a position's ulp.)
            const T Xg = (T)p0 * ginv;
            T fnx;
            const int nx = floor_split<T>(Xg + (T)0.5, fnx);
            const int ix = nx - 1 - (x0 - TH);  // tile x index of the first stencil node
            bool tiled = ix >= 0 && ix + 2 < T1X;
            T wx[3], wy[3];
            if (tiled) {
                tsc_w<T>(Xg - fnx, wx);
                const T *r1 = t1 + (ix * LB_Y + ly) * LB_Z + lz;
                p1 = (float)((T)p1 - (wx[0] * r1[0] + wx[1] * r1[LB_Y * LB_Z] + wx[2] * r1[2 * LB_Y * LB_Z]));
                // direction 2: x and y off nodes, z on nodes (folded into d2)
                const T Yg = (T)p1 * ginv;
                T fny;
                const int ny = floor_split<T>(Yg + (T)0.5, fny);
                const int iy = ny - 1 - (y0 - TH);
                tiled = iy >= 0 && iy + 2 < T2Y;
                if (tiled) {
                    tsc_w<T>(Yg - fny, wy);
                    T sv = 0;
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        const T *r2 = t2 + ((ix + i) * T2Y + iy) * LB_Z + lz;
                        sv += wx[i] * (wy[0] * r2[0] + wy[1] * r2[LB_Z] + wy[2] * r2[2 * LB_Z]);
                    }
                    p2 = (float)((T)p2 - sv);
                }
            }
            if (!tiled) {
                // restart the off-node gathers from global memory
                p1 = y * spacing;
                p2 = z * spacing;
                displace_global<T>(N, rpd, ginv, d1, d2, y, z, p0, p1, p2);
            }
            if (posraw_out) {  // before the wrap: the velocity gather's positions
                const long id = ((long)x * N + y) * N + z;
                posraw_out[3 * id] = p0;
                posraw_out[3 * id + 1] = p1;
                posraw_out[3 * id + 2] = p2;
            }
            p0 = fwrapf(p0, Lf);
            p1 = fwrapf(p1, Lf);
            p2 = fwrapf(p2, Lf);
            if (pos_out) {
                const long id = ((long)x * N + y) * N + z;
                pos_out[3 * id] = p0;
                pos_out[3 * id + 1] = p1;
                pos_out[3 * id + 2] = p2;
            }
            // CIC (analyse/src/mitos_read.c:288-333), one unit of mean density per particle (M = N)
            const T X = grid_coord<T>((T)p0, ginv, ginv_lo), Y = grid_coord<T>((T)p1, ginv, ginv_lo),
                    Z = grid_coord<T>((T)p2, ginv, ginv_lo);
            T fX, fY, fZ;
            const int iX = floor_split<T>(X, fX), iY = floor_split<T>(Y, fY), iZ = floor_split<T>(Z, fZ);
            const T dx = X - fX, dy = Y - fY, dz = Z - fZ;
            // region indices; the periodic wrap only for the bricks on the box faces
            int rx = iX - x0 + 1, ry = iY - y0 + 1, rz = iZ - z0 + LR_Z0;
            if ((unsigned)rx >= (unsigned)N) rx = wrapn(rx, N);
            if ((unsigned)ry >= (unsigned)N) ry = wrapn(ry, N);
            if ((unsigned)rz >= (unsigned)N) rz = wrapn(rz, N);
            if (rx < LR_X - 1 && ry < LR_Y - 1 && rz < LR_Z - 1) {
                A *c = reg + (rx * LR_Y + ry) * LR_Z + rz;
                const T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
                RegAcc<T>::add(c, tx * ty * tz);
                RegAcc<T>::add(c + 1, tx * ty * dz);
                RegAcc<T>::add(c + LR_Z, tx * dy * tz);
                RegAcc<T>::add(c + LR_Z + 1, tx * dy * dz);
                RegAcc<T>::add(c + LR_Y * LR_Z, dx * ty * tz);
                RegAcc<T>::add(c + LR_Y * LR_Z + 1, dx * ty * dz);
                RegAcc<T>::add(c + LR_Y * LR_Z + LR_Z, dx * dy * tz);
                RegAcc<T>::add(c + LR_Y * LR_Z + LR_Z + 1, dx * dy * dz);
            } else {
                cic_global<T>(rho, N, rpo, iX, iY, iZ, dx, dy, dz);
            }
        }
        __syncthreads();
        // flush and re-zero: rows of LR_Z cells starting at z0 - 4 (a multiple of 4, so 16-byte
        // aligned with the 16-byte aligned row pitch rpo)
        constexpr int Q = LR_Z / 4;
        for (int i = threadIdx.x; i < LR_X * LR_Y * Q; i += LB_THREADS) {
            const int qz = i % Q, qy = (i / Q) % LR_Y, qx = i / (Q * LR_Y);
            A *c = reg + (qx * LR_Y + qy) * LR_Z + 4 * qz;
            const A c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
            if (c0 == (A)0 && c1 == (A)0 && c2 == (A)0 && c3 == (A)0) continue;
            c[0] = 0; c[1] = 0; c[2] = 0; c[3] = 0;
            const T v[4] = {RegAcc<T>::value(c0), RegAcc<T>::value(c1), RegAcc<T>::value(c2), RegAcc<T>::value(c3)};
            const long row = ((long)wrapn(x0 - 1 + qx, N) * N + wrapn(y0 - 1 + qy, N)) * rpo;
            const int gz = z0 - LR_Z0 + 4 * qz;
            if constexpr (sizeof(T) == 4) {
                if (gz >= 0 && gz + 3 < N) {
                    red_add_v4((float *)rho + row + gz, (float)v[0], (float)v[1], (float)v[2], (float)v[3]);
                    continue;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (v[k] != (T)0) atomicAdd(rho + row + wrapn(gz + k, N), v[k]);
        }
        // the zeroed accumulators and the free tile buffer are published by the barrier at the
        // top of the next brick
    }
    cp_async_wait_all();
}

static size_t lattice_smem(size_t elem) {
    // the region accumulators have the size of one element in either precision; two mbarriers
    return elem * ((size_t)LR_X * LR_Y * LR_Z + 2 * (size_t)TILE_ELEMS) + 2 * sizeof(uint64_t);
}

// the fault flag reaches the host through a pinned word, copied behind the deposit on the library
// stream and read once the caller has synchronised it
static int *g_fault_host = nullptr;
int lattice_fault_fetch() {
    if (!g_fault_host) {
        MITOS_CUDA(cudaHostAlloc((void **)&g_fault_host, sizeof(int), cudaHostAllocDefault));
        *g_fault_host = 0;
    }
    MITOS_CUDA(cudaMemcpyFromSymbolAsync(g_fault_host, g_lattice_fault, sizeof(int), 0, cudaMemcpyDeviceToHost, stream()));
    return 0;
}
int lattice_fault_check() {
    // the Z passes' row copies too (their word is written by the kernels themselves)
    if (const int z = zrow_fault_check()) return z;
    if (!g_fault_host || !*g_fault_host) return 0;
    *g_fault_host = 0;
    const int zero = 0;
    MITOS_CUDA(cudaMemcpyToSymbolAsync(g_lattice_fault, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    set_error(6, "a displacement tile copy of the deposit did not complete (bounded wait timed out)");
    return 6;
}

// brick order by 8 x 8 x 4 regions (on by default where the bricks tile into them)
static bool g_lattice_region = true;
void set_lattice_region(bool on) { g_lattice_region = on; }
bool lattice_region() { return g_lattice_region; }

// tensor-copy staging of the interior bricks (on by default; off: 16-byte cp.async for all)
static bool g_lattice_tma = true;
void set_lattice_tma(bool on) { g_lattice_tma = on; }
bool lattice_tma() { return g_lattice_tma; }

template <typename T>
static int lattice_launch(int N, int rpd, int rpo, float spacing, float Lf, double boxlen, const void *d0, const void *d1,
                          const void *d2, void *rho, float *pos_out, int batch, size_t bstride, float *posraw_out) {
    static int blocks_per_sm[2] = {0, 0};  // per precision, for the current device
    static int sms = 0;
    const size_t smem = lattice_smem(sizeof(T));
    auto kern = k_lattice_cic<T>;
    int &bps = blocks_per_sm[sizeof(T) == 4];
    if (!bps) {
        MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int dev = 0;
        MITOS_CUDA(cudaGetDevice(&dev));
        MITOS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        MITOS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, LB_THREADS, smem));
        if (bps < 1) bps = 1;
    }
    const long nbricks = (long)(N / LB_X) * (N / LB_Y) * (N / LB_Z);
    const int nb = batch > 1 ? batch : 1;
    const unsigned blocks = (unsigned)std::max<long>(1, std::min<long>(nbricks, (long)sms * bps / nb));
    // tensor maps of the three grids (one realisation: batched launches stage with cp.async)
    LatticeMaps maps;
    memset(&maps, 0, sizeof maps);
    const bool f64 = sizeof(T) == 8;
    int use_tma = g_lattice_tma && nb == 1 &&
                  encode_grid_map(&maps.m0, d0, f64, N, N, rpd, LB_Z, LB_Y, LB_X) &&
                  encode_grid_map(&maps.m1, d1, f64, N, N, rpd, LB_Z, LB_Y, T1X) &&
                  encode_grid_map(&maps.m2, d2, f64, N, N, rpd, LB_Z, T2Y, T1X);
    // brick order: regions of 8 x 8 x 4 bricks where they tile the grid, else x, y, z rows
    const int bxn = N / LB_X, byn = N / LB_Y, bzn = N / LB_Z;
    const int region = g_lattice_region && bxn % 8 == 0 && byn % 8 == 0 && bzn % 4 == 0;
    const FastDiv dx = make_fastdiv((unsigned)(region ? bxn / 8 : bxn)), dy = make_fastdiv((unsigned)(region ? byn / 8 : byn));
    T g, g_lo;
    grid_scale<T>(N, boxlen, g, g_lo);
    kern<<<dim3(blocks, nb), LB_THREADS, smem, stream()>>>(N, rpd, rpo, spacing, Lf, g, g_lo, (const T *)d0,
                                                           (const T *)d1, (const T *)d2, (T *)rho, pos_out, bstride,
                                                           dx, dy, posraw_out, maps, use_tma, region);
    return 0;
}

int lattice_deposit(int N, double boxlen, int precision, const void *d0, const void *d1, const void *d2,
                    int disp_pitch, void *rho, int rho_pitch, float *pos_out, int batch, size_t bstride,
                    float *posraw_out) {
    const size_t es = precision == MITOS_FP32 ? 4 : 8;
    if (N % LB_Z || N % LB_Y || N % LB_X || (rho_pitch * es) % 16 || (disp_pitch * es) % 16 ||
        ((uintptr_t)d0 | (uintptr_t)d1 | (uintptr_t)d2 | (uintptr_t)rho) % 16)
        return 3;
    const float Lf = (float)boxlen;
    const float spacing = Lf / N;  // src/particle.c:102-103 with M = N
    launch_begin("lattice_cic");
    const int e = precision == MITOS_FP32
                      ? lattice_launch<float>(N, disp_pitch, rho_pitch, spacing, Lf, boxlen, d0, d1, d2, rho, pos_out,
                                              batch, bstride, posraw_out)
                      : lattice_launch<double>(N, disp_pitch, rho_pitch, spacing, Lf, boxlen, d0, d1, d2, rho, pos_out,
                                               batch, bstride, posraw_out);
    if (e) return e;
    count_launch();
    MITOS_LAUNCH_CHECK("lattice CIC");
    return 0;
}

// whether lattice coordinate i * spacing lands exactly on grid node i for every i, in the
// arithmetic of both the reference (double, x N / boxlen) and the FP32 path
bool lattice_aligned(int N, int M, double boxlen) {
    if (M != N || N % LB_Z || N % LB_Y || N % LB_X) return false;
    const float Lf = (float)boxlen;
    const float spacing = Lf / M;
    float g, g_lo;
    grid_scale<float>(N, boxlen, g, g_lo);
    for (int i = 0; i < M; i++) {
        const float x = i * spacing;
        if ((double)x * N / boxlen != (double)i) return false;
        if ((float)x * (float)N / Lf != (float)i) return false;
        if (fmaf(x, g, x * g_lo) != (float)i) return false;  // grid_coord of the FP32 kernels
        if ((double)x / (boxlen / N) != (double)i) return false;
    }
    return true;
}

// CIC of given positions (cic_deposit_dg)
template <typename T>
__global__ void k_cic(long n, int N, T L, T gfac, T g, T g_lo, T val, const float *__restrict__ pos, T *__restrict__ rho) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // x = fwrap(x, L) in the working precision, X = x / (L / N) (analyse/src/mitos_read.c:284-290);
    // FP32 through grid_coord
    const T px = fwrapT<T>((T)pos[3 * i], L), py = fwrapT<T>((T)pos[3 * i + 1], L), pz = fwrapT<T>((T)pos[3 * i + 2], L);
    T X, Y, Z;
    if constexpr (sizeof(T) == 4) {
        X = grid_coord<T>(px, g, g_lo);
        Y = grid_coord<T>(py, g, g_lo);
        Z = grid_coord<T>(pz, g, g_lo);
    } else {
        X = px / gfac;
        Y = py / gfac;
        Z = pz / gfac;
    }
    const int iX = (int)dfloor<T>(X), iY = (int)dfloor<T>(Y), iZ = (int)dfloor<T>(Z);
    const T dx = X - iX, dy = Y - iY, dz = Z - iZ;
    const T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
    const long rp = N + 2;
    const int x0 = wrapn(iX, N), x1 = wrapn(iX + 1, N);
    const int y0 = wrapn(iY, N), y1 = wrapn(iY + 1, N);
    const int z0 = wrapn(iZ, N), z1 = wrapn(iZ + 1, N);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z0, val * tx * ty * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z0, val * dx * ty * tz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z0, val * tx * dy * tz);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z1, val * tx * ty * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z0, val * dx * dy * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z1, val * dx * ty * dz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z1, val * tx * dy * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z1, val * dx * dy * dz);
}

int displace_and_deposit(int N, int M, double boxlen, int precision, const void *d0, const void *d1,
                         const void *d2, void *rho, float *pos_out, float *posraw_out) {
    const long np = (long)M * M * M;
    const float Lf = (float)boxlen;
    const float spacing = Lf / M;  // src/particle.c:102-103
    const double gfac = boxlen / N;
    const double val = ((double)N * N * N) / ((double)M * M * M);
    const unsigned blocks = (unsigned)((np + 255) / 256);
    launch_begin("displace_cic");
    if (precision == MITOS_FP32) {
        float g, g_lo;
        grid_scale<float>(N, boxlen, g, g_lo);
        k_displace_cic<float><<<blocks, 256, 0, stream()>>>(N, M, spacing, (float)boxlen, (float)gfac, g, g_lo, (float)val,
                                                            (const float *)d0, (const float *)d1, (const float *)d2,
                                                            (float *)rho, pos_out, posraw_out);
    } else {
        k_displace_cic<double><<<blocks, 256, 0, stream()>>>(N, M, spacing, boxlen, gfac, 0.0, 0.0, val, (const double *)d0,
                                                             (const double *)d1, (const double *)d2, (double *)rho,
                                                             pos_out, posraw_out);
    }
    count_launch();
    MITOS_LAUNCH_CHECK("displace + CIC");
    return 0;
}

// Particle velocities (src/mitos.c:865-908): the TSC gather (src/grids_interp.c:267-309) of each
// velocity grid (pitch N + 2) at the displaced, not yet wrapped position, X = x N / boxlen; float out.
// The node offsets and weights are computed once for the three grids; `ld(g, x, y, z)` reads grid g at
// node (x, y, z) in the caller's indexing (wrapped global indices, or tile indices).
template <typename T>
struct VelStencil {
    int nx, ny, nz;
    T wx[3], wy[3], wz[3];
};
template <typename T>
__device__ __forceinline__ VelStencil<T> vel_stencil(const float *p, int N, T boxlen) {
    const T Nf = (T)N;
    const T X = (T)p[0] * Nf / boxlen, Y = (T)p[1] * Nf / boxlen, Z = (T)p[2] * Nf / boxlen;
    const T half = (T)0.5;
    VelStencil<T> st;
    st.nx = (int)dfloor<T>(X + half);
    st.ny = (int)dfloor<T>(Y + half);
    st.nz = (int)dfloor<T>(Z + half);
    const T dx = X - (T)st.nx, dy = Y - (T)st.ny, dz = Z - (T)st.nz;
    st.wx[0] = half * (half - dx) * (half - dx); st.wx[1] = (T)0.75 - dx * dx; st.wx[2] = half * (half + dx) * (half + dx);
    st.wy[0] = half * (half - dy) * (half - dy); st.wy[1] = (T)0.75 - dy * dy; st.wy[2] = half * (half + dy) * (half + dy);
    st.wz[0] = half * (half - dz) * (half - dz); st.wz[1] = (T)0.75 - dz * dz; st.wz[2] = half * (half + dz) * (half + dz);
    return st;
}
// the sums over the 27 nodes in the order of tsc_gather; xi/yi/zi: the nodes' indices for ld
template <typename T, typename Ld>
__device__ __forceinline__ void vel_sums(const VelStencil<T> &st, const int *xi, const int *yi, const int *zi, Ld ld,
                                         float *out) {
    T s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T y0 = 0, y1 = 0, y2 = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T z0 = 0, z1 = 0, z2 = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                z0 += st.wz[k] * ld(0, xi[i], yi[j], zi[k]);
                z1 += st.wz[k] * ld(1, xi[i], yi[j], zi[k]);
                z2 += st.wz[k] * ld(2, xi[i], yi[j], zi[k]);
            }
            y0 += st.wy[j] * z0;
            y1 += st.wy[j] * z1;
            y2 += st.wy[j] * z2;
        }
        s0 += st.wx[i] * y0;
        s1 += st.wx[i] * y1;
        s2 += st.wx[i] * y2;
    }
    out[0] = (float)s0;
    out[1] = (float)s1;
    out[2] = (float)s2;
}

template <typename T>
__device__ __forceinline__ void vel_gather_global(const float *p, int N, int pitch, T boxlen, const T *__restrict__ v0,
                                                  const T *__restrict__ v1, const T *__restrict__ v2, float *out) {
    const VelStencil<T> st = vel_stencil<T>(p, N, boxlen);
    int zi[3], yi[3], xi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        zi[k] = wrapn(st.nz - 1 + k, N);
        yi[k] = wrapn(st.ny - 1 + k, N);
        xi[k] = wrapn(st.nx - 1 + k, N);
    }
    const long rp = pitch;
    auto ld = [&](int g, int x, int y, int z) {
        const long o = ((long)x * N + y) * rp + z;
        return __ldg((g == 0 ? v0 : g == 1 ? v1 : v2) + o);
    };
    vel_sums<T>(st, xi, yi, zi, ld, out);
}

template <typename T>
__global__ void k_vel_gather(long np, int N, int pitch, T boxlen, const float *__restrict__ pos, const T *__restrict__ v0,
                             const T *__restrict__ v1, const T *__restrict__ v2, float *__restrict__ vel) {
    const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= np) return;
    vel_gather_global<T>(pos + 3 * id, N, pitch, boxlen, v0, v1, v2, vel + 3 * id);
}

// Lattice-aligned form (M = N, particle i near node i): one 8 x 8 x 32 brick of particles a block,
// the three velocity tiles staged in shared memory with a one-node halo in x and y and rows of 40 z
// (z0 - 4 .. z0 + 35: 16-byte aligned, the halo of one inside), so the 81 reads of a particle come
// from shared memory.  A particle whose stencil leaves the tiles (displaced by over half a cell, a few
// in 10^5 at z = 31 with 2 Mpc/h cells) reads global memory; the arithmetic is the same either way.
#define VB_X 8
#define VB_Y 8
#define VB_Z 32
#define VB_THREADS 256
#define VR_X (VB_X + 2)
#define VR_Y (VB_Y + 2)
#define VR_Z (VB_Z + 8)
#define VR_Z0 4

// the three tiles plus the tensor copies' mbarrier
static size_t vel_tiled_smem(size_t elem) { return 3 * elem * (size_t)VR_X * VR_Y * VR_Z + sizeof(uint64_t); }

// tensor maps of the three velocity grids, box {VR_Z, VR_Y, VR_X} (z innermost)
struct VelMaps {
    CUtensorMap m[3];
};

// Bricks whose tiles stay inside the box (not on a face in x, y or z) are staged by three tensor
// copies from one thread on an mbarrier; the others, whose halos wrap, by 16-byte cp.async.
template <typename T>
__global__ void __launch_bounds__(VB_THREADS) k_vel_gather_tiled(int N, int pitch, T boxlen, const float *__restrict__ pos,
                                                                 const T *__restrict__ v0, const T *__restrict__ v1,
                                                                 const T *__restrict__ v2, float *__restrict__ vel,
                                                                 FastDiv div_bx, FastDiv div_by,
                                                                 const __grid_constant__ VelMaps maps, int use_tma) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *tile = reinterpret_cast<T *>(smraw);  // [grid][VR_X][VR_Y][VR_Z]
    const int bx_n = N / VB_X, by_n = N / VB_Y, bz_n = N / VB_Z;
    const unsigned b = blockIdx.x;
    const unsigned q = fdiv(b, div_bx);
    const int bx = (int)(b - q * bx_n), bz = (int)fdiv(q, div_by), by = (int)(q - bz * by_n);
    const int x0 = bx * VB_X, y0 = by * VB_Y, z0 = bz * VB_Z;
    const long rp = pitch;
    constexpr int TILE = VR_X * VR_Y * VR_Z;
    const bool tma = use_tma && bx > 0 && bx < bx_n - 1 && by > 0 && by < by_n - 1 && bz > 0 && bz < bz_n - 1 &&
                     (smem_u32(tile) & 127) == 0;
    if (tma) {
        uint64_t *bar = reinterpret_cast<uint64_t *>(tile + 3 * TILE);
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            mbar_init_fence();
            mbar_expect_tx(bar, (unsigned)(3 * TILE * sizeof(T)));
            for (int g = 0; g < 3; g++) tma_load_3d(tile + g * TILE, &maps.m[g], z0 - VR_Z0, y0 - 1, x0 - 1, bar);
        }
        __syncthreads();  // the barrier is initialised before anyone polls it
        const bool ok = mbar_wait(bar, 0);
        if (__syncthreads_or(!ok)) {  // a copy that never completed: flag it, wait once more (bounded), stop
            if (threadIdx.x == 0) atomicExch(&g_lattice_fault, 1);
            mbar_wait(bar, 0);
            return;
        }
    } else {
        constexpr int CH = 16 / sizeof(T), RC = VR_Z / CH, ROWS = VR_X * VR_Y;
        for (int c = threadIdx.x; c < 3 * ROWS * RC; c += VB_THREADS) {
            const int g = c / (ROWS * RC), r = (c / RC) % ROWS, ch = c % RC;
            const int lx = r / VR_Y, ly = r % VR_Y;
            const T *src = (g == 0 ? v0 : g == 1 ? v1 : v2) +
                           ((long)wrapn(x0 - 1 + lx, N) * N + wrapn(y0 - 1 + ly, N)) * rp +
                           wrapn(z0 - VR_Z0 + ch * CH, N);  // chunks never straddle the wrap: N % CH == 0
            cp_async16(tile + (long)c * CH, src);
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
    }
    const int lz = threadIdx.x % VB_Z, ly = (threadIdx.x / VB_Z) % VB_Y;
#pragma unroll 1
    for (int lx = threadIdx.x / (VB_Z * VB_Y); lx < VB_X; lx += VB_THREADS / (VB_Z * VB_Y)) {
        const long id = ((long)(x0 + lx) * N + y0 + ly) * N + z0 + lz;
        const float *p = pos + 3 * id;
        const VelStencil<T> st = vel_stencil<T>(p, N, boxlen);
        // tile indices of the first stencil node
        const int ix = st.nx - x0, iy = st.ny - y0, iz = st.nz - 1 - (z0 - VR_Z0);
        if (ix >= 0 && ix + 2 < VR_X && iy >= 0 && iy + 2 < VR_Y && iz >= 0 && iz + 2 < VR_Z) {
            const int xi[3] = {ix, ix + 1, ix + 2}, yi[3] = {iy, iy + 1, iy + 2}, zi[3] = {iz, iz + 1, iz + 2};
            auto ld = [&](int g, int x, int y, int z) { return tile[((g * VR_X + x) * VR_Y + y) * VR_Z + z]; };
            vel_sums<T>(st, xi, yi, zi, ld, vel + 3 * id);
        } else {
            vel_gather_global<T>(p, N, pitch, boxlen, v0, v1, v2, vel + 3 * id);
        }
    }
}

int velocity_gather(long np, int N, int pitch, double boxlen, int precision, const float *pos, const void *v0,
                    const void *v1, const void *v2, float *vel) {
    const size_t es = precision == MITOS_FP32 ? 4 : 8;
    // the brick-tiled form: lattice particles (np = N^3 in lattice order), bricks that tile the grid,
    // 16-byte aligned grid rows
    if (np == (long)N * N * N && N % VB_X == 0 && N % VB_Y == 0 && N % VB_Z == 0 && (pitch * es) % 16 == 0 &&
        ((uintptr_t)v0 | (uintptr_t)v1 | (uintptr_t)v2) % 16 == 0) {
        const size_t smem = vel_tiled_smem(es);
        const unsigned nb = (unsigned)((N / VB_X) * (N / VB_Y) * (N / VB_Z));
        const FastDiv dbx = make_fastdiv((unsigned)(N / VB_X)), dby = make_fastdiv((unsigned)(N / VB_Y));
        VelMaps maps;
        memset(&maps, 0, sizeof maps);
        const bool f64 = precision != MITOS_FP32;
        const void *vg[3] = {v0, v1, v2};
        int use_tma = lattice_tma() ? 1 : 0;
        for (int gi = 0; gi < 3 && use_tma; gi++)
            use_tma = encode_grid_map(&maps.m[gi], vg[gi], f64, N, N, pitch, VR_Z, VR_Y, VR_X) ? 1 : 0;
        launch_begin("vel_gather");
        if (precision == MITOS_FP32) {
            MITOS_CUDA(cudaFuncSetAttribute(k_vel_gather_tiled<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_vel_gather_tiled<float><<<nb, VB_THREADS, smem, stream()>>>(N, pitch, (float)boxlen, pos, (const float *)v0,
                                                                          (const float *)v1, (const float *)v2, vel, dbx, dby,
                                                                          maps, use_tma);
        } else {
            MITOS_CUDA(cudaFuncSetAttribute(k_vel_gather_tiled<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_vel_gather_tiled<double><<<nb, VB_THREADS, smem, stream()>>>(N, pitch, boxlen, pos, (const double *)v0,
                                                                           (const double *)v1, (const double *)v2, vel, dbx, dby,
                                                                           maps, use_tma);
        }
        count_launch();
        MITOS_LAUNCH_CHECK("velocity gather (tiled)");
        return 0;
    }
    const unsigned blocks = (unsigned)((np + 255) / 256);
    launch_begin("vel_gather");
    if (precision == MITOS_FP32)
        k_vel_gather<float><<<blocks, 256, 0, stream()>>>(np, N, pitch, (float)boxlen, pos, (const float *)v0,
                                                          (const float *)v1, (const float *)v2, vel);
    else
        k_vel_gather<double><<<blocks, 256, 0, stream()>>>(np, N, pitch, boxlen, pos, (const double *)v0,
                                                           (const double *)v1, (const double *)v2, vel);
    count_launch();
    MITOS_LAUNCH_CHECK("velocity gather");
    return 0;
}

// the particle datasets of the snapshot (src/mitos.c:1106-1117): Coordinates and Velocities as
// double (from the float particle fields), Masses as double of the float mass, ParticleIDs the
// row-major lattice index plus the species' first id (src/particle.c:114-121); any output may be null
__global__ void k_snapshot(long n, const float *__restrict__ pos, const float *__restrict__ vel, float mass,
                           long long id_first, double *__restrict__ coords, double *__restrict__ vels,
                           double *__restrict__ masses, long long *__restrict__ ids) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (coords)
            for (int c = 0; c < 3; c++) coords[3 * i + c] = (double)pos[3 * i + c];
        if (vels)
            for (int c = 0; c < 3; c++) vels[3 * i + c] = vel ? (double)vel[3 * i + c] : 0.0;
        if (masses) masses[i] = (double)mass;
        if (ids) ids[i] = id_first + i;
    }
}

int snapshot_arrays(long n, const float *pos, const float *vel, float mass, long long id_first, double *coords,
                    double *vels, double *masses, long long *ids) {
    const unsigned blocks = (unsigned)std::min<long>((n + 255) / 256, 152L * 16);
    launch_begin("snapshot");
    k_snapshot<<<blocks, 256, 0, stream()>>>(n, pos, vel, mass, id_first, coords, vels, masses, ids);
    count_launch();
    MITOS_LAUNCH_CHECK("snapshot arrays");
    return 0;
}

// real-space grid of either precision as doubles in its padded layout (N x N x (N + 2))
__global__ void k_widen(long n, const float *__restrict__ src, double *__restrict__ dst) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

int widen_to_double(long n, const float *src, double *dst) {
    const unsigned blocks = (unsigned)std::min<long>((n + 255) / 256, 152L * 16);
    launch_begin("widen");
    k_widen<<<blocks, 256, 0, stream()>>>(n, src, dst);
    count_launch();
    MITOS_LAUNCH_CHECK("widen to double");
    return 0;
}

int cic_positions(long n, int N, double boxlen, int precision, const float *pos, double val, void *rho) {
    const double gfac = boxlen / N;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    launch_begin("cic");
    if (precision == MITOS_FP32) {
        float g, g_lo;
        grid_scale<float>(N, boxlen, g, g_lo);
        k_cic<float><<<blocks, 256, 0, stream()>>>(n, N, (float)boxlen, (float)gfac, g, g_lo, (float)val, pos, (float *)rho);
    } else {
        k_cic<double><<<blocks, 256, 0, stream()>>>(n, N, boxlen, gfac, 0.0, 0.0, val, pos, (double *)rho);
    }
    count_launch();
    MITOS_LAUNCH_CHECK("CIC");
    return 0;
}

}  // namespace mitos
