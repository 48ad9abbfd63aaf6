// particles.cu -- lattice particles displaced by TSC-gathered displacement grids, then CIC mass
// assignment onto a grid.
//
// Follows src/particle.c:87-129 (float lattice positions), src/mitos.c:843-862 (one TSC gather
// per direction; the gather of direction d sees the displacements of directions < d already
// applied), src/mitos.c:1072-1077 (periodic wrap) and analyse/src/mitos_read.c:280-334 (CIC).
// The deposit is accumulated in units of the mean density: each particle adds (N/M)^3 split
// over its 8 cells, so the overdensity is the deposited value minus one.
#include <math.h>

#include "context.cuh"
#include "particles.cuh"

namespace mitos {

template <typename T> __device__ __forceinline__ T dfloor(T x);
template <> __device__ __forceinline__ float dfloor<float>(float x) { return floorf(x); }
template <> __device__ __forceinline__ double dfloor<double>(double x) { return floor(x); }

__device__ __forceinline__ int wrapi(int i, int N) {
    i %= N;
    return i < 0 ? i + N : i;
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
    int zi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) zi[k] = wrapi(nz - 1 + k, N);
    const long rp = N + 2;
    T sum = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const long xo = (long)wrapi(nx - 1 + i, N) * N;
        T sy = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const T *row = box + (xo + wrapi(ny - 1 + j, N)) * rp;
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

template <typename T>
__global__ void __launch_bounds__(256)
k_displace_cic(int N, int M, float spacing, T boxlen, T gfac, T val,
               const T *__restrict__ d0, const T *__restrict__ d1, const T *__restrict__ d2,
               T *__restrict__ rho, float *__restrict__ pos_out) {
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
        // X = x N / boxlen (src/grids_interp.c:269-271)
        const T disp = tsc_gather<T>(dd[dir], N, (T)p[0] * Nf / boxlen, (T)p[1] * Nf / boxlen,
                                     (T)p[2] * Nf / boxlen);
        p[dir] = (float)((T)p[dir] - disp);
    }
    const float Lf = (float)boxlen;
#pragma unroll
    for (int c = 0; c < 3; c++) p[c] = fwrapf(p[c], Lf);
    if (pos_out) {
        pos_out[3 * id] = p[0];
        pos_out[3 * id + 1] = p[1];
        pos_out[3 * id + 2] = p[2];
    }
    // CIC: X = x / (L / N) (analyse/src/mitos_read.c:288-333)
    const T X = (T)p[0] / gfac, Y = (T)p[1] / gfac, Z = (T)p[2] / gfac;
    const int iX = (int)dfloor<T>(X), iY = (int)dfloor<T>(Y), iZ = (int)dfloor<T>(Z);
    const T dx = X - iX, dy = Y - iY, dz = Z - iZ;
    const T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
    const long rp = N + 2;
    const int x0 = wrapi(iX, N), x1 = wrapi(iX + 1, N);
    const int y0 = wrapi(iY, N), y1 = wrapi(iY + 1, N);
    const int z0 = wrapi(iZ, N), z1 = wrapi(iZ + 1, N);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z0, val * tx * ty * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z0, val * dx * ty * tz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z0, val * tx * dy * tz);
    atomicAdd(rho + ((long)x0 * N + y0) * rp + z1, val * tx * ty * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z0, val * dx * dy * tz);
    atomicAdd(rho + ((long)x1 * N + y0) * rp + z1, val * dx * ty * dz);
    atomicAdd(rho + ((long)x0 * N + y1) * rp + z1, val * tx * dy * dz);
    atomicAdd(rho + ((long)x1 * N + y1) * rp + z1, val * dx * dy * dz);
}

// CIC of given positions (cic_deposit_dg)
template <typename T>
__global__ void k_cic(long n, int N, T gfac, T val, const float *__restrict__ pos, T *__restrict__ rho) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // x = fwrap(x, L) in the working precision, X = x / (L / N) (analyse/src/mitos_read.c:284-290)
    const T L = gfac * (T)N;
    const T X = fwrapT<T>((T)pos[3 * i], L) / gfac, Y = fwrapT<T>((T)pos[3 * i + 1], L) / gfac,
            Z = fwrapT<T>((T)pos[3 * i + 2], L) / gfac;
    const int iX = (int)dfloor<T>(X), iY = (int)dfloor<T>(Y), iZ = (int)dfloor<T>(Z);
    const T dx = X - iX, dy = Y - iY, dz = Z - iZ;
    const T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
    const long rp = N + 2;
    const int x0 = wrapi(iX, N), x1 = wrapi(iX + 1, N);
    const int y0 = wrapi(iY, N), y1 = wrapi(iY + 1, N);
    const int z0 = wrapi(iZ, N), z1 = wrapi(iZ + 1, N);
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
                         const void *d2, void *rho, float *pos_out) {
    const long np = (long)M * M * M;
    const float Lf = (float)boxlen;
    const float spacing = Lf / M;  // src/particle.c:102-103
    const double gfac = boxlen / N;
    const double val = ((double)N * N * N) / ((double)M * M * M);
    const unsigned blocks = (unsigned)((np + 255) / 256);
    launch_begin("displace_cic");
    if (precision == MITOS_FP32)
        k_displace_cic<float><<<blocks, 256, 0, stream()>>>(N, M, spacing, (float)boxlen, (float)gfac, (float)val,
                                                            (const float *)d0, (const float *)d1, (const float *)d2,
                                                            (float *)rho, pos_out);
    else
        k_displace_cic<double><<<blocks, 256, 0, stream()>>>(N, M, spacing, boxlen, gfac, val, (const double *)d0,
                                                             (const double *)d1, (const double *)d2, (double *)rho,
                                                             pos_out);
    count_launch();
    MITOS_LAUNCH_CHECK("displace + CIC");
    return 0;
}

int cic_positions(long n, int N, double boxlen, int precision, const float *pos, double val, void *rho) {
    const double gfac = boxlen / N;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    launch_begin("cic");
    if (precision == MITOS_FP32)
        k_cic<float><<<blocks, 256, 0, stream()>>>(n, N, (float)gfac, (float)val, pos, (float *)rho);
    else
        k_cic<double><<<blocks, 256, 0, stream()>>>(n, N, gfac, val, pos, (double *)rho);
    count_launch();
    MITOS_LAUNCH_CHECK("CIC");
    return 0;
}

}  // namespace mitos
