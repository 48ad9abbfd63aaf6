// fft_kernels.cuh -- X / Y / Z pass kernels of the 3D real FFT with fused k-space operations,
// and their launch templates.  NL = 0 instantiates the runtime-plan kernels; NL > 0 the
// compile-time specialisation for that transform length (fft_ct*.cu).
#pragma once

#include "context.cuh"
#include "tma.cuh"

namespace mitos {

template <typename T> __device__ __forceinline__ T dev_sqrt(T x);
template <> __device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }

// ------------------------------------------------------------------------------------------
// X and Y passes: complex FFTs along a strided axis.  Block = P pencils; thread (t, p) with
// p fastest so that a warp reads P consecutive columns of each row.
// ------------------------------------------------------------------------------------------
// The multi-output Y passes (Hessian, displacement) of the compile-time lengths run 256-thread
// blocks (4 pencils), three an SM with up to 80 registers.  Everything else runs 512-thread blocks
// (the X passes need the wider pencil groups for coalescing: their pencils are adjacent columns of
// an x-plane).
template <int AXIS, int OP, int NL> constexpr bool strided_heavy() {
    return NL > 0 && AXIS == 1 && (OP == YOP_DISP_A || OP == YOP_HESS_A || OP == YOP_HESS_B);
}

// Blocks per SM the register allocation is sized for (measured at 512^3): the Hessian X pass one
// 512-thread block with up to 128 registers (at 64 it spills 216 bytes a thread: 0.70 ms against
// 0.85); the displacement Y pass three 256-thread blocks (79 registers, no spills: 0.905 ms against
// 0.972 with two) and so do the single-input Hessian Y passes (a three-input pass needed 128
// registers at two blocks: 1.66 ms, against 1.41 for the three single-input passes).  The
// displacement Y step is split the same way (a two-input pass and a stencil-only pass).
// (The X passes keep 8 pencils a block: 64-byte row segments.  With 4 pencils in 256-thread blocks,
// three a SM, x_combine_disp ran 1.00 ms against 0.87 and x_hess 1.05 against 0.70.)
template <int AXIS, int OP, int NL, int PC, int E> constexpr int strided_threads() {
    return NL > 0 ? PC * (NL / E) : (strided_heavy<AXIS, OP, NL>() ? 256 : 512);
}
template <int AXIS, int OP, int NL, int PC, int E> constexpr int strided_min_blocks() {
    return (NL > 0 && AXIS == 0 && OP == XOP_HESS) ? 1
           : (NL > 0 && AXIS == 1 && (OP == YOP_DISP_A || OP == YOP_HESS_A || OP == YOP_HESS_B)) ? (E > 12 ? 2 : 3) : 2;
}

template <typename T, int E, int SIGN, int AXIS, int OP, int NL, int PC>
__global__ void __launch_bounds__(strided_threads<AXIS, OP, NL, PC, E>(), strided_min_blocks<AXIS, OP, NL, PC, E>()) k_strided(GridGeom g, PassArgs a, const T *__restrict__ win) {
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smraw);
    const FFTPlan &pl = g.plN;
    const int P = PC > 0 ? PC : g.P_xy;
    const int tid = threadIdx.x, p = tid % P, t = tid / P;
    const int N = g.N, H = g.H;
    long base, stride;
    bool valid;
    int ix = 0, iy = 0, iz;
    if (AXIS == 0) {
        long col = (long)blockIdx.x * P + p;
        valid = col < g.plane;
        if (!valid) col = 0;
        base = col;
        stride = g.plane;
        iy = kint((int)(col / H), N);
        iz = (int)(col % H);
    } else {
        int tiles = (H + P - 1) / P;
        int x = blockIdx.x / tiles;
        int kz = (blockIdx.x % tiles) * P + p;
        valid = kz < H;
        if (!valid) kz = 0;
        base = (long)x * g.plane + kz;
        stride = H;
        ix = kint(x, N);
        iz = kz;
    }
    const cplx<T> *tw = reinterpret_cast<const cplx<T> *>(g.twN);
    const T dk = parg<T>(a.dk, a.fdk);
    const T scale = parg<T>(a.scale, a.fscale);
    cplx<T> *psm = sm + p;
    const size_t bo = (size_t)blockIdx.y * (size_t)a.bstride;  // realisation of a batched launch

    // P(k): one power histogram per warp behind the FFT exchange buffer (the counts and the
    // wavenumber sums of the bins depend only on the geometry and are tabulated on the host)
    T *hp = nullptr;
    if constexpr (OP == XOP_PK) {
        size_t off = (size_t)P * spad_len(N) * sizeof(cplx<T>);
        T *hist = reinterpret_cast<T *>(smraw + off);
        const int nw = blockDim.x >> 5;
        for (int i = tid; i < a.nbins * nw; i += blockDim.x) hist[i] = 0;
        hp = hist + (tid >> 5) * a.nbins;
        __syncthreads();
    }

    // the forward X passes that combine with a second grid (2LPT combine, Monge-Ampere update) read
    // it after their transform: its elements go to shared memory by cp.async first ([e][thread],
    // behind the exchange buffer; each thread reads back only its own copies)
    constexpr bool STAGE2 = AXIS == 0 && (OP == XOP_COMBINE_2LPT || OP == XOP_ADD_POISSON);
    cplx<T> *ph = sm + (long)P * spad_len(N) + threadIdx.x;
    if constexpr (STAGE2) {
        const cplx<T> *in2 = bat<const cplx<T>>(a.in2, bo);
#pragma unroll
        for (int e = 0; e < E; e++) {
            const cplx<T> *s2 = in2 + base + (long)nout_any<NL, E>(pl, t, e) * stride;
            const unsigned d = (unsigned)__cvta_generic_to_shared(ph + e * blockDim.x);
            if (sizeof(cplx<T>) == 8)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(s2) : "memory");
            else
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(s2) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }

    constexpr int NIN = 1;
    cplx<T> raw[E];
    cplx<T> v[E];
#pragma unroll 1
    for (int i = 0; i < NIN; i++) {
        const cplx<T> *src = bat<const cplx<T>>(a.in[i], bo);
#pragma unroll
        for (int e = 0; e < E; e++) {
            int n = nin_any<NL, E>(pl, t, e);
            raw[e] = valid ? src[base + (long)n * stride] : mk<T>(0, 0);
            // window undo applied on load by the inverse X passes (XOP_DISP / XOP_HESS)
            if constexpr (AXIS == 0 && (OP == XOP_DISP || OP == XOP_HESS)) {
                if (win) raw[e] = cscale<T>(raw[e], win[kint(n, N) + N / 2] * win[iy + N / 2] * win[iz + N / 2]);
            }
        }
        // outputs produced from input i: (output index, factor) with factor 0: 1, 1: i k, 2: -k^2
        int nout = 1;
        int outs[3] = {0, 0, 0}, facs[3] = {0, 0, 0};
        if (AXIS == 0 && OP == XOP_HESS) { nout = 3; outs[1] = 1; outs[2] = 2; facs[1] = 1; facs[2] = 2; }
        if (AXIS == 0 && OP == XOP_DISP) { nout = 2; outs[1] = 1; facs[1] = 1; }
        if (AXIS == 1 && OP == YOP_DISP_A) { nout = 2; outs[1] = 1; facs[0] = 1; }
        if (AXIS == 1 && OP == YOP_HESS_A) { nout = 3; outs[1] = 1; outs[2] = 2; facs[0] = 2; facs[1] = 1; }
        if (AXIS == 1 && OP == YOP_HESS_B) { nout = 2; outs[1] = 1; facs[0] = 1; }
        constexpr int MU = (OP == YOP_HESS_A || OP == YOP_HESS_B || OP == YOP_DISP_A) ? 3 : 1;
#pragma unroll MU
        for (int m = 0; m < nout; m++) {
            const int fac = facs[m];
            // on-node TSC stencil of the displacement passes, applied to the k-space input:
            // x for the d_x chain (X output 1), y for the d_x and d_y chains (Y outputs 0, 1)
            const T *stn = nullptr;
            if constexpr ((AXIS == 0 && OP == XOP_DISP) || (AXIS == 1 && (OP == YOP_DISP_A || OP == YOP_STN))) {
                if ((AXIS == 0 && outs[m] == 1) || (AXIS == 1 && outs[m] == 0))
                    stn = reinterpret_cast<const T *>(a.stencil);
            }
#pragma unroll
            for (int e = 0; e < E; e++) {
                cplx<T> x = raw[e];
                if (fac != 0) {
                    T kk = (T)kint(nin_any<NL, E>(pl, t, e), N) * dk;
                    x = (fac == 1) ? cmul_is<T>(x, kk) : cscale<T>(x, -kk * kk);
                }
                if (stn) x = cscale<T>(x, stn[kint(nin_any<NL, E>(pl, t, e), N) + N / 2]);
                v[e] = x;
            }
            fft_any<T, E, SIGN, NL, PC>(pl, v, psm, P, t, tw);
            // the P(k) epilogue keeps the whole warp together (warp-level bin sums)
            if constexpr (STAGE2) asm volatile("cp.async.wait_all;" ::: "memory");  // every thread
            if (!valid && OP != XOP_PK) continue;
            cplx<T> *dst = bat<cplx<T>>(a.out[outs[m]], bo);
#pragma unroll
            for (int e = 0; e < E; e++) {
                int n = nout_any<NL, E>(pl, t, e);
                long idx = base + (long)n * stride;
                cplx<T> r = cscale<T>(v[e], scale);
                if constexpr (AXIS == 0 && (OP == XOP_COMBINE_2LPT || OP == XOP_ADD_POISSON ||
                                            OP == XOP_PK)) {
                    const int jx = kint(n, N);
                    // |n|^2 <= 3 (N/2)^2 fits an int; a 64-bit integer -> float conversion would
                    // run on the FP64 pipe
                    const int n2 = jx * jx + iy * iy + iz * iz;
                    if constexpr (OP == XOP_PK) {
                        if (win) r = cscale<T>(r, win[jx + N / 2] * win[iy + N / 2] * win[iz + N / 2]);
                        const int bin = valid ? a.bin_of_n2[n2] : -1;
                        const T mult = (iz == 0 || iz == N / 2) ? (T)1 : (T)2;
                        T pw = valid ? mult * (r.x * r.x + r.y * r.y) : (T)0;
                        // runs of equal bins in lane order (the lanes of a warp hold consecutive
                        // x indices of a pencil, so a bin covers a run of lanes): a segmented
                        // inclusive scan over the run, whose last lane adds the run's sum to the
                        // warp's histogram (shared atomics: two runs of one warp may share a bin)
                        const int lane = threadIdx.x & 31;
                        const int prev = __shfl_up_sync(0xffffffffu, bin, 1);
                        const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != bin);
                        const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
                        for (int off = 1; off < 32; off <<= 1) {
                            const T y = __shfl_up_sync(0xffffffffu, pw, off);
                            if (lane - off >= start) pw += y;
                        }
                        const bool last = lane == 31 || ((heads >> (lane + 1)) & 1u);
                        if (last && bin >= 0) atomicAdd(hp + bin, pw);
                        if (valid && a.out[0]) dst[idx] = r;
                    } else {
                        const T kk2 = (T)n2 * dk * dk;
                        const T G = (n2 > 0) ? (T)-1 / kk2 : (T)1;
                        const cplx<T> q = ph[e * blockDim.x];
                        cplx<T> o;
                        if constexpr (OP == XOP_COMBINE_2LPT) {
                            const T f1 = parg<T>(a.f1, a.ff1), f2 = parg<T>(a.f2, a.ff2);
                            o = mk<T>(f1 * q.x + f2 * G * r.x, f1 * q.y + f2 * G * r.y);
                        } else {
                            o = mk<T>(q.x + G * r.x, q.y + G * r.y);
                        }
                        if (win) o = cscale<T>(o, win[jx + N / 2] * win[iy + N / 2] * win[iz + N / 2]);
                        dst[idx] = o;
                    }
                } else {
                    dst[idx] = r;
                }
            }
        }
    }
    if constexpr (OP == XOP_PK) {
        __syncthreads();
        const size_t off = (size_t)P * spad_len(N) * sizeof(cplx<T>);
        const T *hist = reinterpret_cast<const T *>(smraw + off);
        const int nw = blockDim.x >> 5;
        // the warps' histograms summed in the kernel's precision (one FP64 conversion and atomic
        // per bin and block: FP64 arithmetic runs at a small fraction of the FP32 rate)
        for (int i = tid; i < a.nbins; i += blockDim.x) {
            T sum = 0;
            for (int w = 0; w < nw; w++) sum += hist[w * a.nbins + i];
            if (sum != (T)0) atomicAdd(a.bin_p + (size_t)blockIdx.y * a.acc_stride + i, (double)sum);
        }
    }
}


// ------------------------------------------------------------------------------------------
// X pass that closes the 2LPT potential and opens the displacement grids in one sweep:
// forward FFT of the source spectrum, phi = (f1 phi1 - f2 S/k^2) / W_TSC, then the inverse
// FFTs of phi and i kx phi (with the on-node stencil of the d_x chain when requested).
// ------------------------------------------------------------------------------------------
// (16 elements a thread: one block an SM, up to 128 registers)
template <typename T, int E, int NL, int PC>
__global__ void __launch_bounds__(512, E > 12 ? 1 : 2) k_x_combine_disp(GridGeom g, PassArgs a, const T *__restrict__ win) {
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smraw);
    const FFTPlan &pl = g.plN;
    const int P = PC > 0 ? PC : g.P_xy;
    const int tid = threadIdx.x, p = tid % P, t = tid / P;
    const int N = g.N, H = g.H;
    long col = (long)blockIdx.x * P + p;
    const bool valid = col < g.plane;
    if (!valid) col = 0;
    const int iy = kint((int)(col / H), N), iz = (int)(col % H);
    const cplx<T> *tw = reinterpret_cast<const cplx<T> *>(g.twN);
    const T dk = parg<T>(a.dk, a.fdk), scale = parg<T>(a.scale, a.fscale), f1 = parg<T>(a.f1, a.ff1),
            f2 = parg<T>(a.f2, a.ff2);
    const T *stn = reinterpret_cast<const T *>(a.stencil);
    cplx<T> *psm = sm + p;
    const size_t bo = (size_t)blockIdx.y * (size_t)a.bstride;
    const cplx<T> *src = bat<const cplx<T>>(a.in[0], bo);
    const cplx<T> *phi1 = bat<const cplx<T>>(a.in2, bo);
    // phi_1 is read after the forward transform: its elements go to shared memory by cp.async now
    // ([e][thread], behind the exchange buffer; each thread reads back only its own copies), so the
    // loads overlap the transform.  (An L2 prefetch instead: 0.81 ms at 512^3, none: 0.86.)
    cplx<T> *ph = sm + (long)P * spad_len(N) + threadIdx.x;
#pragma unroll
    for (int e = 0; e < E; e++) {
        const cplx<T> *src1 = phi1 + col + (long)nout_any<NL, E>(pl, t, e) * g.plane;
        const unsigned d = (unsigned)__cvta_generic_to_shared(ph + e * blockDim.x);
        if (sizeof(cplx<T>) == 8)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src1) : "memory");
        else
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src1) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    cplx<T> v[E];
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = valid ? src[col + (long)nin_any<NL, E>(pl, t, e) * g.plane] : mk<T>(0, 0);
    fft_any<T, E, -1, NL, PC>(pl, v, psm, P, t, tw);
    const T wyz = win ? win[iy + N / 2] * win[iz + N / 2] : (T)1;
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int n = nout_any<NL, E>(pl, t, e);
        const int jx = kint(n, N);
        const int n2 = jx * jx + iy * iy + iz * iz;  // int: see the strided X passes
        const T G = (n2 > 0) ? (T)-1 / ((T)n2 * dk * dk) : (T)1;
        if (e == 0) asm volatile("cp.async.wait_all;" ::: "memory");
        const cplx<T> q = valid ? ph[e * blockDim.x] : mk<T>(0, 0);
        const cplx<T> r = cscale<T>(v[e], scale);
        cplx<T> o = mk<T>(f1 * q.x + f2 * G * r.x, f1 * q.y + f2 * G * r.y);
        if (win) o = cscale<T>(o, win[jx + N / 2] * wyz);
        psm[spad(n) * P] = o;
    }
    __syncthreads();
    // phi to this thread's own slots of the staging area (phi_1 is consumed): both inverse
    // transforms read it from there rather than keep E more values in registers
#pragma unroll
    for (int e = 0; e < E; e++) ph[e * blockDim.x] = psm[spad(nin_any<NL, E>(pl, t, e)) * P];
    __syncthreads();
#pragma unroll 1
    for (int m = 0; m < 2; m++) {
#pragma unroll
        for (int e = 0; e < E; e++) {
            cplx<T> x = ph[e * blockDim.x];
            if (m == 1) {
                const int jx = kint(nin_any<NL, E>(pl, t, e), N);
                x = cmul_is<T>(x, (T)jx * dk);
                if (stn) x = cscale<T>(x, stn[jx + N / 2]);
            }
            v[e] = x;
        }
        fft_any<T, E, 1, NL, PC>(pl, v, psm, P, t, tw);
        if (valid) {
            cplx<T> *dst = bat<cplx<T>>(a.out[m], bo);
#pragma unroll
            for (int e = 0; e < E; e++) dst[col + (long)nout_any<NL, E>(pl, t, e) * g.plane] = v[e];
        }
    }
}
// ------------------------------------------------------------------------------------------
// Z c2r: rows of N/2+1 complex -> N reals via an N/2-point complex inverse FFT.
// ------------------------------------------------------------------------------------------
// one row of the lean Monge-Ampere residual (order xx, yy, zz, yz, xy, xz; see k_z_c2r): h the
// row's value, o0..o2 the kept rows, R the sum
template <typename T>
__device__ __forceinline__ void ma_lean_step(int q, T h, T &o0, T &o1, T &o2, T &R) {
    if (q == 0) {
        o0 = h;  // xx
    } else if (q == 1) {
        o1 = h;  // yy
    } else if (q == 2) {  // zz
        const T xx = o0, yy = o1, zz = h;
        R = -((xx + yy) + zz) - ((zz * yy + zz * xx) + yy * xx) - (xx * yy) * zz;
        o0 = (T)1 + xx;
        o1 = (T)1 + yy;
        o2 = (T)1 + zz;
    } else if (q == 3) {  // yz
        R += h * h * o0;
        o0 = h;
    } else if (q == 4) {  // xy
        R += h * h * o2;
        o0 = h * o0;
    } else {  // xz
        R += h * h * o1 - (T)2 * o0 * h;
    }
}

// two 256-thread blocks per SM (<= 128 registers) except for the Monge-Ampere residual passes with
// the source output, which keep all six Hessian rows live
template <typename T, int E, int OP, int NL>
__global__ void __launch_bounds__(256, (OP == ZOP_HESS_MA || OP == ZOP_HESS_MA_KS) ? 1 : 2) k_z_c2r(GridGeom g, PassArgs a) {
    constexpr bool S2 = OP == ZOP_HESS_2LPT || OP == ZOP_HESS_2LPT_K;  // the 2LPT source passes
    constexpr bool MA = OP == ZOP_HESS_MA || OP == ZOP_HESS_MA_K || OP == ZOP_HESS_MA_KS;  // residual passes
    constexpr bool LEAN = OP == ZOP_HESS_MA_K;  // the residual accumulated as the rows arrive
    constexpr bool MAK = OP == ZOP_HESS_MA_K || OP == ZOP_HESS_MA_KS;  // residual r2c along z in the pass
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smraw);
    const FFTPlan &pl = g.plH;
    const int h = pl.n, N = g.N, H = g.H;
    const int tpp = h / E;
    const int tid = threadIdx.x, t = tid % tpp, p = tid / tpp;
    long row = (long)blockIdx.x * g.P_z + p;
    const bool valid = row < (long)N * N;
    if (!valid) row = 0;
    const cplx<T> *tw = reinterpret_cast<const cplx<T> *>(g.twN);
    // the 2LPT source pass converts the double copies: its 128-register allocation then keeps the
    // transforms free of spills (measured at 512^3: 1.29 ms, against 1.42 with the FP32 copies)
    const T dk = S2 ? (T)a.dk : parg<T>(a.dk, a.fdk);
    const T scale = S2 ? (T)a.scale : parg<T>(a.scale, a.fscale);
    cplx<T> *psm = sm + (long)p * spad_len(h);
    const size_t bo = (size_t)blockIdx.y * (size_t)a.bstride;
    constexpr int NIN = (OP == ZOP_C2R) ? 1 : (OP == ZOP_DISP) ? 3 : 6;
    // inputs of the Hessian passes are [xx, xy, xz, yy, yz, zz]; the 2LPT source is accumulated
    // in the reference's term order (src/2lpt.c:111-112): zz yy + zz xx + yy xx - xy^2 - yz^2 - xz^2.
    // The lean residual pass takes the rows in the order xx, yy, zz, yz, xy, xz and accumulates
    // R = -tr H - s2(H) - det H (src/monge_ampere.c:119-145 expanded; residual = rho + R):
    //   zz:  R = -((xx + yy) + zz) - ((zz yy + zz xx) + yy xx) - (xx yy) zz; keep 1+xx, 1+yy, 1+zz
    //   yz:  R += yz^2 (1 + xx)              keep yz (in 1+xx's place)
    //   xy:  R += xy^2 (1 + zz)              keep Q = xy yz
    //   xz:  R += xz^2 (1 + yy) - 2 Q xz
    // (the coefficient rows 1 + h carry h's rounding at the size of the product's own; the residual
    // is never formed as a difference of 1 + rho and det(I + H))
    constexpr int NKEEP = LEAN ? 3 : MA ? 6 : S2 ? 2 : 1;
    cplx<T> o[NKEEP][E];
    cplx<T> acc[E];
    T *dst_row = nullptr;
    auto field = [&](int q) {
        return S2 ? (q == 0 ? 0 : q == 1 ? 3 : q == 2 ? 5 : q == 3 ? 1 : q == 4 ? 4 : 2)
                  : LEAN ? (q == 0 ? 0 : q == 1 ? 3 : q == 2 ? 5 : q == 3 ? 4 : q == 4 ? 1 : 2) : q;
    };
    // Input rows of the lean Monge-Ampere residual pass (FP32, compile-time lengths with one pencil
    // a warp or half a warp): the pencil's first lane copies each row into one of the pencil's two row buffers
    // with a bulk copy (cp.async.bulk) completing on the buffer's mbarrier, two rows ahead, so the
    // global reads run while the rows before transform, and the lanes read X[k] and X[h - k] from
    // shared memory.  A row is copied from the 16-byte boundary below it to the one above its end
    // (its own bytes and at most 8 of each neighbour's: inside the grid, whose size is a multiple
    // of 16).  A wait that times out (bounded) flags a.fault and the pencil's warp reads the rest
    // from global memory.  (At 256^3 the pass takes 0.316 against 0.323 ms, its spills 64 bytes a
    // thread against 380.  The 2LPT-source and displacement passes ran slower this way at 512^3:
    // 1.49 against 1.25 ms and 0.81 against 0.66; they read their rows from global memory.)
    constexpr bool ZT = sizeof(T) == 4 && LEAN && NL > 0 && (NL / E == 32 || NL / E == 16);
    const int zrb = ((H * (int)sizeof(cplx<T>) + 8 + 15) / 16) * 16;  // bytes a row buffer
    unsigned char *zb0 = nullptr;
    uint64_t *zbar = nullptr;
    bool zok = true;              // warp-uniform: the row buffers are in use
    unsigned zph = 0, zpend = 0;  // per buffer: parity of its next completion, a copy in flight
    auto zissue = [&](int q, int b) {  // the pencil's first lane: row of input q into buffer b
        const uintptr_t s = reinterpret_cast<uintptr_t>(bat<const cplx<T>>(a.in[field(q)], bo) + row * H);
        const uintptr_t s0 = s & ~(uintptr_t)15;
        const uintptr_t s1 = (s + (uintptr_t)H * sizeof(cplx<T>) + 15) & ~(uintptr_t)15;
        fence_proxy_async();  // the lanes' reads of the buffer before the copy's writes
        mbar_expect_tx(zbar + b, (unsigned)(s1 - s0));
        bulk_load_g2s(zb0 + b * zrb, reinterpret_cast<const void *>(s0), (unsigned)(s1 - s0), zbar + b);
    };
    if constexpr (ZT) {
        const int pb = (int)blockDim.x / tpp;  // pencils a block
        unsigned char *zbase = smraw + (((size_t)pb * spad_len(h) * sizeof(cplx<T>) + 15) & ~(size_t)15);
        zb0 = zbase + (size_t)p * 2 * zrb;
        zbar = reinterpret_cast<uint64_t *>(zbase + (size_t)pb * 2 * zrb) + 2 * p;
        if (t == 0) {
            mbar_init(zbar, 1);
            mbar_init(zbar + 1, 1);
            mbar_init_fence();
        }
        __syncwarp();
        if (t == 0) {
            zissue(0, 0);
            zissue(1, 1);
        }
        zpend = 3;
    }
#pragma unroll
    for (int q = 0; q < NIN; q++) {
        const int f = field(q);
        // kz factor of input f: 0 -> 1, 1 -> i kz, 2 -> -kz^2
        int fac = 0;
        if (S2 || MA) fac = (f == 2 || f == 4) ? 1 : (f == 5 ? 2 : 0);
        if (OP == ZOP_DISP) fac = (f == 2) ? 1 : 0;
        const cplx<T> *src = bat<const cplx<T>>(a.in[f], bo) + row * H;
        // the displacement pass starts the next field's row towards L2 while this one is transformed
        // (one 32-byte sector a lane; measured at 512^3: 0.68 ms against 0.74.  In the 2LPT source
        // pass the same prefetch cost its register allocation: 1.30 ms against 1.09)
        if constexpr (OP == ZOP_DISP) {
            if (q + 1 < NIN) {
                const char *nxt = reinterpret_cast<const char *>(bat<const cplx<T>>(a.in[q + 1], bo) + row * H);
                const int nsec = (int)((H * sizeof(cplx<T>) + 31) / 32);
                for (int sct = t; sct < nsec; sct += tpp) prefetch_l2(nxt + 32 * sct);
            }
        }
        const cplx<T> *rs = src;  // where this row's X[k] and X[h - k] are read
        if constexpr (ZT) {
            const int b = q & 1;
            if (zok) {
                const bool got = __all_sync(0xffffffffu, mbar_wait(zbar + b, (zph >> b) & 1u));
                if (got) {
                    zph ^= 1u << b;
                    zpend &= ~(1u << b);
                    const uintptr_t sa = reinterpret_cast<uintptr_t>(src);
                    rs = reinterpret_cast<const cplx<T> *>(zb0 + b * zrb) + ((sa & 15) ? 1 : 0);
                } else {
                    zok = false;
                    if (t == 0 && a.fault) atomicExch(a.fault, 1);
                }
            }
        }
        cplx<T> v[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int k = nin_any<NL, E>(pl, t, e);
            cplx<T> X = rs[k], Y = rs[h - k];
            if (fac != 0) {
                const T k1 = (T)k * dk, k2 = (T)(h - k) * dk;
                if (fac == 1) { X = cmul_is<T>(X, k1); Y = cmul_is<T>(Y, k2); }
                else { X = cscale<T>(X, -k1 * k1); Y = cscale<T>(Y, -k2 * k2); }
            }
            if constexpr (OP == ZOP_DISP) {
                const T *stn = reinterpret_cast<const T *>(a.stencil);
                if (stn) { X = cscale<T>(X, stn[k + N / 2]); Y = cscale<T>(Y, stn[h - k + N / 2]); }
            }
            if (k == 0) { X.y = 0; Y.y = 0; }
            // E' = X + conj(Y), O' = (X - conj(Y)) e^{+2 pi i k / N}, Z = E' + i O'
            const cplx<T> w = __ldg(tw + k);  // exp(-2 pi i k / N)
            const cplx<T> Ep = mk<T>(X.x + Y.x, X.y - Y.y);
            const cplx<T> D = mk<T>(X.x - Y.x, X.y + Y.y);
            const cplx<T> Op = mk<T>(D.x * w.x + D.y * w.y, D.y * w.x - D.x * w.y);
            v[e] = mk<T>(Ep.x - Op.y, Ep.y + Op.x);
        }
        if constexpr (ZT) {
            // every lane has read buffer q & 1: it takes row q + 2
            if (zok && q + 2 < NIN) {
                __syncwarp();
                if (t == 0) zissue(q + 2, q & 1);
                zpend |= 1u << (q & 1);
            }
        }
        fft_any<T, E, 1, NL, 1>(pl, v, psm, 1, t, tw);
        if constexpr (OP == ZOP_C2R || OP == ZOP_DISP) {
            if (valid) {
                T *dst = bat<T>(a.out[f], bo) + row * a.rp_out;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const int n = nout_any<NL, E>(pl, t, e);
                    *reinterpret_cast<cplx<T> *>(dst + 2 * n) = cscale<T>(v[e], scale);
                }
                if (t == 0 && a.rp_out > N) { dst[N] = 0; dst[N + 1] = 0; }
            }
        } else if constexpr (S2) {
#pragma unroll
            for (int e = 0; e < E; e++) {
                const cplx<T> x = cscale<T>(v[e], scale);
                if (q == 0) o[0][e] = x;  // xx
                else if (q == 1) o[1][e] = x;  // yy
                else if (q == 2) {  // zz: zz yy + zz xx + yy xx
                    acc[e] = mk<T>(x.x * o[1][e].x + x.x * o[0][e].x + o[1][e].x * o[0][e].x,
                                   x.y * o[1][e].y + x.y * o[0][e].y + o[1][e].y * o[0][e].y);
                } else {  // - xy^2, - yz^2, - xz^2
                    acc[e] = mk<T>(acc[e].x - x.x * x.x, acc[e].y - x.y * x.y);
                }
            }
        } else if constexpr (LEAN) {
#pragma unroll
            for (int e = 0; e < E; e++) {
                const cplx<T> x = cscale<T>(v[e], scale);
                ma_lean_step<T>(q, x.x, o[0][e].x, o[1][e].x, o[2][e].x, acc[e].x);
                ma_lean_step<T>(q, x.y, o[0][e].y, o[1][e].y, o[2][e].y, acc[e].y);
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; e++) o[f][e] = v[e];
        }
    }
    (void)dst_row;
    if constexpr (ZT) {
        // after a timed-out wait: the copies still in flight land (bounded) before the block's
        // shared memory is released
        if (!zok) {
            for (int b = 0; b < 2; b++)
                if ((zpend >> b) & 1u) mbar_wait(zbar + b, (zph >> b) & 1u);
        }
    }
    if constexpr (OP == ZOP_HESS_2LPT_K) {
        // the r2c of the S row, as k_z_r2c does it from global memory: the row to the transform's
        // input order through the row's exchange buffer, the N/2-point forward FFT, the split into
        // N/2+1 modes.  Every thread takes part (the exchanges synchronise); invalid rows store nothing.
#pragma unroll
        for (int e = 0; e < E; e++) psm[xpos<NL, 1>(nout_any<NL, E>(pl, t, e))] = acc[e];
        if constexpr (NL > 0) pencil_sync<NL, E, 1>();
        else __syncthreads();
        cplx<T> v[E];
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = psm[xpos<NL, 1>(nin_any<NL, E>(pl, t, e))];
        if constexpr (NL > 0) pencil_sync<NL, E, 1>();
        else __syncthreads();
        fft_any<T, E, -1, NL, 1>(pl, v, psm, 1, t, tw);
#pragma unroll
        for (int e = 0; e < E; e++) psm[xpos<NL, 1>(nout_any<NL, E>(pl, t, e))] = v[e];
        if constexpr (NL > 0) pencil_sync<NL, E, 1>();
        else __syncthreads();
        if (a.zero) {
            // this block's slice of the region to clear (the deposit's density grid; under 2^31
            // 16-byte words), streaming stores
            const unsigned n16 = (unsigned)(a.zero_bytes / 16), nb = gridDim.x * gridDim.y;
            const unsigned per = (n16 + nb - 1) / nb, b0 = (blockIdx.y * gridDim.x + blockIdx.x) * per;
            const unsigned b1 = min(b0 + per, n16);
            uint4 *z = reinterpret_cast<uint4 *>(a.zero);
            for (unsigned i = b0 + threadIdx.x; i < b1; i += blockDim.x) __stcs(z + i, make_uint4(0u, 0u, 0u, 0u));
        }
        if (!valid) return;
        cplx<T> *dst = bat<cplx<T>>(a.out[0], bo) + row * H;
        for (int k = t; k <= h; k += tpp) {
            const cplx<T> Z = psm[xpos<NL, 1>(k == h ? 0 : k)];
            const cplx<T> Zc = psm[xpos<NL, 1>(k == 0 ? 0 : h - k)];
            const cplx<T> ev = mk<T>((T)0.5 * (Z.x + Zc.x), (T)0.5 * (Z.y - Zc.y));
            const cplx<T> od = mk<T>((T)0.5 * (Z.y + Zc.y), (T)-0.5 * (Z.x - Zc.x));
            const cplx<T> w = __ldg(tw + k);
            dst[k] = cadd<T>(ev, cmul<T>(od, w));
        }
        return;
    }
    // (the residual passes keep every thread to the end: their reductions and exchanges need the
    // whole warp and block)
    if (!valid && !MA) return;
    if constexpr (OP == ZOP_HESS_2LPT) {
        T *dst = bat<T>(a.out[0], bo) + row * a.rp_out;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int n = nout_any<NL, E>(pl, t, e);
            *reinterpret_cast<cplx<T> *>(dst + 2 * n) = acc[e];
        }
        if (t == 0 && a.rp_out > N) { dst[N] = 0; dst[N + 1] = 0; }
        return;
    }
    if constexpr (MA) {
        // the residual per element (valid rows: the FP64 sums; invalid rows compute on row 0 and
        // add nothing), stored, or kept for the r2c of ZOP_HESS_MA_K
        T *dst = bat<T>(a.out[0], bo) + row * a.rp_out;
        double sres = 0, srho = 0;
        const T *rho = bat<const T>(a.in2, bo) + row * a.rp_in;
        cplx<T> resv[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int n = nout_any<NL, E>(pl, t, e);
            T res2[2], s2v[2];
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if constexpr (LEAN) {
                    const T r = rho[2 * n + c];
                    const T res = r + (c ? acc[e].y : acc[e].x);
                    res2[c] = res;
                    s2v[c] = 0;
                    sres += (double)res * (double)res;
                    srho += (double)r * (double)r;
                    continue;
                }
                const T xx = (c ? o[0][e].y : o[0][e].x) * scale;
                const T xy = (c ? o[1][e].y : o[1][e].x) * scale;
                const T xz = (c ? o[2][e].y : o[2][e].x) * scale;
                const T yy = (c ? o[3][e].y : o[3][e].x) * scale;
                const T yz = (c ? o[4][e].y : o[4][e].x) * scale;
                const T zz = (c ? o[5][e].y : o[5][e].x) * scale;
                // second invariant of the Hessian (src/2lpt.c:111-112)
                const T s2 = zz * yy + zz * xx + yy * xx - xy * xy - yz * yz - xz * xz;
                s2v[c] = s2;
                // (1 + rho) - det(I + H) = (rho - tr H) - s2 - det H  (src/monge_ampere.c:119-145)
                const T d3 = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
                const T r = rho[2 * n + c];
                const T res = ((r - xx) - yy - zz) - s2 - d3;
                res2[c] = res;
                sres += (double)res * (double)res;
                srho += (double)r * (double)r;
            }
            resv[e] = mk<T>(res2[0], res2[1]);
            if constexpr (OP == ZOP_HESS_MA) {
                if (valid) *reinterpret_cast<cplx<T> *>(dst + 2 * n) = resv[e];
            }
            // optional second output: the second-order source S of the same Hessian
            if (!LEAN && valid && a.out[1])
                *reinterpret_cast<cplx<T> *>(bat<T>(a.out[1], bo) + row * a.rp_out + 2 * n) = mk<T>(s2v[0], s2v[1]);
        }
        if constexpr (OP == ZOP_HESS_MA) {
            if (valid && t == 0 && a.rp_out > N) { dst[N] = 0; dst[N + 1] = 0; }
        }
        if (!valid) { sres = 0; srho = 0; }
        for (int off = 16; off > 0; off >>= 1) {
            sres += __shfl_down_sync(0xffffffffu, sres, off);
            srho += __shfl_down_sync(0xffffffffu, srho, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(a.red + (size_t)blockIdx.y * a.acc_stride + 0, sres);
            atomicAdd(a.red + (size_t)blockIdx.y * a.acc_stride + 1, srho);
        }
        if constexpr (MAK) {
            // the residual row's r2c along z (as in ZOP_HESS_2LPT_K)
#pragma unroll
            for (int e = 0; e < E; e++) psm[xpos<NL, 1>(nout_any<NL, E>(pl, t, e))] = resv[e];
            if constexpr (NL > 0) pencil_sync<NL, E, 1>();
            else __syncthreads();
            cplx<T> v[E];
#pragma unroll
            for (int e = 0; e < E; e++) v[e] = psm[xpos<NL, 1>(nin_any<NL, E>(pl, t, e))];
            if constexpr (NL > 0) pencil_sync<NL, E, 1>();
            else __syncthreads();
            fft_any<T, E, -1, NL, 1>(pl, v, psm, 1, t, tw);
#pragma unroll
            for (int e = 0; e < E; e++) psm[xpos<NL, 1>(nout_any<NL, E>(pl, t, e))] = v[e];
            if constexpr (NL > 0) pencil_sync<NL, E, 1>();
            else __syncthreads();
            if (!valid) return;
            cplx<T> *dk_row = bat<cplx<T>>(a.out[0], bo) + row * H;
            for (int k = t; k <= h; k += tpp) {
                const cplx<T> Z = psm[xpos<NL, 1>(k == h ? 0 : k)];
                const cplx<T> Zc = psm[xpos<NL, 1>(k == 0 ? 0 : h - k)];
                const cplx<T> ev = mk<T>((T)0.5 * (Z.x + Zc.x), (T)0.5 * (Z.y - Zc.y));
                const cplx<T> od = mk<T>((T)0.5 * (Z.y + Zc.y), (T)-0.5 * (Z.x - Zc.x));
                const cplx<T> w = __ldg(tw + k);
                dk_row[k] = cadd<T>(ev, cmul<T>(od, w));
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Z r2c: N reals -> N/2+1 complex via an N/2-point forward FFT and the split step.
// ------------------------------------------------------------------------------------------
template <typename T, int E, int NL>
__global__ void __launch_bounds__(256) k_z_r2c(GridGeom g, PassArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smraw);
    const FFTPlan &pl = g.plH;
    const int h = pl.n, N = g.N, H = g.H;
    const int tpp = h / E;
    const int tid = threadIdx.x, t = tid % tpp, p = tid / tpp;
    long row = (long)blockIdx.x * g.P_z + p;
    const bool valid = row < (long)N * N;
    if (!valid) row = 0;
    const cplx<T> *tw = reinterpret_cast<const cplx<T> *>(g.twN);
    cplx<T> *psm = sm + (long)p * spad_len(h);
    const T ra = parg<T>(a.rho_a, a.frho_a), rb = parg<T>(a.rho_b, a.frho_b);
    const size_t bo = (size_t)blockIdx.y * (size_t)a.bstride;
    const T *src = bat<const T>(a.in[0], bo) + row * a.rp_in;
    cplx<T> v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int n = nin_any<NL, E>(pl, t, e);
        cplx<T> z = *reinterpret_cast<const cplx<T> *>(src + 2 * n);
        if (ra != (T)1 || rb != (T)0) z = mk<T>(z.x * ra + rb, z.y * ra + rb);
        v[e] = z;
    }
    fft_any<T, E, -1, NL, 1>(pl, v, psm, 1, t, tw);
#pragma unroll
    for (int e = 0; e < E; e++) psm[xpos<NL, 1>(nout_any<NL, E>(pl, t, e))] = v[e];
    if constexpr (NL > 0) pencil_sync<NL, E, 1>();
    else __syncthreads();
    if (!valid) return;
    cplx<T> *dst = bat<cplx<T>>(a.out[0], bo) + row * H;
    for (int k = t; k <= h; k += tpp) {
        const cplx<T> Z = psm[xpos<NL, 1>(k == h ? 0 : k)];
        const cplx<T> Zc = psm[xpos<NL, 1>(k == 0 ? 0 : h - k)];
        // even = (Z + conj Zc)/2, odd = (Z - conj Zc)/(2i), X = even + e^{-2 pi i k/N} odd
        const cplx<T> ev = mk<T>((T)0.5 * (Z.x + Zc.x), (T)0.5 * (Z.y - Zc.y));
        const cplx<T> od = mk<T>((T)0.5 * (Z.y + Zc.y), (T)-0.5 * (Z.x - Zc.x));
        const cplx<T> w = __ldg(tw + k);
        dst[k] = cadd<T>(ev, cmul<T>(od, w));
    }
}

// ------------------------------------------------------------------------------------------
// launchers (NL = 0: runtime plan; NL > 0: the compile-time specialisation for that length)
// ------------------------------------------------------------------------------------------

template <typename T, int E, int SIGN, int AXIS, int OP, int NL, int PC>
static int launch_strided_e(const GridGeom &g, const PassArgs &a, const T *win) {
    const int P = PC > 0 ? PC : g.P_xy;
    const int threads = P * (g.N / E);
    size_t smem = (size_t)P * spad_len(g.N) * sizeof(cplx<T>);
    if (OP == XOP_PK && AXIS == 0) smem += (size_t)a.nbins * (threads / 32) * sizeof(T);
    if ((OP == XOP_COMBINE_2LPT || OP == XOP_ADD_POISSON) && AXIS == 0) smem += (size_t)threads * E * sizeof(cplx<T>);
    long blocks = (AXIS == 0) ? (g.plane + P - 1) / P : (long)g.N * ((g.H + P - 1) / P);
    auto kern = k_strided<T, E, SIGN, AXIS, OP, NL, PC>;
    if (smem > 48 * 1024) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch_begin(AXIS == 0 ? (OP == XOP_HESS ? "x_hess" : OP == XOP_DISP ? "x_disp" : OP == XOP_COMBINE_2LPT ? "x_combine" : OP == XOP_ADD_POISSON ? "x_add_poisson" : OP == XOP_PK ? "x_pk" : "x_plain")
                        : (OP == YOP_HESS_A ? "y_hess_a" : OP == YOP_HESS_B ? "y_hess_b" : OP == YOP_DISP_A ? "y_disp_a" : OP == YOP_STN ? "y_stn" : "y_plain"));
    kern<<<dim3((unsigned)blocks, a.batch > 1 ? a.batch : 1), threads, smem, stream()>>>(g, with_f32(a), win);
    count_launch();
    MITOS_LAUNCH_CHECK("strided FFT pass");
    return 0;
}

// Elements a thread of the compile-time passes: 8 for 2^k, 12 for 3 2^k, and 16 for the 256-, 512-
// and 1024-point Y passes and Hessian and P(k) X passes and the 1024-point combine X pass.  Those keep
// the block's threads with twice the pencils (sixteen or eight in 512 threads, eight or four in the
// 256-thread multi-output Y passes): row segments twice as long, half the requests for each plane
// the block touches.  At 512^3: y_hess_a 0.72 -> 0.55 ms, x_hess 0.71 -> 0.62, y_hess_b and
// y_disp_a 0.44 -> 0.39, x_pk 0.43 -> 0.40, y_plain 0.25 -> 0.23; the 512-point combine pass stays
// at 8 (0.75 against 0.86 ms: its phi_1 staging makes a 16-element block one an SM).  At 256^3
// (where the rows are already 64 or 128 bytes) the IC 1.208 -> 1.187 ms, a Monge-Ampere solve
// 2.758 -> 2.699 ms.
template <int NL, int AXIS, int OP> constexpr int ct_elems() {
    return NL % 3 == 0 ? 12
           : ((NL == 256 || NL == 512 || NL == 1024) && (AXIS == 1 || OP == XOP_HESS || OP == XOP_PK)) ? 16
           : (NL == 1024 && OP == XOP_COMBINE_DISP) ? 16 : 8;
}
// pencils a block for ct_elems (PC: the pencils of the length's default elements)
template <int NL, int AXIS, int OP, int PC> constexpr int ct_pencils() {
    return PC * ct_elems<NL, AXIS, OP>() / (NL % 3 == 0 ? 12 : 8);
}

template <typename T, int SIGN, int AXIS, int OP, int NL, int PC>
static int launch_strided(const GridGeom &g, const PassArgs &a, const T *win) {
    if constexpr (NL > 0)
        return launch_strided_e<T, ct_elems<NL, AXIS, OP>(), SIGN, AXIS, OP, NL, ct_pencils<NL, AXIS, OP, PC>()>(g, a, win);
    else {
        if (g.E == 8) return launch_strided_e<T, 8, SIGN, AXIS, OP, 0, 0>(g, a, win);
        return launch_strided_e<T, 12, SIGN, AXIS, OP, 0, 0>(g, a, win);
    }
}

template <typename T, int E, int NL, int PC>
static int launch_combine_disp(const GridGeom &g, const PassArgs &a, const T *win) {
    const int P = PC > 0 ? PC : g.P_xy;
    const int threads = P * (g.N / E);
    // the exchange buffer, then phi_1's elements of every thread
    const size_t smem = (size_t)P * spad_len(g.N) * sizeof(cplx<T>) + (size_t)threads * E * sizeof(cplx<T>);
    const long blocks = (g.plane + P - 1) / P;
    launch_begin("x_combine_disp");
    auto kern = k_x_combine_disp<T, E, NL, PC>;
    if (smem > 48 * 1024) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<dim3((unsigned)blocks, a.batch > 1 ? a.batch : 1), threads, smem, stream()>>>(g, with_f32(a), win);
    count_launch();
    MITOS_LAUNCH_CHECK("x combine + displacement pass");
    return 0;
}

// pencils per block of the multi-output Y passes of the compile-time lengths (256 threads)
template <int NL, int PC> constexpr int pc_heavy() { return NL > 0 ? PC / 2 : PC; }

template <typename T, int NL, int PC>
int launch_x_t(const GridGeom &g, XOp op, int sign, const PassArgs &a) {
    const int prec = sizeof(T) == 4 ? MITOS_FP32 : MITOS_FP64;
    const T *win = a.window_order ? (const T *)window_table(g.N, a.window_order, prec) : nullptr;
    if (a.window_order && !win) return 5;
    switch (op) {
    case XOP_PLAIN:
        return sign < 0 ? launch_strided<T, -1, 0, XOP_PLAIN, NL, PC>(g, a, win) : launch_strided<T, 1, 0, XOP_PLAIN, NL, PC>(g, a, win);
    case XOP_HESS: return launch_strided<T, 1, 0, XOP_HESS, NL, PC>(g, a, win);
    case XOP_DISP: return launch_strided<T, 1, 0, XOP_DISP, NL, PC>(g, a, win);
    case XOP_COMBINE_2LPT: return launch_strided<T, -1, 0, XOP_COMBINE_2LPT, NL, PC>(g, a, win);
    case XOP_ADD_POISSON: return launch_strided<T, -1, 0, XOP_ADD_POISSON, NL, PC>(g, a, win);
    case XOP_PK: return launch_strided<T, -1, 0, XOP_PK, NL, PC>(g, a, win);
    case XOP_COMBINE_DISP:
        if constexpr (NL > 0)
            return launch_combine_disp<T, ct_elems<NL, 0, XOP_COMBINE_DISP>(), NL, ct_pencils<NL, 0, XOP_COMBINE_DISP, PC>()>(g, a, win);
        else if (g.E == 8) return launch_combine_disp<T, 8, 0, 0>(g, a, win);
        else return launch_combine_disp<T, 12, 0, 0>(g, a, win);
    }
    return 3;
}

template <typename T, int NL, int PC>
int launch_y_t(const GridGeom &g, YOp op, int sign, const PassArgs &a) {
    constexpr int PCH = pc_heavy<NL, PC>();
    switch (op) {
    case YOP_PLAIN:
        return sign < 0 ? launch_strided<T, -1, 1, YOP_PLAIN, NL, PC>(g, a, nullptr) : launch_strided<T, 1, 1, YOP_PLAIN, NL, PC>(g, a, nullptr);
    case YOP_DISP_A: return launch_strided<T, 1, 1, YOP_DISP_A, NL, PCH>(g, a, nullptr);
    case YOP_STN: return launch_strided<T, 1, 1, YOP_STN, NL, PC>(g, a, nullptr);
    case YOP_HESS_A: return launch_strided<T, 1, 1, YOP_HESS_A, NL, PCH>(g, a, nullptr);
    case YOP_HESS_B: return launch_strided<T, 1, 1, YOP_HESS_B, NL, PCH>(g, a, nullptr);
    }
    return 3;
}

template <typename T, int E, int OP, int NLZ>
static int launch_zc_e(const GridGeom &g, const PassArgs &a) {
    const int h = g.N / 2;
    const int tpp = h / E;
    int P = g.P_z;
    const int threads = P * tpp;
    size_t smem = (size_t)P * spad_len(h) * sizeof(cplx<T>);
    // the lean Monge-Ampere residual pass (FP32, compile-time lengths with one pencil a warp or half
    // a warp): two row buffers and two mbarriers a pencil behind the exchange buffer (k_z_c2r)
    constexpr bool ZT = sizeof(T) == 4 && OP == ZOP_HESS_MA_K && NLZ > 0 && (NLZ / E == 32 || NLZ / E == 16);
    PassArgs b = with_f32(a);
    if constexpr (ZT) {
        const size_t zrb = ((g.H * sizeof(cplx<T>) + 8 + 15) / 16) * 16;
        smem = ((smem + 15) & ~(size_t)15) + (size_t)P * 2 * zrb + (size_t)P * 2 * sizeof(uint64_t);
        if (!b.fault) b.fault = zrow_fault_device();
    }
    const long rows = (long)g.N * g.N;
    auto kern = k_z_c2r<T, E, OP, NLZ>;
    if (smem > 48 * 1024) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch_begin(OP == ZOP_C2R ? "z_c2r" : OP == ZOP_HESS_2LPT ? "z_hess_2lpt" : OP == ZOP_HESS_2LPT_K ? "z_hess_2lpt_r2c"
                 : OP == ZOP_HESS_MA ? "z_hess_ma" : OP == ZOP_HESS_MA_K ? "z_hess_ma_r2c"
                 : OP == ZOP_HESS_MA_KS ? "z_hess_ma_r2c_s" : "z_disp");
    kern<<<dim3((unsigned)((rows + P - 1) / P), a.batch > 1 ? a.batch : 1), threads, smem, stream()>>>(g, b);
    count_launch();
    MITOS_LAUNCH_CHECK("z c2r pass");
    return 0;
}

template <typename T, int NLZ>
int launch_zc_t(const GridGeom &g, ZOp op, const PassArgs &a) {
    constexpr int EC = (NLZ > 0 && NLZ % 3 == 0) ? 12 : 8;  // the compile-time lengths' elements
    if (NLZ > 0 || g.E == 8) {
        switch (op) {
        case ZOP_C2R: return launch_zc_e<T, EC, ZOP_C2R, NLZ>(g, a);
        case ZOP_HESS_2LPT: return launch_zc_e<T, EC, ZOP_HESS_2LPT, NLZ>(g, a);
        case ZOP_HESS_MA: return launch_zc_e<T, EC, ZOP_HESS_MA, NLZ>(g, a);
        case ZOP_DISP: return launch_zc_e<T, EC, ZOP_DISP, NLZ>(g, a);
        case ZOP_HESS_2LPT_K: return launch_zc_e<T, EC, ZOP_HESS_2LPT_K, NLZ>(g, a);
        case ZOP_HESS_MA_K: return launch_zc_e<T, EC, ZOP_HESS_MA_K, NLZ>(g, a);
        case ZOP_HESS_MA_KS: return launch_zc_e<T, EC, ZOP_HESS_MA_KS, NLZ>(g, a);
        }
    } else {
        switch (op) {
        case ZOP_C2R: return launch_zc_e<T, 12, ZOP_C2R, 0>(g, a);
        case ZOP_HESS_2LPT: return launch_zc_e<T, 12, ZOP_HESS_2LPT, 0>(g, a);
        case ZOP_HESS_MA: return launch_zc_e<T, 12, ZOP_HESS_MA, 0>(g, a);
        case ZOP_DISP: return launch_zc_e<T, 12, ZOP_DISP, 0>(g, a);
        case ZOP_HESS_2LPT_K: return launch_zc_e<T, 12, ZOP_HESS_2LPT_K, 0>(g, a);
        case ZOP_HESS_MA_K: return launch_zc_e<T, 12, ZOP_HESS_MA_K, 0>(g, a);
        case ZOP_HESS_MA_KS: return launch_zc_e<T, 12, ZOP_HESS_MA_KS, 0>(g, a);
        }
    }
    return 3;
}

template <typename T, int E, int NLZ>
static int launch_zr_e(const GridGeom &g, const PassArgs &a) {
    const int h = g.N / 2;
    const int tpp = h / E;
    const int P = g.P_z;
    const size_t smem = (size_t)P * spad_len(h) * sizeof(cplx<T>);
    const long rows = (long)g.N * g.N;
    auto kern = k_z_r2c<T, E, NLZ>;
    if (smem > 48 * 1024) MITOS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch_begin("z_r2c");
    kern<<<dim3((unsigned)((rows + P - 1) / P), a.batch > 1 ? a.batch : 1), P * tpp, smem, stream()>>>(g, with_f32(a));
    count_launch();
    MITOS_LAUNCH_CHECK("z r2c pass");
    return 0;
}

template <typename T, int NLZ>
int launch_zr_t(const GridGeom &g, const PassArgs &a) {
    if (NLZ > 0 || g.E == 8) return launch_zr_e<T, (NLZ > 0 && NLZ % 3 == 0 ? 12 : 8), NLZ>(g, a);
    return launch_zr_e<T, 12, 0>(g, a);
}

}  // namespace mitos
