// fft_core.cuh -- register-resident mixed-radix Stockham FFT over pencils held by thread groups.
//
// A pencil of length n is transformed by n/E threads; each thread owns E complex values.
// Stage s applies radix R_s (R_s divides E) to the thread's E/R_s butterflies.  The first
// stage works on values the caller loaded from global memory (so loads can be fused with
// k-space factors and coalesced), the last stage leaves the results in registers (so stores
// can be fused with epilogues); the stages in between exchange through shared memory.
//
// Index maps (t = thread index inside the pencil, j_b = t + b * (n / E)):
//   input  element e = b * R_first + r  holds x[j_b + r * (n / R_first)]
//   output element e = b * R_last  + r  holds X[j_b + r * (n / R_last)]
// The stage arithmetic is the Stockham autosort formulation: a butterfly j of a stage with
// radix R and current length Ns reads x[j + r n/R] * w^(r (j mod Ns) n/(Ns R)) and writes
// X[(j / Ns) Ns R + (j mod Ns) + r Ns].
#pragma once

#include "common.cuh"

namespace mitos {

#define MITOS_MAX_STAGES 12

struct FFTPlan {
    int n;                         // transform length
    int nst;                       // number of stages
    int rad[MITOS_MAX_STAGES];     // radices, first to last
    int tw_scale;                  // twiddle table length / n
    int lgNs[MITOS_MAX_STAGES];    // log2 of the combined length before stage s, -1 if not 2^k
    int twstep[MITOS_MAX_STAGES];  // n / (Ns R) * tw_scale: table stride of stage s
};

// j / Ns and j % Ns, by shifts when Ns is a power of two
__device__ __forceinline__ void divmod_ns(int j, int Ns, int lg, int &q, int &r) {
    if (lg >= 0) {
        q = j >> lg;
        r = j & (Ns - 1);
    } else {
        q = j / Ns;
        r = j - q * Ns;
    }
}

// unnormalised R-point DFT in registers; SIGN = -1 forward, +1 backward
template <typename T, int SIGN> __device__ __forceinline__ void dft2(cplx<T> &a, cplx<T> &b) {
    cplx<T> t = a;
    a = cadd<T>(t, b);
    b = csub<T>(t, b);
}

// multiply by -i (SIGN = -1) or +i (SIGN = +1)
template <typename T, int SIGN> __device__ __forceinline__ cplx<T> rot90(cplx<T> a) {
    return SIGN < 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}

template <typename T, int SIGN> __device__ __forceinline__ void dft4(cplx<T> *v) {
    cplx<T> a0 = cadd<T>(v[0], v[2]), a1 = csub<T>(v[0], v[2]);
    cplx<T> b0 = cadd<T>(v[1], v[3]), b1 = rot90<T, SIGN>(csub<T>(v[1], v[3]));
    v[0] = cadd<T>(a0, b0);
    v[2] = csub<T>(a0, b0);
    v[1] = cadd<T>(a1, b1);
    v[3] = csub<T>(a1, b1);
}

template <typename T, int SIGN> __device__ __forceinline__ void dft8(cplx<T> *v) {
    const T h = (T)0.70710678118654752440084436210485;
    cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
    cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<T, SIGN>(e);
    dft4<T, SIGN>(o);
    // w8^k = exp(SIGN 2 pi i k / 8)
    cplx<T> o1 = mk<T>((o[1].x - SIGN * o[1].y) * h, (o[1].y + SIGN * o[1].x) * h);
    cplx<T> o2 = rot90<T, SIGN>(o[2]);  // w8^2 = SIGN i
    cplx<T> o3 = mk<T>((-o[3].x - SIGN * o[3].y) * h, (-o[3].y + SIGN * o[3].x) * h);
    v[0] = cadd<T>(e[0], o[0]);
    v[4] = csub<T>(e[0], o[0]);
    v[1] = cadd<T>(e[1], o1);
    v[5] = csub<T>(e[1], o1);
    v[2] = cadd<T>(e[2], o2);
    v[6] = csub<T>(e[2], o2);
    v[3] = cadd<T>(e[3], o3);
    v[7] = csub<T>(e[3], o3);
}

template <typename T, int SIGN> __device__ __forceinline__ void dft3(cplx<T> *v) {
    const T c = (T)-0.5;
    const T s = (T)(SIGN) * (T)0.86602540378443864676372317075294;
    cplx<T> t1 = cadd<T>(v[1], v[2]);
    cplx<T> t2 = csub<T>(v[1], v[2]);
    cplx<T> m = mk<T>(v[0].x + c * t1.x, v[0].y + c * t1.y);
    v[0] = cadd<T>(v[0], t1);
    // i s t2 = (-s t2.y, s t2.x)
    v[1] = mk<T>(m.x - s * t2.y, m.y + s * t2.x);
    v[2] = mk<T>(m.x + s * t2.y, m.y - s * t2.x);
}

template <typename T, int R, int SIGN> __device__ __forceinline__ void dft(cplx<T> *v) {
    if constexpr (R == 2) dft2<T, SIGN>(v[0], v[1]);
    else if constexpr (R == 3) dft3<T, SIGN>(v);
    else if constexpr (R == 4) dft4<T, SIGN>(v);
    else if constexpr (R == 8) dft8<T, SIGN>(v);
}

// padded shared-memory index of element n (one pad slot every 8) to spread bank accesses
__device__ __forceinline__ int spad(int n) { return n + (n >> 3); }
__host__ __device__ __forceinline__ int spad_len(int n) { return n + (n >> 3) + 1; }

// first stage: DFT of each butterfly group in registers (twiddles are all one)
template <typename T, int E, int R, int SIGN>
__device__ __forceinline__ void stage_first(cplx<T> *v) {
#pragma unroll
    for (int b = 0; b < E / R; b++) dft<T, R, SIGN>(v + b * R);
}

// write stage outputs to shared memory (layout: element n of pencil at sm[spad(n)*sn])
template <typename T, int E, int R>
__device__ __forceinline__ void stage_write(const cplx<T> *v, cplx<T> *sm, int sn, int n, int t,
                                            int Ns, int lg) {
#pragma unroll
    for (int b = 0; b < E / R; b++) {
        int j = t + b * (n / E);
        int jd, jm;
        divmod_ns(j, Ns, lg, jd, jm);
        int idxD = jd * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) sm[spad(idxD + r * Ns) * sn] = v[b * R + r];
    }
}

// read stage inputs from shared memory, apply twiddles and the radix-R DFT
template <typename T, int E, int R, int SIGN>
__device__ __forceinline__ void stage_read_dft(cplx<T> *v, const cplx<T> *sm, int sn, int n, int t,
                                               int Ns, int lg, const cplx<T> *__restrict__ tw,
                                               int twstep) {
#pragma unroll
    for (int b = 0; b < E / R; b++) {
        int j = t + b * (n / E);
        int jd, jm;
        divmod_ns(j, Ns, lg, jd, jm);
        int step = jm * twstep;
#pragma unroll
        for (int r = 0; r < R; r++) {
            cplx<T> x = sm[spad(j + r * (n / R)) * sn];
            if (r > 0) {
                cplx<T> w = __ldg(tw + r * step);
                if (SIGN > 0) w.y = -w.y;
                x = cmul<T>(x, w);
            }
            v[b * R + r] = x;
        }
        dft<T, R, SIGN>(v + b * R);
    }
}

template <typename T, int E, int SIGN>
__device__ __forceinline__ void first_dispatch(int R, cplx<T> *v) {
    if constexpr (E % 8 == 0) { if (R == 8) { stage_first<T, E, 8, SIGN>(v); return; } }
    if constexpr (E % 4 == 0) { if (R == 4) { stage_first<T, E, 4, SIGN>(v); return; } }
    if constexpr (E % 3 == 0) { if (R == 3) { stage_first<T, E, 3, SIGN>(v); return; } }
    if constexpr (E % 2 == 0) { if (R == 2) { stage_first<T, E, 2, SIGN>(v); return; } }
}

template <typename T, int E>
__device__ __forceinline__ void write_dispatch(int R, const cplx<T> *v, cplx<T> *sm, int sn, int n,
                                               int t, int Ns, int lg) {
    if constexpr (E % 8 == 0) { if (R == 8) { stage_write<T, E, 8>(v, sm, sn, n, t, Ns, lg); return; } }
    if constexpr (E % 4 == 0) { if (R == 4) { stage_write<T, E, 4>(v, sm, sn, n, t, Ns, lg); return; } }
    if constexpr (E % 3 == 0) { if (R == 3) { stage_write<T, E, 3>(v, sm, sn, n, t, Ns, lg); return; } }
    if constexpr (E % 2 == 0) { if (R == 2) { stage_write<T, E, 2>(v, sm, sn, n, t, Ns, lg); return; } }
}

template <typename T, int E, int SIGN>
__device__ __forceinline__ void read_dispatch(int R, cplx<T> *v, const cplx<T> *sm, int sn, int n,
                                              int t, int Ns, int lg, const cplx<T> *tw, int tws) {
    if constexpr (E % 8 == 0) { if (R == 8) { stage_read_dft<T, E, 8, SIGN>(v, sm, sn, n, t, Ns, lg, tw, tws); return; } }
    if constexpr (E % 4 == 0) { if (R == 4) { stage_read_dft<T, E, 4, SIGN>(v, sm, sn, n, t, Ns, lg, tw, tws); return; } }
    if constexpr (E % 3 == 0) { if (R == 3) { stage_read_dft<T, E, 3, SIGN>(v, sm, sn, n, t, Ns, lg, tw, tws); return; } }
    if constexpr (E % 2 == 0) { if (R == 2) { stage_read_dft<T, E, 2, SIGN>(v, sm, sn, n, t, Ns, lg, tw, tws); return; } }
}

// Transform the pencils of a thread block.  v holds the stage-1 inputs on entry and the
// outputs on return (index maps above).  sm points at this pencil's shared memory slice,
// elements sn apart; the whole block must call this together (it synchronises).
template <typename T, int E, int SIGN>
__device__ __forceinline__ void fft_regs(const FFTPlan &pl, cplx<T> *v, cplx<T> *sm, int sn, int t,
                                         const cplx<T> *__restrict__ tw) {
    const int n = pl.n;
    first_dispatch<T, E, SIGN>(pl.rad[0], v);
    int Ns = pl.rad[0];
    int Nsp = 1;
    for (int s = 1; s < pl.nst; s++) {
        write_dispatch<T, E>(pl.rad[s - 1], v, sm, sn, n, t, Nsp, pl.lgNs[s - 1]);
        __syncthreads();
        read_dispatch<T, E, SIGN>(pl.rad[s], v, sm, sn, n, t, Ns, pl.lgNs[s], tw, pl.twstep[s]);
        __syncthreads();
        Nsp = Ns;
        Ns *= pl.rad[s];
    }
}

// element index maps
__device__ __forceinline__ int n_in(const FFTPlan &pl, int E, int t, int e) {
    int R = pl.rad[0];
    int b = e / R, r = e % R;
    return t + b * (pl.n / E) + r * (pl.n / R);
}
__device__ __forceinline__ int n_out(const FFTPlan &pl, int E, int t, int e) {
    int R = pl.rad[pl.nst - 1];
    int b = e / R, r = e % R;
    return t + b * (pl.n / E) + r * (pl.n / R);
}

// host: radix schedule of a length for a given E (radices dividing E, largest first)
bool make_plan(int n, int E, int tw_len, FFTPlan *pl);

}  // namespace mitos
