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
    // the compile-time kernels' twiddles (the default schedule), stage by stage: for each stage
    // s >= 1, Ns rows (jm < Ns) of w^(r jm n / (Ns R)), r = 1 .. R-1, each row tw_row(R) entries
    // (16-byte aligned for vector loads); the same values as the table twN holds.  twst16: the
    // same for the schedule of the 16-element compile-time kernels (ct_radix_at(n, 16, s))
    const void *twst;
    const void *twst16;
};

// entries of a stage's twiddle row (R - 1 used)
__host__ __device__ constexpr int tw_row(int R) { return R - 1 <= 2 ? 2 : (R - 1 <= 4 ? 4 : (R - 1 <= 8 ? 8 : 16)); }

// Radix of stage s of the compile-time schedule of length NL at E elements a thread (0 past the
// last stage): 8s, 4s, 2s, 3s, after 16s for the 256-point 16-element kernels ([16, 16]: one
// exchange instead of two; 256^3 IC 1.191 -> 1.151 ms, Monge-Ampere solve 2.645 -> 2.544 ms).  At
// 512 ([16, 16, 2] against [8, 8, 8]) the IC took 8.01 -> 8.14 ms and at 1024 ([16, 16, 4]) 74.15 ->
// 73.92, so those keep 8s.
__host__ __device__ constexpr bool ct_r16(int NL) { return NL == 256; }
__host__ __device__ constexpr int ct_radix_at(int NL, int E, int s) {
    int rem = NL, idx = 0;
    if (E % 16 == 0 && ct_r16(NL))
        while (rem % 16 == 0) { if (idx == s) return 16; rem /= 16; idx++; }
    if (E % 8 == 0)
        while (rem % 8 == 0) { if (idx == s) return 8; rem /= 8; idx++; }
    while (E % 4 == 0 && rem % 4 == 0) { if (idx == s) return 4; rem /= 4; idx++; }
    while (E % 2 == 0 && rem % 2 == 0) { if (idx == s) return 2; rem /= 2; idx++; }
    while (E % 3 == 0 && rem % 3 == 0) { if (idx == s) return 3; rem /= 3; idx++; }
    return 0;
}

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

// a + rot90(b) and a - rot90(b) lane by lane: the rotation swaps the lanes, so a packed pair
// operation would first have to move them
template <typename T, int SIGN> __device__ __forceinline__ cplx<T> add_rot(cplx<T> a, cplx<T> b) {
    return SIGN < 0 ? mk<T>(a.x + b.y, a.y - b.x) : mk<T>(a.x - b.y, a.y + b.x);
}
template <typename T, int SIGN> __device__ __forceinline__ cplx<T> sub_rot(cplx<T> a, cplx<T> b) {
    return SIGN < 0 ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, a.y - b.x);
}

template <typename T, int SIGN> __device__ __forceinline__ void dft4(cplx<T> *v) {
    cplx<T> a0 = cadd<T>(v[0], v[2]), a1 = csub<T>(v[0], v[2]);
    cplx<T> b0 = cadd<T>(v[1], v[3]), d = csub<T>(v[1], v[3]);
    v[0] = cadd<T>(a0, b0);
    v[2] = csub<T>(a0, b0);
    v[1] = add_rot<T, SIGN>(a1, d);
    v[3] = sub_rot<T, SIGN>(a1, d);
}

template <typename T, int SIGN> __device__ __forceinline__ void dft8(cplx<T> *v) {
    const T h = (T)0.70710678118654752440084436210485;
    cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
    cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<T, SIGN>(e);
    dft4<T, SIGN>(o);
    // w8^k = exp(SIGN 2 pi i k / 8)
    cplx<T> o1 = mk<T>((o[1].x - SIGN * o[1].y) * h, (o[1].y + SIGN * o[1].x) * h);
    cplx<T> o3 = mk<T>((-o[3].x - SIGN * o[3].y) * h, (-o[3].y + SIGN * o[3].x) * h);
    v[0] = cadd<T>(e[0], o[0]);
    v[4] = csub<T>(e[0], o[0]);
    v[1] = cadd<T>(e[1], o1);
    v[5] = csub<T>(e[1], o1);
    v[2] = add_rot<T, SIGN>(e[2], o[2]);  // w8^2 = SIGN i
    v[6] = sub_rot<T, SIGN>(e[2], o[2]);
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

// 16-point DFT as 4 x 4 (n = 4 n1 + n2, k = k1 + 4 k2): DFT4s over n1 for each n2, the twiddles
// w16^(n2 k1) with w16 = exp(SIGN 2 pi i / 16), DFT4s over n2 for each k1; natural order in and out
template <typename T, int SIGN> __device__ __forceinline__ void dft16(cplx<T> *v) {
    const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173, h = (T)0.70710678118654752440;
    const T S = (T)SIGN;
    cplx<T> y[16];  // y[4 n2 + k1]
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
        cplx<T> q[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
        dft4<T, SIGN>(q);
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) y[4 * n2 + k1] = q[k1];
    }
    y[5] = cmul<T>(y[5], mk<T>(c1, S * s1));     // w^1
    y[6] = cmul<T>(y[6], mk<T>(h, S * h));       // w^2
    y[7] = cmul<T>(y[7], mk<T>(s1, S * c1));     // w^3
    y[9] = cmul<T>(y[9], mk<T>(h, S * h));       // w^2
    y[10] = rot90<T, SIGN>(y[10]);               // w^4 = SIGN i
    y[11] = cmul<T>(y[11], mk<T>(-h, S * h));    // w^6
    y[13] = cmul<T>(y[13], mk<T>(s1, S * c1));   // w^3
    y[14] = cmul<T>(y[14], mk<T>(-h, S * h));    // w^6
    y[15] = cmul<T>(y[15], mk<T>(-c1, -S * s1)); // w^9
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        cplx<T> q[4] = {y[k1], y[4 + k1], y[8 + k1], y[12 + k1]};
        dft4<T, SIGN>(q);
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = q[k2];
    }
}

template <typename T, int R, int SIGN> __device__ __forceinline__ void dft(cplx<T> *v) {
    if constexpr (R == 2) dft2<T, SIGN>(v[0], v[1]);
    else if constexpr (R == 3) dft3<T, SIGN>(v);
    else if constexpr (R == 4) dft4<T, SIGN>(v);
    else if constexpr (R == 8) dft8<T, SIGN>(v);
    else if constexpr (R == 16) dft16<T, SIGN>(v);
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


// ---- compile-time specialisation (length NL, elements per thread E) ----------------------
// Same schedule and stage arithmetic as fft_regs with every length, radix and stride a
// constant, so shared-memory offsets and index splits fold away.
template <int NL, int E> struct CTSched {
    static constexpr int radix_at(int s) { return ct_radix_at(NL, E, s); }
    static constexpr int count() {
        int n = 0;
        while (radix_at(n)) n++;
        return n;
    }
    static constexpr int nst = count();
    static constexpr int ns_before(int s) {
        int p = 1;
        for (int i = 0; i < s; i++) p *= radix_at(i);
        return p;
    }
    static constexpr int first = radix_at(0);
    static constexpr int last = radix_at(nst - 1);
    // offset (entries) of stage s's rows in the stage twiddle table
    static constexpr int tw_off(int s) {
        int o = 0;
        for (int i = 1; i < s; i++) o += ns_before(i) * tw_row(radix_at(i));
        return o;
    }
};

// padded index of i + D from the padded index of i, when D is a multiple of 8 (or i + D stays
// inside one group of 8)
template <int D> __device__ __forceinline__ int spad_plus(int i, int si) {
    if constexpr (D % 8 == 0) return si + D + D / 8;
    else return spad(i + D);
}

// Exchange slot of element i of a pencil.  With pencils interleaved across the lanes (SN > 1)
// or a runtime length: the padded index i + i/8.  With one pencil per (half-)warp (SN == 1, the
// Z passes): an XOR swizzle of bits 0-3 by bits 3-6, under which the stage writes (stride Nsp)
// and the contiguous stage reads of 8-byte elements fill each half-warp's 128-byte wavefront
// without bank conflicts.
template <int NL, int SN> __device__ __forceinline__ int xpos(int i) {
    if constexpr (NL > 0 && SN == 1) return i ^ ((i >> 3) & 3) ^ (((i >> 5) & 3) << 2);
    else return spad(i);
}

// Barrier of a stage exchange.  A pencil held by one warp or half-warp (SN == 1: pencils are not
// interleaved across lanes) exchanges only within that warp: __syncwarp.  Otherwise the block's.
// (Blocks are whole warps: the tile setter rejects others.)
template <int NL, int E, int SN> constexpr bool warp_pencil() {
    return SN == 1 && NL / E <= 32 && 32 % (NL / E) == 0;
}
// A pencil of whole warps whose threads are contiguous (SN == 1, NL / E a multiple of 32: the Z
// passes of N = 1024, two warps a row) synchronises on a named barrier of its own warps, id 1 + its
// index in the block (the Z tiles hold at most 256 threads, so at most 4 such pencils).
template <int NL, int E, int SN> __device__ __forceinline__ void pencil_sync() {
    if constexpr (warp_pencil<NL, E, SN>()) {
        __syncwarp();
    } else if constexpr (NL > 0 && SN == 1 && (NL / E) % 32 == 0) {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)threadIdx.x / (NL / E)), "n"(NL / E) : "memory");
    } else {
        __syncthreads();
    }
}

template <typename T, int E, int SIGN, int NL, int SN, int S>
struct CTStage {
    using Sch = CTSched<NL, E>;
    static __device__ __forceinline__ void run(cplx<T> *v, cplx<T> *sm, int t, const cplx<T> *__restrict__ twst) {
        if constexpr (S < Sch::nst) {
            constexpr int Rp = Sch::radix_at(S - 1);
            constexpr int Nsp = Sch::ns_before(S - 1);
            constexpr int R = Sch::radix_at(S);
            constexpr int Ns = Sch::ns_before(S);
#pragma unroll
            for (int b = 0; b < E / Rp; b++) {
                const int j = t + b * (NL / E);
                const int idxD = (j / Nsp) * Nsp * Rp + (j % Nsp);
                if constexpr (SN == 1) {
#pragma unroll
                    for (int r = 0; r < Rp; r++) sm[xpos<NL, SN>(idxD + r * Nsp)] = v[b * Rp + r];
                } else if constexpr (Nsp == 1 && Rp <= 8) {
                    // idxD = j Rp and the Rp outputs stay in one padding group when Rp divides 8
                    const int base = spad(idxD);
#pragma unroll
                    for (int r = 0; r < Rp; r++)
                        sm[(8 % Rp == 0 ? base + r : spad(idxD + r)) * SN] = v[b * Rp + r];
                } else {
                    const int base = spad(idxD);
#pragma unroll
                    for (int r = 0; r < Rp; r++) {
                        const int o = (Nsp % 8 == 0) ? base + r * Nsp + (r * Nsp) / 8 : spad(idxD + r * Nsp);
                        sm[o * SN] = v[b * Rp + r];
                    }
                }
            }
            pencil_sync<NL, E, SN>();
#pragma unroll
            for (int b = 0; b < E / R; b++) {
                const int j = t + b * (NL / E);
                const int jm = j % Ns;
                const int base = spad(j);
                // the butterfly's R - 1 twiddles, one contiguous row: 16-byte vector loads
                constexpr int TR = tw_row(R);
                const cplx<T> *row = twst + Sch::tw_off(S) + jm * TR;
                cplx<T> tws[TR];
                if constexpr (sizeof(cplx<T>) == 8) {
#pragma unroll
                    for (int k = 0; k < TR / 2; k++) {
                        const float4 q = __ldg(reinterpret_cast<const float4 *>(row) + k);
                        tws[2 * k] = mk<T>(q.x, q.y);
                        tws[2 * k + 1] = mk<T>(q.z, q.w);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < R - 1; k++) tws[k] = __ldg(row + k);
                }
#pragma unroll
                for (int r = 0; r < R; r++) {
                    constexpr int D = NL / R;
                    const int o = (SN == 1) ? xpos<NL, SN>(j + r * D)
                                  : ((D % 8) == 0) ? base + r * D + (r * D) / 8 : spad(j + r * D);
                    cplx<T> x = sm[o * SN];
                    if (r > 0) {
                        cplx<T> w = tws[r - 1];
                        if (SIGN > 0) w.y = -w.y;
                        x = cmul<T>(x, w);
                    }
                    v[b * R + r] = x;
                }
                dft<T, R, SIGN>(v + b * R);
            }
            pencil_sync<NL, E, SN>();
            CTStage<T, E, SIGN, NL, SN, S + 1>::run(v, sm, t, twst);
        }
    }
};

// fft_regs with the length, the exchange stride SN and the schedule fixed at compile time; twst:
// the plan's stage twiddle table (FFTPlan::twst)
template <typename T, int E, int SIGN, int NL, int SN>
__device__ __forceinline__ void fft_regs_ct(cplx<T> *v, cplx<T> *sm, int t, const cplx<T> *__restrict__ twst) {
    stage_first<T, E, CTSched<NL, E>::first, SIGN>(v);
    CTStage<T, E, SIGN, NL, SN, 1>::run(v, sm, t, twst);
}

template <int NL, int E> __device__ __forceinline__ int n_in_ct(int t, int e) {
    constexpr int R = CTSched<NL, E>::first;
    return t + (e / R) * (NL / E) + (e % R) * (NL / R);
}
template <int NL, int E> __device__ __forceinline__ int n_out_ct(int t, int e) {
    constexpr int R = CTSched<NL, E>::last;
    return t + (e / R) * (NL / E) + (e % R) * (NL / R);
}

// one entry point for both variants: NL = 0 runs the runtime plan
template <typename T, int E, int SIGN, int NL, int SN>
__device__ __forceinline__ void fft_any(const FFTPlan &pl, cplx<T> *v, cplx<T> *sm, int sn, int t,
                                        const cplx<T> *__restrict__ tw) {
    if constexpr (NL > 0)
        fft_regs_ct<T, E, SIGN, NL, SN>(v, sm, t, reinterpret_cast<const cplx<T> *>(E == 16 ? pl.twst16 : pl.twst));
    else fft_regs<T, E, SIGN>(pl, v, sm, sn, t, tw);
}
template <int NL, int E> __device__ __forceinline__ int nin_any(const FFTPlan &pl, int t, int e) {
    if constexpr (NL > 0) return n_in_ct<NL, E>(t, e);
    else return n_in(pl, E, t, e);
}
template <int NL, int E> __device__ __forceinline__ int nout_any(const FFTPlan &pl, int t, int e) {
    if constexpr (NL > 0) return n_out_ct<NL, E>(t, e);
    else return n_out(pl, E, t, e);
}

// host: radix schedule of a length for a given E (radices dividing E, largest first)
bool make_plan(int n, int E, int tw_len, FFTPlan *pl);

}  // namespace mitos
