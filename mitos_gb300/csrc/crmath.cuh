// crmath.cuh -- correctly rounded FP64 log and cos for the white noise's Box-Muller transform
// (sampleNorm, src/random.c:34-49: sqrt(-2 log u) cos(2 pi v)), identical on the GPU and the host.
//
// Method: Ziv's two-step strategy (A. Ziv, "Fast evaluation of elementary mathematical functions
// with correctly rounded last bit", ACM TOMS 17(3), 1991).  A fast step evaluates the function in
// double-double arithmetic with a relative error below 2^-68 and returns its rounding when the
// error interval [r - eps, r + eps], eps = 2^-64 |r|, rounds to one double (all but ~2^-10 of the
// inputs); otherwise an accurate step evaluates it in triple-double arithmetic (relative error
// near 2^-140, far below the ~2^-118 that the hardest double-precision inputs of log and cos
// need) and rounds that exactly, resolving an exact tie of the leading parts by the sign of the
// last one.  The building blocks are the error-free transformations TwoSum (Knuth), Fast2Sum
// (Dekker) and TwoProd by FMA, with double-double and triple-double sums and products in the
// style of Dekker (1971) and Lauter's triple-double library (2005).  Each operation is an explicit
// round-to-nearest intrinsic on the device and an uncontracted operation on the host (the library
// is built with -ffp-contract=off), so both sides compute the same values.
//
// log(x), x > 0 finite: x = 2^K m / r_i (1 + z) with i the top 7 fraction bits of m in [1, 2),
// r_i an 8-bit approximation of the inverse of the interval's midpoint and z = m r_i - 1 exact
// (one FMA; |z| < 2^-7): log x = K ln 2 + L_i + log1p(z), L_i = -log r_i (or -log 2 r_i with K
// raised by one for m >= 1.414, so that x just below 1 has K = 0, L = 0 and no cancellation).
// log1p(z) is its Taylor series (through z^10 in the fast step, z^19 in the accurate one).
//
// cos(y), |y| < 8: y = k pi/2 + t with pi/2 in four parts (k P1, k P2, k P3 exact, so t has a
// relative error below 2^-140 even for the y closest to a multiple of pi/2); |t| = j/128 + b,
// |b| <= 1/256; sin and cos of b by their series and the table values sin(j/128), cos(j/128);
// cos y = cos t, -sin t, -cos t or sin t by k mod 4.
//
// The tables (crmath_tables.h) are the mathematical values evaluated with 400-bit arithmetic by
// gen_crmath_tables.py.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "crmath_tables.h"

#if defined(__CUDACC__)
#define CR_HD __host__ __device__ __forceinline__
#define CR_HD_COLD static __host__ __device__ __noinline__  // the rare accurate steps: out of line
#else
#define CR_HD static inline
#define CR_HD_COLD static
#endif

namespace crm {

#if defined(__CUDACC__)
// device copies (global memory, read through the data cache) and host copies of each table
static __device__ const double d_log_r[128] = CR_LOG_R_INIT;
static __device__ const double d_log_l[3 * 128] = CR_LOG_L_INIT;
static __device__ const double d_inv_n[3 * 24] = CR_INV_N_INIT;
static __device__ const double d_sincos[6 * CR_COS_NJ] = CR_SINCOS_INIT;
static __device__ const double d_inv_fact[3 * 17] = CR_INV_FACT_INIT;
#endif
static const double h_log_r[128] = CR_LOG_R_INIT;
static const double h_log_l[3 * 128] = CR_LOG_L_INIT;
static const double h_inv_n[3 * 24] = CR_INV_N_INIT;
static const double h_sincos[6 * CR_COS_NJ] = CR_SINCOS_INIT;
static const double h_inv_fact[3 * 17] = CR_INV_FACT_INIT;
#if defined(__CUDA_ARCH__)
#define CR_T(name) d_##name
#else
#define CR_T(name) h_##name
#endif

CR_HD uint64_t as_u64(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}
CR_HD double as_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

// ---- round-to-nearest operations, identical on both sides ----------------------------------
CR_HD double add(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CR_HD double sub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
CR_HD double mul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CR_HD double fmaf64(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

// ---- error-free transformations --------------------------------------------------------------
// s + e = a + b exactly
CR_HD void two_sum(double a, double b, double &s, double &e) {
    s = add(a, b);
    const double bb = sub(s, a);
    e = add(sub(a, sub(s, bb)), sub(b, bb));
}
// s + e = a + b exactly, for |a| >= |b| (or a == 0)
CR_HD void fast_two_sum(double a, double b, double &s, double &e) {
    s = add(a, b);
    e = sub(b, sub(s, a));
}
// p + e = a b exactly
CR_HD void two_prod(double a, double b, double &p, double &e) {
    p = mul(a, b);
    e = fmaf64(a, b, -p);
}

// ---- double-double ---------------------------------------------------------------------------
struct dd {
    double h, l;
};
CR_HD dd dd_add(dd a, dd b) {
    double s, e, t, f;
    two_sum(a.h, b.h, s, e);
    two_sum(a.l, b.l, t, f);
    e = add(e, t);
    fast_two_sum(s, e, s, e);
    e = add(e, f);
    fast_two_sum(s, e, s, e);
    return {s, e};
}
// the same when |a.h| >= |b.h| or a.h == 0 (Dekker's sum): about half the operations
CR_HD dd dd_add_fast(dd a, dd b) {
    double s, e;
    fast_two_sum(a.h, b.h, s, e);
    e = add(e, add(a.l, b.l));
    fast_two_sum(s, e, s, e);
    return {s, e};
}
CR_HD dd dd_mul(dd a, dd b) {
    double p, e;
    two_prod(a.h, b.h, p, e);
    e = fmaf64(a.h, b.l, e);
    e = fmaf64(a.l, b.h, e);
    fast_two_sum(p, e, p, e);
    return {p, e};
}

// ---- triple-double (x0 + x1 + x2, renormalised so that x0 = RN(x0 + x1)) ---------------------
struct td {
    double x0, x1, x2;
};
// exact renormalisation: the value is unchanged, x0 = RN(value of x0 + x1), x1 + x2 non-overlapping
CR_HD td renorm(double a0, double a1, double a2) {
    double s, e, r0, f, r1, r2;
    two_sum(a1, a2, s, e);
    two_sum(a0, s, r0, f);
    two_sum(f, e, r1, r2);
    fast_two_sum(r0, r1, r0, r1);
    two_sum(r1, r2, r1, r2);
    return {r0, r1, r2};
}
CR_HD td td_add(td a, td b) {
    double s0, e0, s1, e1, s2, e2, t1, f1;
    two_sum(a.x0, b.x0, s0, e0);
    two_sum(a.x1, b.x1, s1, e1);
    two_sum(a.x2, b.x2, s2, e2);
    two_sum(e0, s1, t1, f1);
    const double t2 = add(add(add(f1, e1), s2), e2);
    return renorm(s0, t1, t2);
}
CR_HD td td_mul_d(td a, double d) {
    double p0, e0, p1, e1, t1, f1;
    two_prod(a.x0, d, p0, e0);
    two_prod(a.x1, d, p1, e1);
    two_sum(e0, p1, t1, f1);
    const double t2 = add(add(f1, e1), mul(a.x2, d));
    return renorm(p0, t1, t2);
}
CR_HD td td_mul(td a, td b) {
    double p, e00, q1, e01, q2, e10, m, fm, m2, fm2;
    two_prod(a.x0, b.x0, p, e00);
    two_prod(a.x0, b.x1, q1, e01);
    two_prod(a.x1, b.x0, q2, e10);
    two_sum(q1, q2, m, fm);
    two_sum(m, e00, m2, fm2);
    double low = add(fm, fm2);
    low = add(low, add(e01, e10));
    low = fmaf64(a.x1, b.x1, low);
    low = fmaf64(a.x0, b.x2, low);
    low = fmaf64(a.x2, b.x0, low);
    return renorm(p, m2, low);
}
CR_HD td td_neg(td a) { return {-a.x0, -a.x1, -a.x2}; }

// the double nearest to r0 + r1 + r2 (renormalised: r0 = RN(r0 + r1), r1 + r2 non-overlapping)
CR_HD double round_td(td r) {
    if (r.x1 == 0) return r.x0;
    const double nb = nextafter(r.x0, r.x1 > 0 ? INFINITY : -INFINITY);
    const double half = mul(sub(nb, r.x0), 0.5);  // the gap is a power of two: exact
    if (r.x1 != half) return fabs(r.x1) < fabs(half) ? r.x0 : nb;
    if (r.x2 == 0) {  // an exact tie (never for log or cos of a double other than the trivial ones)
        return (as_u64(r.x0) & 1) ? nb : r.x0;
    }
    return ((r.x2 > 0) == (r.x1 > 0)) ? nb : r.x0;
}

// Ziv's rounding test: RN(r) when every value within eps |r| of r rounds to it, else NaN
CR_HD double ziv_round(dd r, double eps) {
    const double e = mul(eps, fabs(r.h));
    const double a = add(r.h, sub(r.l, e)), b = add(r.h, add(r.l, e));
    return a == b ? a : NAN;
}
constexpr double kZivEps = 0x1p-64;  // the fast steps' error bounds are below 2^-68

// ---- log ----------------------------------------------------------------------------------
struct LogArg {
    int K, i;
    double z;
};
CR_HD LogArg log_reduce(double x) {
    int e = 0;
    // x = 2^e m, m in [1, 2), from the bits (subnormals scaled by 2^54 first)
    uint64_t b = as_u64(x);
    if ((b >> 52) == 0) {
        b = as_u64(mul(x, 0x1p54));
        e = -54;
    }
    e += (int)(b >> 52) - 1023;
    const int i = (int)((b >> 45) & 127);
    const double m = as_f64((b & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL);
    const double r = CR_T(log_r)[i];
    return {e + (i >= CR_LOG_SPLIT ? 1 : 0), i, fmaf64(m, r, -1.0)};
}

// fast step: log x as a double-double with relative error below 2^-68
CR_HD dd log_fast(const LogArg &a) {
    const double z = a.z;
    // log1p(z) = z - z^2/2 + z^3 q(z), q = sum_{n=3}^{10} (-1)^(n+1) z^(n-3) / n
    double q = -1.0 / 10;
    q = fmaf64(q, z, 1.0 / 9);
    q = fmaf64(q, z, -1.0 / 8);
    q = fmaf64(q, z, 1.0 / 7);
    q = fmaf64(q, z, -1.0 / 6);
    q = fmaf64(q, z, 1.0 / 5);
    q = fmaf64(q, z, -1.0 / 4);
    q = fmaf64(q, z, CR_T(inv_n)[3 * 2]);  // 1/3 (leading part)
    double h, hl, s, se;
    two_prod(z, z, h, hl);
    two_sum(z, mul(-0.5, h), s, se);
    const double lo = add(sub(se, mul(0.5, hl)), mul(mul(h, z), q));
    dd p;
    fast_two_sum(s, lo, p.h, p.l);
    const double K = (double)a.K;
    dd kl2;
    kl2.h = mul(K, CR_LN2_0);                       // exact: 42-bit ln2_0, |K| < 2^11
    kl2.l = fmaf64(K, CR_LN2_2, mul(K, CR_LN2_1));  // K ln2_1 exact, one rounding
    const double *L = CR_T(log_l) + 3 * a.i;
    // |K ln 2| >= ln 2 > |L_i| unless K = 0; |L_i| > 0.0117 > |log1p z| unless L_i = 0
    const dd c = dd_add_fast(kl2, dd{L[0], L[1]});
    return dd_add_fast(c, p);
}

// accurate step: log x as a triple-double with relative error near 2^-140
CR_HD_COLD td log_accurate(const LogArg &a) {
    const double z = a.z;
    const double *inv = CR_T(inv_n);
    // Q(z) = sum_{n=1}^{19} (-1)^(n+1) z^(n-1) / n by Horner; log1p(z) = z Q(z)
    td Q = {inv[3 * 18], inv[3 * 18 + 1], inv[3 * 18 + 2]};
    for (int n = 18; n >= 1; n--) {
        const double sg = (n & 1) ? 1.0 : -1.0;
        const td c = {sg * inv[3 * (n - 1)], sg * inv[3 * (n - 1) + 1], sg * inv[3 * (n - 1) + 2]};
        Q = td_add(c, td_mul_d(Q, z));
    }
    const td p = td_mul_d(Q, z);
    const double K = (double)a.K;
    // K ln2_0 and K ln2_1 exact; K ln2_2 rounded (2^-53 of a 2^-84 part)
    const td kl2 = renorm(mul(K, CR_LN2_0), mul(K, CR_LN2_1), mul(K, CR_LN2_2));
    const double *L = CR_T(log_l) + 3 * a.i;
    const td c = td_add(kl2, td{L[0], L[1], L[2]});
    return td_add(c, p);
}

// the double nearest to log(x), x > 0 finite
CR_HD double cr_log(double x) {
    if (x == 1.0) return 0.0;
    const LogArg a = log_reduce(x);
    const double r = ziv_round(log_fast(a), kZivEps);
    if (r == r) return r;
    return round_td(log_accurate(a));
}

// ---- cos ----------------------------------------------------------------------------------
struct CosArg {
    double y;
    int k;       // quadrant: y = k pi/2 + t
    int j;       // |t| = j/128 + b
    int neg;     // t < 0
};

// t = y - k pi/2 as a triple-double (exact to 2^-200 absolute for |y| < 8)
CR_HD td cos_reduce(double y, int &k) {
    k = (int)rint(mul(y, CR_2_OVER_PI));
    const double K = (double)k;
    const double a = sub(y, mul(K, CR_PIO2_0));   // exact: k P1 exact, y - k P1 by Sterbenz
    double t0, t1;
    two_sum(a, -mul(K, CR_PIO2_1), t0, t1);       // exact
    td t = renorm(t0, t1, 0.0);
    t = td_add(t, renorm(-mul(K, CR_PIO2_2), -mul(K, CR_PIO2_3), 0.0));
    return t;
}

// fast step: cos y as a double-double with relative error below 2^-68, or NaN when y lies within
// 2^-20 of a nonzero multiple of pi/2 (the accurate step's reduction keeps more digits there)
CR_HD dd cos_fast(double y, CosArg &ca) {
    ca.y = y;
    ca.k = (int)rint(mul(y, CR_2_OVER_PI));
    const double K = (double)ca.k;
    // t = y - k (P1 + P2 + P3): y - k P1 and the sum with -k P2 exact, k P3 folded into the low
    // part with one rounding; the dropped k P4 is below 2^-154
    double t0, t1;
    two_sum(sub(y, mul(K, CR_PIO2_0)), -mul(K, CR_PIO2_1), t0, t1);
    t1 = sub(t1, mul(K, CR_PIO2_2));
    fast_two_sum(t0, t1, t0, t1);
    if (ca.k != 0 && fabs(t0) < 0x1p-20) return {NAN, 0.0};  // (k = 0: t = y exactly)
    ca.neg = t0 < 0;
    if (ca.neg) {
        t0 = -t0;
        t1 = -t1;
    }
    ca.j = (int)rint(mul(t0, 128.0));
    const double b0 = sub(t0, mul((double)ca.j, 0x1p-7));  // exact
    const double b1 = t1;
    // b^2 = q + ql
    double q, ql;
    two_prod(b0, b0, q, ql);
    ql = fmaf64(2.0 * b0, b1, ql);
    // sin b = b0 + b1 + b0^3 S(b^2) - b0^2 b1 / 2, S = -1/6 + b^2/120 - b^4/5040 + b^6/362880
    double S = 1.0 / 362880;
    S = fmaf64(S, q, -1.0 / 5040);
    S = fmaf64(S, q, 1.0 / 120);
    S = fmaf64(S, q, -1.0 / 6);
    double slo = fmaf64(mul(q, b0), S, b1);
    slo = fmaf64(mul(-0.5, q), b1, slo);
    dd sb;
    fast_two_sum(b0, slo, sb.h, sb.l);
    // cos b = 1 - q/2 - ql/2 + q^2 C(q), C = 1/24 - q/720 + q^2/40320 - q^3/3628800
    double C = -1.0 / 3628800;
    C = fmaf64(C, q, 1.0 / 40320);
    C = fmaf64(C, q, -1.0 / 720);
    C = fmaf64(C, q, 1.0 / 24);
    double c0, ce;
    two_sum(1.0, mul(-0.5, q), c0, ce);
    const double clo = fmaf64(mul(q, q), C, sub(ce, mul(0.5, ql)));
    dd cb;
    fast_two_sum(c0, clo, cb.h, cb.l);
    const double *T = CR_T(sincos) + 6 * ca.j;
    const dd sj = {T[0], T[1]}, cj = {T[3], T[4]};
    dd r;
    // the first product is the larger (or zero: j = 0): |sin(j/128) cos b| >= 2 |cos(j/128) sin b|
    // for j >= 1, and cos(j/128) cos b >= 0.7 > 128 |sin(j/128) sin b|
    if (ca.k & 1) {  // sin |t| = sin(a) cos b + cos(a) sin b
        r = dd_add_fast(dd_mul(sj, cb), dd_mul(cj, sb));
        const bool negate = ((ca.k & 3) == 1) != (ca.neg != 0);  // -sin t for k = 1 mod 4, sin t for 3
        if (negate) r = {-r.h, -r.l};
    } else {  // cos |t| = cos(a) cos b - sin(a) sin b
        r = dd_add_fast(dd_mul(cj, cb), dd_mul(dd{-sj.h, -sj.l}, sb));
        if (ca.k & 2) r = {-r.h, -r.l};
    }
    return r;
}

// accurate step: cos y as a triple-double with relative error near 2^-140
CR_HD_COLD td cos_accurate(double y) {
    CosArg ca;
    td t = cos_reduce(y, ca.k);
    ca.neg = t.x0 < 0;
    if (ca.neg) t = td_neg(t);
    ca.j = (int)rint(mul(t.x0, 128.0));
    const td b = td_add(t, td{-(double)ca.j * 0x1p-7, 0.0, 0.0});
    const td b2 = td_mul(b, b);
    const double *F = CR_T(inv_fact);
    // sin b = b sum_{n=0}^{6} (-1)^n b^(2n) / (2n+1)!;  cos b = sum_{n=0}^{7} (-1)^n b^(2n) / (2n)!
    td s = {F[3 * 13], F[3 * 13 + 1], F[3 * 13 + 2]};  // +1/13!
    for (int n = 5; n >= 0; n--) {
        const double sg = (n & 1) ? -1.0 : 1.0;
        const double *f = F + 3 * (2 * n + 1);
        s = td_add(td{sg * f[0], sg * f[1], sg * f[2]}, td_mul(s, b2));
    }
    const td sb = td_mul(s, b);
    td c = {-F[3 * 14], -F[3 * 14 + 1], -F[3 * 14 + 2]};  // -1/14!
    for (int n = 6; n >= 0; n--) {
        const double sg = (n & 1) ? -1.0 : 1.0;
        const double *f = F + 3 * (2 * n);
        c = td_add(td{sg * f[0], sg * f[1], sg * f[2]}, td_mul(c, b2));
    }
    const double *T = CR_T(sincos) + 6 * ca.j;
    const td sj = {T[0], T[1], T[2]}, cj = {T[3], T[4], T[5]};
    td r;
    if (ca.k & 1) {
        r = td_add(td_mul(sj, c), td_mul(cj, sb));
        const bool negate = ((ca.k & 3) == 1) != (ca.neg != 0);
        if (negate) r = td_neg(r);
    } else {
        r = td_add(td_mul(cj, c), td_neg(td_mul(sj, sb)));
        if (ca.k & 2) r = td_neg(r);
    }
    return r;
}

// the double nearest to cos(y), |y| < 8
CR_HD double cr_cos(double y) {
    CosArg ca;
    const double r = ziv_round(cos_fast(y, ca), kZivEps);
    if (r == r) return r;
    return round_td(cos_accurate(y));
}

// sampleNorm (src/random.c:34-49) from its two 64-bit draws, with correctly rounded log and cos:
// sqrt(-2 log u) cos(2 pi v), u = (A + 1/2) / 2^64, v likewise (every other operation is a single
// IEEE operation, as in the reference)
CR_HD double box_muller(uint64_t A, uint64_t B) {
#if defined(__CUDA_ARCH__)
    // the division by 2^64 is exact: a multiplication by 2^-64 gives the same double
    const double u = mul(__dadd_rn(__ull2double_rn(A), 0.5), 0x1p-64);
    const double v = mul(__dadd_rn(__ull2double_rn(B), 0.5), 0x1p-64);
    const double r = __dsqrt_rn(mul(-2.0, cr_log(u)));
#else
    const double RMax = 18446744073709551616.0;
    const double u = ((double)A + 0.5) / RMax;
    const double v = ((double)B + 0.5) / RMax;
    const double r = sqrt(-2.0 * cr_log(u));
#endif
    return mul(r, cr_cos(mul(2 * 3.14159265358979323846, v)));
}

}  // namespace crm
