/*
 * mitos_oracle.c -- CPU restatement (FP64, OpenMP) of the Mitos initial-condition hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker and the CPU baseline.  Nothing in the GPU library
 * links, loads or calls this code.  Each function names the reference file:line it follows.
 * Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts give identical results.
 *
 * The 3D FFT restates the published algorithm of FFTW3 (the reference's dependency, version
 * unpinned: Makefile:7 links -lfftw3 -lfftw3_mpi) with FFTW's conventions: unnormalised,
 * forward sign -1, r2c = real z transform then complex y and x transforms, c2r = complex
 * x and y transforms then a z c2r that reads only the real parts of the kz = 0 and
 * kz = N/2 elements.  The 1D transforms are a mixed-radix (4, 2, 3, 5) Stockham FFT with
 * twiddles from the host libm.
 */
#include "mitos_oracle.h"
#include "thermal_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ===================================================================================== */
/* Random numbers                                                                         */
/* ===================================================================================== */

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* splitmix64 seeding of xoshiro256**: include/random_xorshift.h:38-59 */
void orc_rng_init(uint64_t seed, uint64_t s[4]) {
    uint64_t st = seed;
    for (int i = 0; i < 4; i++) {
        uint64_t r = st;
        st = r + 0x9E3779B97f4A7C15ULL;
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ULL;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBULL;
        s[i] = r ^ (r >> 31);
    }
}

/* xoshiro256**: include/random_xorshift.h:15-29 */
uint64_t orc_rng_next(uint64_t s[4]) {
    const uint64_t result = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

void orc_rng_advance(uint64_t s[4], uint64_t n) {
    for (uint64_t i = 0; i < n; i++) (void)orc_rng_next(s);
}

/* sampleUniform: src/random.c:27-31 */
double orc_sample_uniform(uint64_t s[4]) {
    const uint64_t A = orc_rng_next(s);
    const double RM = (double)UINT64_MAX + 1;
    return ((double)A + 0.5) / RM;
}

/* sampleNorm (Box-Muller, cosine branch only): src/random.c:34-49 */
double orc_sample_norm(uint64_t s[4]) {
    const uint64_t A = orc_rng_next(s);
    const uint64_t B = orc_rng_next(s);
    const double RMax = (double)UINT64_MAX + 1;
    const double u = ((double)A + 0.5) / RMax;
    const double v = ((double)B + 0.5) / RMax;
    return sqrt(-2 * log(u)) * cos(2 * M_PI * v);
}

void orc_draws(uint64_t seed, int64_t n, uint64_t *out) {
    uint64_t s[4];
    orc_rng_init(seed, s);
    for (int64_t i = 0; i < n; i++) out[i] = orc_rng_next(s);
}

void orc_norms(uint64_t seed, int64_t n, double *out) {
    uint64_t s[4];
    orc_rng_init(seed, s);
    for (int64_t i = 0; i < n; i++) out[i] = orc_sample_norm(s);
}

/* ===================================================================================== */
/* Wavevectors and k-space kernels                                                        */
/* ===================================================================================== */

/* fft_wavevector: src/fft.c:29-35 */
void orc_wavevector(int x, int y, int z, int N, double dk, double *kx, double *ky, double *kz,
                    double *k) {
    *kx = (x > N / 2) ? (x - N) * dk : x * dk;
    *ky = (y > N / 2) ? (y - N) * dk : y * dk;
    *kz = (z > N / 2) ? (z - N) * dk : z * dk;
    *k = sqrt((*kx) * (*kx) + (*ky) * (*ky) + (*kz) * (*kz));
}

static inline long idx_half(int N, int x, int y, int z) {
    return ((long)x * N + y) * (N / 2 + 1) + z;
}

/* ===================================================================================== */
/* White noise                                                                            */
/* ===================================================================================== */

/* generate_complex_grf: src/grf.c:26-69 (one rank: X0 = 0, NX = N, seed = Seed + 0) */
int orc_generate_grf(int N, double boxlen, uint64_t seed, double *fbox) {
    const double boxvol = boxlen * boxlen * boxlen;
    const double factor = sqrt(boxvol / 2);
    const double dk = 2 * M_PI / boxlen;
    uint64_t s[4];
    orc_rng_init(seed, s);
    double kx, ky, kz, k;
    for (int x = 0; x < N; x++) {
        for (int y = 0; y < N; y++) {
            for (int z = 0; z <= N / 2; z++) {
                orc_wavevector(x, y, z, N, dk, &kx, &ky, &kz, &k);
                long id = idx_half(N, x, y, z);
                if (k > 0) {
                    double a = orc_sample_norm(s) * factor;
                    double b = orc_sample_norm(s) * factor;
                    fbox[2 * id] = a;
                    fbox[2 * id + 1] = b;
                } else {
                    fbox[2 * id] = 0;
                    fbox[2 * id + 1] = 0;
                }
            }
        }
    }
    return 0;
}

/* enforce_hermiticity: src/grf.c:78-175 (the gathered plane is the whole plane on one rank) */
int orc_enforce_hermiticity(int N, double *fbox) {
    double *plane = malloc(sizeof(double) * 2 * (size_t)N * N);
    if (!plane) return 5;
    for (int z = 0; z <= N / 2; z += N / 2) {
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++) {
                long id = idx_half(N, x, y, z);
                plane[2 * ((long)x * N + y)] = fbox[2 * id];
                plane[2 * ((long)x * N + y) + 1] = fbox[2 * id + 1];
            }
        for (int x = 0; x < N; x++) {
            for (int y = 0; y < N; y++) {
                if (x > N / 2) continue;
                if ((x == 0 || x == N / 2) && y > N / 2) continue;
                int invx = (x > 0) ? N - x : 0;
                int invy = (y > 0) ? N - y : 0;
                int invz = (z > 0) ? N - z : 0;
                long id = idx_half(N, x, y, z);
                if (invx == x && invy == y && invz == z) {
                    fbox[2 * id + 1] = 0;
                } else {
                    long src = (long)invx * N + invy;
                    fbox[2 * id] = plane[2 * src];
                    fbox[2 * id + 1] = -plane[2 * src + 1];
                }
            }
        }
        if (N / 2 == 0) break;
    }
    free(plane);
    return 0;
}

/* primordialPower: src/primordial.c:25-33 */
double orc_primordial_power(double k, const struct orc_cosmo *c) {
    if (k == 0) return 0;
    return c->A_s * pow(k / c->k_pivot, c->n_s - 1.) * k * (2. * M_PI * M_PI);
}

/* ===================================================================================== */
/* Perturbation spline: src/perturb_spline.c                                              */
/* ===================================================================================== */

/* initPerturbSpline: src/perturb_spline.c:30-63 */
int orc_spline_init(struct orc_perturb *sp, int k_acc_size) {
    sp->k_acc = malloc(sizeof(double) * k_acc_size);
    if (!sp->k_acc) return 1;
    sp->k_acc_size = k_acc_size;
    int k_size = sp->k_size;
    double k_min = sp->k[0];
    double k_max = sp->k[k_size - 1];
    for (int i = 0; i < k_acc_size; i++) {
        double u = (double)i / k_acc_size;
        double v = k_min + u * (k_max - k_min);
        double maxJ = 0;
        for (int j = 0; j < k_size; j++)
            if (sp->k[j] < v) maxJ = j;
        sp->k_acc[i] = maxJ;
    }
    return 0;
}

void orc_spline_free(struct orc_perturb *sp) {
    free(sp->k_acc);
    sp->k_acc = NULL;
}

/* perturbSplineFindTau: src/perturb_spline.c:73-106 */
void orc_spline_find_tau(const struct orc_perturb *sp, double log_tau, int *index, double *u) {
    int tau_size = sp->tau_size;
    if (log_tau < sp->log_tau[0]) {
        *index = 0;
        *u = 0.f;
        return;
    } else if (log_tau >= sp->log_tau[tau_size - 1]) {
        *index = tau_size - 2;
        *u = 1.f;
        return;
    }
    for (int i = 1; i < tau_size; i++) {
        if (sp->log_tau[i] >= log_tau) {
            *index = i - 1;
            break;
        }
    }
    double left = sp->log_tau[*index];
    double right = sp->log_tau[*index + 1];
    *u = (log_tau - left) / (right - left);
}

/* perturbSplineFindK: src/perturb_spline.c:109-147 (the search never reaches the
 * out-of-bounds read at i = k_size - 1 for grid wavenumbers inside the table) */
void orc_spline_find_k(const struct orc_perturb *sp, double k, int *index, double *u) {
    int k_acc_size = sp->k_acc_size;
    int k_size = sp->k_size;
    double k_min = sp->k[0];
    double k_max = sp->k[k_size - 1];
    if (k > k_max) {
        *index = k_size - 2;
        *u = 1.0;
        return;
    }
    double w = (k - k_min) / (k_max - k_min);
    int J = floor(w * k_acc_size);
    int start = sp->k_acc[J < k_acc_size ? J : k_acc_size - 1];
    int i;
    for (i = start; i < k_size - 1; i++)
        if (k >= sp->k[i] && k <= sp->k[i + 1]) break;
    *index = i;
    double left = sp->k[*index];
    double right = sp->k[*index + 1];
    *u = (k - left) / (right - left);
}

/* perturbSplineInterp: src/perturb_spline.c:150-169 */
double orc_spline_interp(const struct orc_perturb *sp, int k_index, int tau_index, double u_k,
                         double u_tau, int index_src) {
    int k_size = sp->k_size, tau_size = sp->tau_size;
    const double *arr = sp->delta + (long)index_src * k_size * tau_size;
    double T11 = arr[k_size * tau_index + k_index];
    double T21 = arr[k_size * tau_index + k_index + 1];
    double T12 = arr[k_size * (tau_index + 1) + k_index];
    double T22 = arr[k_size * (tau_index + 1) + k_index + 1];
    return (1 - u_tau) * ((1 - u_k) * T11 + u_k * T21) + u_tau * ((1 - u_k) * T12 + u_k * T22);
}

/* perturbLogTauAtRedshift: src/perturb_spline.c:240-267 */
double orc_log_tau_at_redshift(const struct orc_perturb *sp, double redshift) {
    int tau_size = sp->tau_size;
    if (redshift > sp->redshift[0]) return sp->log_tau[0];
    else if (redshift <= sp->redshift[tau_size - 1]) return sp->log_tau[tau_size - 1];
    int index;
    for (index = tau_size - 1; index > 0; index--)
        if (sp->redshift[index] >= redshift) break;
    double left = sp->redshift[index];
    double right = sp->redshift[index + 1];
    double u = (redshift - left) / (right - left);
    return (1 - u) * sp->log_tau[index] + u * sp->log_tau[index + 1];
}

/* perturbGrowthFactorAtLogTau: src/perturb_spline.c:201-212 */
double orc_growth_at_log_tau(const struct orc_perturb *sp, double log_tau) {
    int tau_index = 0;
    double u_tau;
    orc_spline_find_tau(sp, log_tau, &tau_index, &u_tau);
    return (1 - u_tau) * sp->D_growth[tau_index] + u_tau * sp->D_growth[tau_index + 1];
}

/* ===================================================================================== */
/* Kernel application: src/fft.c:257-302 with the kernels of include/fft_kernels.h         */
/* ===================================================================================== */

static inline double sinc_ref(double x) { return x == 0 ? 1. : sin(x) / x; }

/* one kernel value (re, im) at a wavevector; include/fft_kernels.h:28-219 */
static void kernel_value(int id, double kx, double ky, double kz, double k, const void *params,
                         double *kr, double *ki) {
    *kr = 0;
    *ki = 0;
    switch (id) {
    case ORC_K_CONSTANT: *kr = *(const double *)params; break;                  /* :28-31 */
    case ORC_K_LOWPASS: *kr = (k < *(const double *)params) ? 1.0 : 0.0; break; /* :33-37 */
    case ORC_K_HIPASS: *kr = (k > *(const double *)params) ? 1.0 : 0.0; break;  /* :39-43 */
    case ORC_K_TOPHAT: {                                                        /* :45-51 */
        const double *p = params;
        *kr = (k >= p[0] && k <= p[1]) ? 1.0 : 0.0;
        break;
    }
    case ORC_K_ELLIPTIC_TOPHAT: { /* :54-68 */
        const double *p = params;
        double kr_ = kx * p[0] + ky * p[1] + kz * p[2];
        double kk = kx * kx + ky * ky + kz * kz;
        double rr = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        double theta = kk * rr + (p[3] - 1) * kr_ * kr_;
        *kr = (theta <= 4 * M_PI * M_PI) ? 1.0 : 0.0;
        break;
    }
    case ORC_K_TRANSLATE: { /* :70-79 */
        const double *p = params;
        double ph = p[0] * kx + p[1] * ky + p[2] * kz;
        *kr = cos(ph);
        *ki = sin(ph);
        break;
    }
    case ORC_K_GAUSSIAN: { /* :81-86 */
        double kR = k * *(const double *)params;
        *kr = exp(-kR * kR);
        break;
    }
    case ORC_K_GAUSSIAN_INV: { /* :88-93 */
        double kR = k * *(const double *)params;
        *kr = exp(kR * kR);
        break;
    }
    case ORC_K_INV_POISSON: *kr = (k > 0) ? -1.0 / k / k : 1.0; break; /* :96-99 */
    case ORC_K_DX: *ki = kx; break;                                    /* :101-104 */
    case ORC_K_DY: *ki = ky; break;                                    /* :106-109 */
    case ORC_K_DZ: *ki = kz; break;                                    /* :111-114 */
    case ORC_K_POWER_NO_TRANSFER:                                      /* :116-121 */
        *kr = sqrt(orc_primordial_power(k, (const struct orc_cosmo *)params));
        break;
    case ORC_K_TRANSFER: /* :131-155 */
    case ORC_K_INV_TRANSFER: /* :158-182 */
        if (k == 0) {
            *kr = 0.f;
        } else {
            const struct orc_transfer_params *tp = params;
            int k_index;
            double u_k;
            orc_spline_find_k(tp->sp, k, &k_index, &u_k);
            double T = orc_spline_interp(tp->sp, k_index, tp->tau_index, u_k, tp->u_tau,
                                         tp->index_src);
            *kr = (id == ORC_K_TRANSFER) ? T : 1.0 / T;
        }
        break;
    case ORC_K_UNDO_HERMITE: /* :198-219 */
        if (k == 0) {
            *kr = 1.0;
        } else {
            const struct orc_hermite_params *p = params;
            double W_x = sinc_ref(0.5 * kx * p->boxlen / p->N);
            double W_y = sinc_ref(0.5 * ky * p->boxlen / p->N);
            double W_z = sinc_ref(0.5 * kz * p->boxlen / p->N);
            double W = pow(W_x * W_y * W_z, p->order);
            *kr = 1.0 / W;
        }
        break;
    default: break;
    }
}

int orc_apply_kernel(int N, double boxlen, double *write, const double *read, int kernel_id,
                     const void *params) {
    const double dk = 2 * M_PI / boxlen;
    if (kernel_id < ORC_K_CONSTANT || kernel_id > ORC_K_UNDO_HERMITE) return 3;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < N; x++) {
        for (int y = 0; y < N; y++) {
            for (int z = 0; z <= N / 2; z++) {
                double kx, ky, kz, k, kr, ki;
                orc_wavevector(x, y, z, N, dk, &kx, &ky, &kz, &k);
                kernel_value(kernel_id, kx, ky, kz, k, params, &kr, &ki);
                long id = idx_half(N, x, y, z);
                double a = read[2 * id], b = read[2 * id + 1];
                /* complex product as GCC expands it for double complex */
                write[2 * id] = a * kr - b * ki;
                write[2 * id + 1] = a * ki + b * kr;
            }
        }
    }
    return 0;
}

/* ===================================================================================== */
/* FFT                                                                                    */
/* ===================================================================================== */

#define MAXST 40
typedef struct {
    int n, nst;
    int rad[MAXST];
    double *twr, *twi; /* exp(-2 pi i m / n), m < n */
    double r3c, r3s, r5c1, r5s1, r5c2, r5s2;
} plan1d;

static plan1d *plan_cache[4097];

static plan1d *make_plan(int n) {
    plan1d *p = calloc(1, sizeof(plan1d));
    p->n = n;
    int m = n, ns = 0;
    while (m % 4 == 0 && m > 1) { p->rad[ns++] = 4; m /= 4; }
    while (m % 2 == 0) { p->rad[ns++] = 2; m /= 2; }
    while (m % 3 == 0) { p->rad[ns++] = 3; m /= 3; }
    while (m % 5 == 0) { p->rad[ns++] = 5; m /= 5; }
    if (m != 1) { free(p); return NULL; }
    p->nst = ns;
    p->twr = malloc(sizeof(double) * n);
    p->twi = malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) {
        double a = 2.0 * M_PI * (double)i / (double)n;
        p->twr[i] = cos(a);
        p->twi[i] = -sin(a);
    }
    p->r3c = cos(2 * M_PI / 3);
    p->r3s = sin(2 * M_PI / 3);
    p->r5c1 = cos(2 * M_PI / 5);
    p->r5s1 = sin(2 * M_PI / 5);
    p->r5c2 = cos(4 * M_PI / 5);
    p->r5s2 = sin(4 * M_PI / 5);
    return p;
}

static plan1d *get_plan(int n) {
    if (n <= 0 || n > 4096) return NULL;
    plan1d *p;
#pragma omp critical(orc_plan)
    {
        if (!plan_cache[n]) plan_cache[n] = make_plan(n);
        p = plan_cache[n];
    }
    return p;
}

/* Batched mixed-radix Stockham FFT.  re/im hold n x B values, element (i, b) at i*B + b.
 * sign = -1 forward, +1 backward (unnormalised). */
static void fft_batch(const plan1d *p, int sign, double *re, double *im, double *wr, double *wi,
                      int B) {
    const int n = p->n;
    double *ar = re, *ai = im, *br = wr, *bi = wi;
    int Ns = 1;
    const double sg = (double)sign;
    for (int st = 0; st < p->nst; st++) {
        const int R = p->rad[st];
        const int nR = n / R;
        for (int j = 0; j < nR; j++) {
            const int jm = j % Ns;
            const int idxD = (j / Ns) * Ns * R + jm;
            const int tstep = jm * (n / (Ns * R));
            double tr[5], ti[5];
            for (int r = 0; r < R; r++) {
                int m = (r * tstep) % n;
                tr[r] = p->twr[m];
                ti[r] = (sign < 0) ? p->twi[m] : -p->twi[m]; /* exp(sign 2 pi i m/n) */
            }
            for (int b = 0; b < B; b++) {
                double vr[5], vi[5];
                for (int r = 0; r < R; r++) {
                    double xr = ar[(long)(j + r * nR) * B + b], xi = ai[(long)(j + r * nR) * B + b];
                    if (r == 0 || tstep == 0) {
                        vr[r] = xr;
                        vi[r] = xi;
                    } else {
                        vr[r] = xr * tr[r] - xi * ti[r];
                        vi[r] = xr * ti[r] + xi * tr[r];
                    }
                }
                double yr[5], yi[5];
                if (R == 2) {
                    yr[0] = vr[0] + vr[1]; yi[0] = vi[0] + vi[1];
                    yr[1] = vr[0] - vr[1]; yi[1] = vi[0] - vi[1];
                } else if (R == 4) {
                    double s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
                    double d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
                    double s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
                    double d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
                    /* multiply d1 by (-i*sign)^... : forward uses -i, backward +i */
                    double er, ei;
                    if (sign < 0) { er = d1i; ei = -d1r; } else { er = -d1i; ei = d1r; }
                    yr[0] = s0r + s1r; yi[0] = s0i + s1i;
                    yr[2] = s0r - s1r; yi[2] = s0i - s1i;
                    yr[1] = d0r + er;  yi[1] = d0i + ei;
                    yr[3] = d0r - er;  yi[3] = d0i - ei;
                } else if (R == 3) {
                    double c = p->r3c, s = sg * p->r3s;
                    double t1r = vr[1] + vr[2], t1i = vi[1] + vi[2];
                    double t2r = vr[1] - vr[2], t2i = vi[1] - vi[2];
                    yr[0] = vr[0] + t1r; yi[0] = vi[0] + t1i;
                    double mr = vr[0] + c * t1r, mi = vi[0] + c * t1i;
                    /* e^{sign i 2pi/3} = c + i s */
                    yr[1] = mr - s * t2i; yi[1] = mi + s * t2r;
                    yr[2] = mr + s * t2i; yi[2] = mi - s * t2r;
                } else { /* R == 5, direct */
                    double cr[5] = {1.0, p->r5c1, p->r5c2, p->r5c2, p->r5c1};
                    double ci[5] = {0.0, p->r5s1, p->r5s2, -p->r5s2, -p->r5s1};
                    for (int k = 0; k < 5; k++) {
                        double sr = 0, si = 0;
                        for (int r = 0; r < 5; r++) {
                            int e = (r * k) % 5;
                            double wr_ = cr[e], wi_ = sg * ci[e];
                            sr += vr[r] * wr_ - vi[r] * wi_;
                            si += vr[r] * wi_ + vi[r] * wr_;
                        }
                        yr[k] = sr; yi[k] = si;
                    }
                }
                for (int r = 0; r < R; r++) {
                    br[(long)(idxD + r * Ns) * B + b] = yr[r];
                    bi[(long)(idxD + r * Ns) * B + b] = yi[r];
                }
            }
        }
        double *t;
        t = ar; ar = br; br = t;
        t = ai; ai = bi; bi = t;
        Ns *= R;
    }
    if (ar != re) {
        memcpy(re, ar, sizeof(double) * (size_t)n * B);
        memcpy(im, ai, sizeof(double) * (size_t)n * B);
    }
}

int orc_fft_1d(int n, int sign, double *data) {
    plan1d *p = get_plan(n);
    if (!p) return 1;
    double *buf = malloc(sizeof(double) * 4 * n);
    double *re = buf, *im = buf + n, *wr = buf + 2 * n, *wi = buf + 3 * n;
    for (int i = 0; i < n; i++) { re[i] = data[2 * i]; im[i] = data[2 * i + 1]; }
    fft_batch(p, sign, re, im, wr, wi, 1);
    for (int i = 0; i < n; i++) { data[2 * i] = re[i]; data[2 * i + 1] = im[i]; }
    free(buf);
    return 0;
}

#define FB 8 /* columns per batch */

/* complex transform along x (stride N*H) or y (stride H) of an N x N x H complex array */
static void fft_axis(int N, int H, double *c, int axis, int sign) {
    plan1d *p = get_plan(N);
    const long HN = (long)H * N;
    if (axis == 0) {
        const long ncols = HN;
        const long nchunks = (ncols + FB - 1) / FB;
#pragma omp parallel
        {
            double *buf = malloc(sizeof(double) * 4 * (size_t)N * FB);
            double *re = buf, *im = buf + (long)N * FB, *wr = buf + 2L * N * FB, *wi = buf + 3L * N * FB;
#pragma omp for schedule(static)
            for (long ch = 0; ch < nchunks; ch++) {
                long j0 = ch * FB;
                int B = (int)((ncols - j0) < FB ? (ncols - j0) : FB);
                for (int x = 0; x < N; x++)
                    for (int b = 0; b < B; b++) {
                        long id = x * HN + j0 + b;
                        re[(long)x * B + b] = c[2 * id];
                        im[(long)x * B + b] = c[2 * id + 1];
                    }
                fft_batch(p, sign, re, im, wr, wi, B);
                for (int x = 0; x < N; x++)
                    for (int b = 0; b < B; b++) {
                        long id = x * HN + j0 + b;
                        c[2 * id] = re[(long)x * B + b];
                        c[2 * id + 1] = im[(long)x * B + b];
                    }
            }
            free(buf);
        }
    } else {
        const long nch_per_plane = (H + FB - 1) / FB;
        const long nchunks = (long)N * nch_per_plane;
#pragma omp parallel
        {
            double *buf = malloc(sizeof(double) * 4 * (size_t)N * FB);
            double *re = buf, *im = buf + (long)N * FB, *wr = buf + 2L * N * FB, *wi = buf + 3L * N * FB;
#pragma omp for schedule(static)
            for (long ch = 0; ch < nchunks; ch++) {
                long x = ch / nch_per_plane;
                int z0 = (int)(ch % nch_per_plane) * FB;
                int B = (H - z0) < FB ? (H - z0) : FB;
                for (int y = 0; y < N; y++)
                    for (int b = 0; b < B; b++) {
                        long id = x * HN + (long)y * H + z0 + b;
                        re[(long)y * B + b] = c[2 * id];
                        im[(long)y * B + b] = c[2 * id + 1];
                    }
                fft_batch(p, sign, re, im, wr, wi, B);
                for (int y = 0; y < N; y++)
                    for (int b = 0; b < B; b++) {
                        long id = x * HN + (long)y * H + z0 + b;
                        c[2 * id] = re[(long)y * B + b];
                        c[2 * id + 1] = im[(long)y * B + b];
                    }
            }
            free(buf);
        }
    }
}

/* real rows of length N (pitch rpitch) -> half-complex rows of length N/2+1 */
static void rows_r2c(int N, const double *in, long rpitch, double *out) {
    const int h = N / 2, H = N / 2 + 1;
    plan1d *p = get_plan(h);
    plan1d *pN = get_plan(N);
    const long nrows = (long)N * N;
    const long nchunks = (nrows + FB - 1) / FB;
#pragma omp parallel
    {
        double *buf = malloc(sizeof(double) * 4 * (size_t)h * FB);
        double *re = buf, *im = buf + (long)h * FB, *wr = buf + 2L * h * FB, *wi = buf + 3L * h * FB;
#pragma omp for schedule(static)
        for (long ch = 0; ch < nchunks; ch++) {
            long r0 = ch * FB;
            int B = (int)((nrows - r0) < FB ? (nrows - r0) : FB);
            for (int b = 0; b < B; b++) {
                const double *row = in + (r0 + b) * rpitch;
                for (int n = 0; n < h; n++) {
                    re[(long)n * B + b] = row[2 * n];
                    im[(long)n * B + b] = row[2 * n + 1];
                }
            }
            fft_batch(p, -1, re, im, wr, wi, B);
            for (int b = 0; b < B; b++) {
                double *orow = out + 2 * (r0 + b) * H;
                for (int k = 0; k <= h; k++) {
                    int k1 = k % h, k2 = (h - k) % h;
                    double zr = re[(long)k1 * B + b], zi = im[(long)k1 * B + b];
                    double cr = re[(long)k2 * B + b], ci = -im[(long)k2 * B + b];
                    double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
                    /* odd = (Z - conj Z')/(2i) */
                    double dr = zr - cr, di = zi - ci;
                    double or_ = 0.5 * di, oi = -0.5 * dr;
                    double wr_ = pN->twr[k % N], wi_ = pN->twi[k % N]; /* exp(-2 pi i k/N) */
                    orow[2 * k] = er + (or_ * wr_ - oi * wi_);
                    orow[2 * k + 1] = ei + (or_ * wi_ + oi * wr_);
                }
            }
        }
        free(buf);
    }
}

/* half-complex rows -> real rows (FFTW c2r: Im of k = 0 and k = N/2 ignored) */
static void rows_c2r(int N, const double *in, double *out, long rpitch) {
    const int h = N / 2, H = N / 2 + 1;
    plan1d *p = get_plan(h);
    plan1d *pN = get_plan(N);
    const long nrows = (long)N * N;
    const long nchunks = (nrows + FB - 1) / FB;
#pragma omp parallel
    {
        double *buf = malloc(sizeof(double) * 4 * (size_t)h * FB);
        double *re = buf, *im = buf + (long)h * FB, *wr = buf + 2L * h * FB, *wi = buf + 3L * h * FB;
#pragma omp for schedule(static)
        for (long ch = 0; ch < nchunks; ch++) {
            long r0 = ch * FB;
            int B = (int)((nrows - r0) < FB ? (nrows - r0) : FB);
            for (int b = 0; b < B; b++) {
                const double *row = in + 2 * (r0 + b) * H;
                for (int k = 0; k < h; k++) {
                    double xr = row[2 * k], xi = row[2 * k + 1];
                    double yr = row[2 * (h - k)], yi = -row[2 * (h - k) + 1]; /* conj X_{h-k} */
                    if (k == 0) { xi = 0; yi = 0; }
                    double er = xr + yr, ei = xi + yi;
                    double dr = xr - yr, di = xi - yi;
                    double wr_ = pN->twr[k], wi_ = -pN->twi[k]; /* exp(+2 pi i k/N) */
                    double or_ = dr * wr_ - di * wi_, oi = dr * wi_ + di * wr_;
                    /* Z = E + i O */
                    re[(long)k * B + b] = er - oi;
                    im[(long)k * B + b] = ei + or_;
                }
            }
            fft_batch(p, +1, re, im, wr, wi, B);
            for (int b = 0; b < B; b++) {
                double *orow = out + (r0 + b) * rpitch;
                for (int n = 0; n < h; n++) {
                    orow[2 * n] = re[(long)n * B + b];
                    orow[2 * n + 1] = im[(long)n * B + b];
                }
                for (long q = N; q < rpitch; q++) orow[q] = 0.0;
            }
        }
        free(buf);
    }
}

int orc_dft_r2c_3d(int N, const double *in, long rpitch, double *out) {
    if (N < 2 || (N & 1) || !get_plan(N) || !get_plan(N / 2)) return 1;
    const int H = N / 2 + 1;
    rows_r2c(N, in, rpitch, out);
    fft_axis(N, H, out, 1, -1);
    fft_axis(N, H, out, 0, -1);
    return 0;
}

int orc_dft_c2r_3d(int N, double *in, double *out, long rpitch) {
    if (N < 2 || (N & 1) || !get_plan(N) || !get_plan(N / 2)) return 1;
    const int H = N / 2 + 1;
    fft_axis(N, H, in, 0, +1);
    fft_axis(N, H, in, 1, +1);
    rows_c2r(N, in, out, rpitch);
    return 0;
}

/* fft_r2c_dg + fft_normalize_r2c_dg: src/fft.c:219-235, :91-106 */
int orc_fft_r2c(int N, double boxlen, const double *box, long rpitch, double *fbox) {
    int err = orc_dft_r2c_3d(N, box, rpitch, fbox);
    if (err) return err;
    const double boxvol = boxlen * boxlen * boxlen;
    const double fac = boxvol / ((long long)N * N * N);
    const long n = (long)N * N * (N / 2 + 1) * 2;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) fbox[i] *= fac;
    return 0;
}

/* fft_c2r_dg + fft_normalize_c2r_dg: src/fft.c:238-254, :110-125 (division by the volume) */
int orc_fft_c2r(int N, double boxlen, double *fbox, double *box, long rpitch) {
    int err = orc_dft_c2r_3d(N, fbox, box, rpitch);
    if (err) return err;
    const double boxvol = boxlen * boxlen * boxlen;
    const long n = (long)N * N * rpitch;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) box[i] /= boxvol;
    return 0;
}

/* ===================================================================================== */
/* Grids and solvers                                                                      */
/* ===================================================================================== */

/* alloc_local_grid: src/distributed_grid.c:23-42 (padding zeroed here) */
int orc_grid_alloc(struct orc_grid *g, int N, double boxlen) {
    size_t n = (size_t)N * N * (N / 2 + 1) * 2;
    g->N = N;
    g->boxlen = boxlen;
    g->momentum_space = 0;
    g->fbox = calloc(n, sizeof(double));
    g->box = calloc(n, sizeof(double));
    return (g->fbox && g->box) ? 0 : 5;
}

void orc_grid_free(struct orc_grid *g) {
    free(g->fbox);
    free(g->box);
    g->fbox = g->box = NULL;
}

int orc_grid_r2c(struct orc_grid *g) {
    int e = orc_fft_r2c(g->N, g->boxlen, g->box, g->N + 2, g->fbox);
    g->momentum_space = 1;
    return e;
}

int orc_grid_c2r(struct orc_grid *g) {
    int e = orc_fft_c2r(g->N, g->boxlen, g->fbox, g->box, g->N + 2);
    g->momentum_space = 0;
    return e;
}

static int grid_kernel(struct orc_grid *w, const struct orc_grid *r, int id, const void *params) {
    if (r->N != w->N) return 1;
    if (r->momentum_space != 1) return 2;
    int e = orc_apply_kernel(r->N, r->boxlen, w->fbox, r->fbox, id, params);
    w->momentum_space = 1;
    return e;
}

/* solvePoisson_dg: src/poisson.c:58-70 */
int orc_solve_poisson(struct orc_grid *g) {
    int e = orc_grid_r2c(g);
    if (!e) e = grid_kernel(g, g, ORC_K_INV_POISSON, NULL);
    if (!e) e = orc_grid_c2r(g);
    return e;
}

/* the six Hessian grids phi_ij of the potential, as src/2lpt.c:84-97 computes them */
static int hessian_grids(struct orc_grid *pot, struct orc_grid d[6]) {
    static const int ia[6] = {0, 0, 0, 1, 1, 2};
    static const int ib[6] = {0, 1, 2, 1, 2, 2};
    static const int kid[3] = {ORC_K_DX, ORC_K_DY, ORC_K_DZ};
    for (int j = 0; j < 6; j++) {
        if (orc_grid_alloc(&d[j], pot->N, pot->boxlen)) return 5;
        grid_kernel(&d[j], pot, kid[ia[j]], NULL);
        grid_kernel(&d[j], &d[j], kid[ib[j]], NULL);
        orc_grid_c2r(&d[j]);
        free(d[j].fbox);
        d[j].fbox = NULL;
    }
    return 0;
}

/* solve2LPT: src/2lpt.c:38-143 */
int orc_solve_2lpt(struct orc_grid *pot, struct orc_grid *dens, struct orc_grid *work, double f1,
                   double f2) {
    const int N = dens->N;
    const long chunk = (long)N * N * (N + 2);
    if (dens->momentum_space != 1) return 1;
    grid_kernel(pot, dens, ORC_K_INV_POISSON, NULL);
    orc_grid_r2c(dens);
    struct orc_grid d[6];
    int e = hessian_grids(pot, d);
    if (e) return e;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < chunk; k++) {
        double d_dxx = d[0].box[k], d_dxy = d[1].box[k], d_dxz = d[2].box[k];
        double d_dyy = d[3].box[k], d_dyz = d[4].box[k], d_dzz = d[5].box[k];
        double delta2 = d_dzz * d_dyy + d_dzz * d_dxx + d_dyy * d_dxx - d_dxy * d_dxy -
                        d_dyz * d_dyz - d_dxz * d_dxz;
        work->box[k] = delta2;
    }
    for (int j = 0; j < 6; j++) free(d[j].box);
    orc_solve_poisson(work);
    orc_grid_c2r(pot);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < chunk; k++) pot->box[k] = pot->box[k] * f1 + f2 * work->box[k];
    orc_grid_r2c(pot);
    return 0;
}

/* det3: src/monge_ampere.c:38-42 */
static inline double det3(const double *M) {
    return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
           M[2] * (M[3] * M[7] - M[4] * M[6]);
}

/* solveMongeAmpere: src/monge_ampere.c:50-183.  eps_out receives the reference's
 * sqrt((sum res^2 / sum rho^2) / N^3) (:177) per cycle; rel_out the same ratio without the
 * 1/N^3, both over the N^3 cells (the padding holds zeros here and adds nothing). */
int orc_solve_ma(struct orc_grid *pot, struct orc_grid *dens, struct orc_grid *work, int cycles,
                 double *eps_out, double *rel_out) {
    const int N = dens->N;
    const long chunk = (long)N * N * (N + 2);
    if (dens->momentum_space != 1) return 1;
    grid_kernel(pot, dens, ORC_K_INV_POISSON, NULL);
    orc_grid_r2c(dens);
    for (int it = 0; it < cycles; it++) {
        struct orc_grid d[6];
        int e = hessian_grids(pot, d);
        if (e) return e;
        double eps = 0.0, norm = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : eps, norm)
        for (long k = 0; k < chunk; k++) {
            double d_dxx = d[0].box[k], d_dxy = d[1].box[k], d_dxz = d[2].box[k];
            double d_dyy = d[3].box[k], d_dyz = d[4].box[k], d_dzz = d[5].box[k];
            double M[] = {1 + d_dxx, d_dxy, d_dxz, d_dxy, 1 + d_dyy, d_dyz, d_dxz, d_dyz, 1 + d_dzz};
            double det = det3(M);
            double rho = dens->box[k];
            double resid = (1 + rho) - det;
            work->box[k] = resid;
            eps += resid * resid;
            norm += rho * rho;
        }
        for (int j = 0; j < 6; j++) free(d[j].box);
        orc_solve_poisson(work);
        orc_grid_c2r(pot);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < chunk; k++) pot->box[k] += work->box[k];
        orc_grid_r2c(pot);
        if (eps_out) eps_out[it] = sqrt((eps / norm) / ((long long)N * N * N));
        if (rel_out) rel_out[it] = sqrt(eps / norm);
    }
    return 0;
}

/* ===================================================================================== */
/* Particles, TSC gather, CIC                                                             */
/* ===================================================================================== */

/* genParticlesFromGrid_local: src/particle.c:87-129 (one rank, all M^3 particles) */
void orc_lattice(int M, double boxlen, float *pos) {
    float len = boxlen;
    float spacing = len / M;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < M; x++)
        for (int y = 0; y < M; y++)
            for (int z = 0; z < M; z++) {
                long id = ((long)x * M + y) * M + z;
                pos[3 * id + 0] = x * spacing;
                pos[3 * id + 1] = y * spacing;
                pos[3 * id + 2] = z * spacing;
            }
}

static inline long wrapi(long i, long N) { return ((i % N) + N) % N; }
/* the same, without divisions for i in [-N, 2N) */
static inline long wrap1(long i, long N) {
    if (i >= 0 && i < N) return i;
    if (i < 0 && i >= -N) return i + N;
    if (i >= N && i < 2 * N) return i - N;
    return wrapi(i, N);
}

/* gridTSC_dg + access_grid on one rank: src/grids_interp.c:267-309, :180-207 */
double orc_tsc_gather(const double *box, int N, double boxlen, double x, double y, double z) {
    double X = x * N / boxlen;
    double Y = y * N / boxlen;
    double Z = z * N / boxlen;
    int iX = (int)floor(X);
    int iY = (int)floor(Y);
    int iZ = (int)floor(Z);
    double lookLength = 1.5;
    int lookLftX = (int)floor((X - iX) - lookLength);
    int lookRgtX = (int)floor((X - iX) + lookLength);
    int lookLftY = (int)floor((Y - iY) - lookLength);
    int lookRgtY = (int)floor((Y - iY) + lookLength);
    int lookLftZ = (int)floor((Z - iZ) - lookLength);
    int lookRgtZ = (int)floor((Z - iZ) + lookLength);
    /* the per-axis weights and wrapped indices, each evaluated once (the same operations as the
     * reference's triple loop, so the same values; the sum keeps its order) */
    double wx[4], wy[4], wz[4];
    long gx[4], gy[4], gz[4];
    const int nx = lookRgtX - lookLftX + 1, ny = lookRgtY - lookLftY + 1, nz = lookRgtZ - lookLftZ + 1;
    if (nx > 4 || ny > 4 || nz > 4) return NAN;
    for (int a = 0; a < nx; a++) {
        const int i = lookLftX + a;
        double xx = fabs(X - (iX + i));
        wx[a] = xx < 0.5 ? (0.75 - xx * xx) : (xx < 1.5 ? 0.5 * (1.5 - xx) * (1.5 - xx) : 0);
        gx[a] = (long)N * (N + 2) * wrap1(iX + i, N);
    }
    for (int a = 0; a < ny; a++) {
        const int j = lookLftY + a;
        double yy = fabs(Y - (iY + j));
        wy[a] = yy < 0.5 ? (0.75 - yy * yy) : (yy < 1.5 ? 0.5 * (1.5 - yy) * (1.5 - yy) : 0);
        gy[a] = (N + 2) * wrap1(iY + j, N);
    }
    for (int a = 0; a < nz; a++) {
        const int k = lookLftZ + a;
        double zz = fabs(Z - (iZ + k));
        wz[a] = zz < 0.5 ? (0.75 - zz * zz) : (zz < 1.5 ? 0.5 * (1.5 - zz) * (1.5 - zz) : 0);
        gz[a] = wrap1(iZ + k, N);
    }
    double sum = 0;
    for (int a = 0; a < nx; a++)
        for (int b = 0; b < ny; b++)
            for (int c = 0; c < nz; c++) sum += box[gx[a] + gy[b] + gz[c]] * (wx[a] * wy[b] * wz[c]);
    return sum;
}

/* displacement loop for one direction: src/mitos.c:843-862.  The position used for the
 * gather of direction dir already carries the displacements of the earlier directions. */
void orc_displace(int M, int N, double boxlen, float *pos, const double *dbox, int dir) {
    const long n = (long)M * M * M;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        double disp = orc_tsc_gather(dbox, N, boxlen, x, y, z);
        pos[3 * i + dir] -= disp;
    }
}

/* fwrap of the positions: src/mitos.c:1072-1077 */
void orc_wrap_positions(long n, double boxlen, float *pos) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < 3 * n; i++) pos[i] = fmod(fmod(pos[i], boxlen) + boxlen, boxlen);
}

/* CIC deposit: analyse/src/mitos_read.c:278-334 (serial, particle order).  Returns the
 * total mass summed as the reference does (:307). */
double orc_cic_deposit(long n, const float *pos, double mass, int N, double boxlen, double *box) {
    double grid_cell_vol = boxlen * boxlen * boxlen / (N * N * N);
    double total_mass = 0;
    for (long l = 0; l < n; l++) {
        double x = fmod(fmod((double)pos[3 * l] * 1, boxlen) + boxlen, boxlen);
        double y = fmod(fmod((double)pos[3 * l + 1] * 1, boxlen) + boxlen, boxlen);
        double z = fmod(fmod((double)pos[3 * l + 2] * 1, boxlen) + boxlen, boxlen);
        double X = x / (boxlen / N);
        double Y = y / (boxlen / N);
        double Z = z / (boxlen / N);
        double Mp = mass;
        total_mass += Mp;
        int iX = (int)floor(X);
        int iY = (int)floor(Y);
        int iZ = (int)floor(Z);
        double dx = X - iX, dy = Y - iY, dz = Z - iZ;
        double tx = 1.0 - dx, ty = 1.0 - dy, tz = 1.0 - dz;
        double val = Mp / grid_cell_vol;
#define RM(i, j, k) ((wrap1(i, N) * N + wrap1(j, N)) * N + wrap1(k, N))
        box[RM(iX, iY, iZ)] += val * tx * ty * tz;
        box[RM(iX + 1, iY, iZ)] += val * dx * ty * tz;
        box[RM(iX, iY + 1, iZ)] += val * tx * dy * tz;
        box[RM(iX, iY, iZ + 1)] += val * tx * ty * dz;
        box[RM(iX + 1, iY + 1, iZ)] += val * dx * dy * tz;
        box[RM(iX + 1, iY, iZ + 1)] += val * dx * ty * dz;
        box[RM(iX, iY + 1, iZ + 1)] += val * tx * dy * dz;
        box[RM(iX + 1, iY + 1, iZ + 1)] += val * dx * dy * dz;
#undef RM
    }
    return total_mass;
}

/* overdensity: analyse/src/mitos_read.c:363-376 */
void orc_overdensity(int N, double boxlen, double total_mass, double *box) {
    double avg_density = total_mass / (boxlen * boxlen * boxlen);
    const long n = (long)N * N * N;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) box[i] = (box[i] - avg_density) / avg_density;
}

/* ===================================================================================== */
/* Power spectrum                                                                         */
/* ===================================================================================== */

static inline int log_bin_k(double k, int bins, double log_min_k, double log_max_k);

/* log bin of a mode whose integer wavevector has squared norm n2, with k = dk sqrt(n2):
 * src/calc_powerspec.c:36-63 (u rounded to float, bin = floor((bins - 1) * u)) */
int orc_log_bin(int N, double boxlen, int bins, long n2) {
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2;
    const double min_k = dk;
    return log_bin_k(sqrt((double)n2) * dk, bins, log(min_k), log(max_k));
}

static inline int log_bin_k(double k, int bins, double log_min_k, double log_max_k) {
    const float u = (log(k) - log_min_k) / (log_max_k - log_min_k);
    return floor((bins - 1) * u);
}

/* calc_bispectrum: src/calc_powerspec.c:295-508.  For each log bin i (k1 = k2 in bin i; k3 in the
 * bin of bins3 log bins picked by theta (type 0) or by the value k3 (type 1)), the field masked to
 * each shell (or ones in volume mode) to real space (c2r / V), and sum delta_1^2 delta_3 over the
 * N^3 cells.  Empty bins keep zeros.  (The reference also prints a line per bin.) */
void orc_bispectrum(int N, double boxlen, const double *fbox, int bins, int bins3, double *k1_in_bins,
                    double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode, int type,
                    double theta, double k3) {
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2;
    const double min_k = dk;
    const double log_max_k = log(max_k);
    const double log_min_k = log(min_k);
    for (int i = 0; i < bins; i++) { k1_in_bins[i] = 0; k2_in_bins[i] = 0; k3_in_bins[i] = 0; bispectrum[i] = 0; }
    const long H = N / 2 + 1, cn = (long)N * N * H;
    double *fbox1 = malloc(sizeof(double) * 2 * cn), *fbox3 = malloc(sizeof(double) * 2 * cn);
    double *m1 = malloc(sizeof(double) * N * N * (N + 2)), *m3 = malloc(sizeof(double) * N * N * (N + 2));
    for (int i = 0; i < bins; i++) {
        double k1_mean = 0., k3_mean = 0.;
        long long k1_obs = 0, k3_obs = 0;
        const int required_bin1 = i;
        int required_bin3;
        if (type == 0) {
            double k1 = exp((i + 0.5) * (log_max_k - log_min_k) / (bins3 - 1) + log_min_k);
            double k2 = exp((i + 0.5) * (log_max_k - log_min_k) / (bins3 - 1) + log_min_k);
            double required_k3 = sqrt(k1 * k1 + k2 * k2 + 2 * k1 * k2 * cos(theta));
            float u3 = (log(required_k3) - log_min_k) / (log_max_k - log_min_k);
            required_bin3 = floor((bins3 - 1) * u3);
        } else if (type == 1) {
            float u3 = (log(k3) - log_min_k) / (log_max_k - log_min_k);
            required_bin3 = floor((bins3 - 1) * u3);
        } else {
            required_bin3 = 0;
        }
        double kx, ky, kz, k;
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++)
                for (int z = 0; z <= N / 2; z++) {
                    orc_wavevector(x, y, z, N, dk, &kx, &ky, &kz, &k);
                    const long id = idx_half(N, x, y, z);
                    if (k == 0) {
                        fbox1[2 * id] = fbox1[2 * id + 1] = 0;
                        fbox3[2 * id] = fbox3[2 * id + 1] = 0;
                        continue;
                    }
                    const float u = (log(k) - log_min_k) / (log_max_k - log_min_k);
                    const int bin = floor((bins - 1) * u);
                    const int bin3 = floor((bins3 - 1) * u);
                    const int multiplicity = (z == 0 || z == N / 2) ? 1 : 2;
                    if (bin == required_bin1) {
                        fbox1[2 * id] = volume_mode ? 1.0 : fbox[2 * id];
                        fbox1[2 * id + 1] = volume_mode ? 0.0 : fbox[2 * id + 1];
                        k1_mean += multiplicity * k;
                        k1_obs += multiplicity;
                    } else {
                        fbox1[2 * id] = fbox1[2 * id + 1] = 0;
                    }
                    if (bin3 == required_bin3) {
                        fbox3[2 * id] = volume_mode ? 1.0 : fbox[2 * id];
                        fbox3[2 * id + 1] = volume_mode ? 0.0 : fbox[2 * id + 1];
                        k3_mean += multiplicity * k;
                        k3_obs += multiplicity;
                    } else {
                        fbox3[2 * id] = fbox3[2 * id + 1] = 0;
                    }
                }
        if (k1_obs == 0 || k3_obs == 0) continue;
        k1_mean /= k1_obs;
        k3_mean /= k3_obs;
        orc_fft_c2r(N, boxlen, fbox1, m1, N + 2);
        orc_fft_c2r(N, boxlen, fbox3, m3, N + 2);
        double sum = 0.;
        for (int x = 0; x < N; x++)
            for (int y = 0; y < N; y++)
                for (int z = 0; z < N; z++) {
                    const long id = ((long)x * N + y) * (N + 2) + z;
                    sum += m1[id] * m1[id] * m3[id];
                }
        bispectrum[i] = sum;
        k1_in_bins[i] = k1_mean;
        k2_in_bins[i] = k1_mean;
        k3_in_bins[i] = k3_mean;
    }
    free(fbox1);
    free(fbox3);
    free(m1);
    free(m3);
}

/* calc_cross_powerspec: src/calc_powerspec.c:32-90 */
void orc_powerspec_log(int N, double boxlen, const double *f1, const double *f2, int bins,
                       double *k_in_bins, double *power_in_bins, long *obs_in_bins) {
    const double boxvol = boxlen * boxlen * boxlen;
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2;
    const double min_k = dk;
    const double log_max_k = log(max_k);
    const double log_min_k = log(min_k);
    for (int i = 0; i < bins; i++) { k_in_bins[i] = 0; power_in_bins[i] = 0; obs_in_bins[i] = 0; }
    double kx, ky, kz, k;
    for (int x = 0; x < N; x++) {
        for (int y = 0; y < N; y++) {
            for (int z = 0; z <= N / 2; z++) {
                orc_wavevector(x, y, z, N, dk, &kx, &ky, &kz, &k);
                if (k == 0) continue;
                const int bin = log_bin_k(k, bins, log_min_k, log_max_k);
                if (bin < 0 || bin >= bins) continue;
                long id = idx_half(N, x, y, z);
                double a1 = f1[2 * id], a2 = f2[2 * id];
                double b1 = f1[2 * id + 1], b2 = f2[2 * id + 1];
                double Power = a1 * a2 + b1 * b2;
                int multiplicity = (z == 0 || z == N / 2) ? 1 : 2;
                k_in_bins[bin] += multiplicity * k;
                power_in_bins[bin] += multiplicity * Power;
                obs_in_bins[bin] += multiplicity;
            }
        }
    }
    for (int i = 0; i < bins; i++) {
        k_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= boxvol;
    }
}

static long isqrt_l(long a) {
    long r = (long)sqrt((double)a);
    while (r * r > a) r--;
    while ((r + 1) * (r + 1) <= a) r++;
    return r;
}

/* linear shells of width k_Nyquist / bins (a stated extension: the reference only has log
 * bins).  The shell index is computed from the integer wavevector so that every platform
 * and precision assigns modes identically: bin = isqrt(n2 * bins^2) / (N/2). */
int orc_lin_bin(int N, int bins, long n2) {
    long t = isqrt_l(n2 * (long)bins * bins);
    return (int)(t / (N / 2));
}

void orc_powerspec_lin(int N, double boxlen, const double *f1, const double *f2, int bins,
                       double *k_in_bins, double *power_in_bins, long *obs_in_bins) {
    const double boxvol = boxlen * boxlen * boxlen;
    const double dk = 2 * M_PI / boxlen;
    for (int i = 0; i < bins; i++) { k_in_bins[i] = 0; power_in_bins[i] = 0; obs_in_bins[i] = 0; }
    double kx, ky, kz, k;
    for (int x = 0; x < N; x++) {
        int nx = x > N / 2 ? x - N : x;
        for (int y = 0; y < N; y++) {
            int ny = y > N / 2 ? y - N : y;
            for (int z = 0; z <= N / 2; z++) {
                long n2 = (long)nx * nx + (long)ny * ny + (long)z * z;
                if (n2 == 0) continue;
                int bin = orc_lin_bin(N, bins, n2);
                if (bin >= bins) continue;
                orc_wavevector(x, y, z, N, dk, &kx, &ky, &kz, &k);
                long id = idx_half(N, x, y, z);
                double Power = f1[2 * id] * f2[2 * id] + f1[2 * id + 1] * f2[2 * id + 1];
                int multiplicity = (z == 0 || z == N / 2) ? 1 : 2;
                k_in_bins[bin] += multiplicity * k;
                power_in_bins[bin] += multiplicity * Power;
                obs_in_bins[bin] += multiplicity;
            }
        }
    }
    for (int i = 0; i < bins; i++) {
        k_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= boxvol;
    }
}

/* calc_cross_powerspec_float_mpi: src/calc_powerspec.c:152-217 on one rank (its three
 * MPI_Allreduce calls, :203-205, leave the slab's sums unchanged).  The slab's row x - X0 holds
 * the modes of x (row_major_half_mpi); the float components are widened to double before the
 * products. */
void orc_powerspec_float_slab(long N, long X0, long NX, double boxlen, const float *box1, const float *box2,
                              int bins, double *k_in_bins, double *power_in_bins, long *obs_in_bins) {
    const double boxvol = boxlen * boxlen * boxlen;
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2;
    const double min_k = dk;
    const double log_max_k = log(max_k);
    const double log_min_k = log(min_k);
    for (int i = 0; i < bins; i++) { k_in_bins[i] = 0; power_in_bins[i] = 0; obs_in_bins[i] = 0; }
    double kx, ky, kz, k;
    for (long x = X0; x < X0 + NX; x++) {
        for (long y = 0; y < N; y++) {
            for (long z = 0; z <= N / 2; z++) {
                orc_wavevector((int)x, (int)y, (int)z, (int)N, dk, &kx, &ky, &kz, &k);
                if (k == 0) continue;
                const int bin = log_bin_k(k, bins, log_min_k, log_max_k);
                if (bin < 0 || bin >= bins) continue;
                const long id = ((x - X0) * N + y) * (N / 2 + 1) + z;
                double a1 = box1[2 * id], a2 = box2[2 * id];
                double b1 = box1[2 * id + 1], b2 = box2[2 * id + 1];
                double Power = a1 * a2 + b1 * b2;
                int multiplicity = (z == 0 || z == N / 2) ? 1 : 2;
                k_in_bins[bin] += multiplicity * k;
                power_in_bins[bin] += multiplicity * Power;
                obs_in_bins[bin] += multiplicity;
            }
        }
    }
    for (int i = 0; i < bins; i++) {
        k_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= obs_in_bins[i];
        power_in_bins[i] /= boxvol;
    }
}

/* ===================================================================================== */
/* The initial-condition pipeline                                                         */
/* ===================================================================================== */

int orc_ic_pipeline(const struct orc_ic_params *p, struct orc_ic_out *o) {
    const int N = p->N, M = p->M;
    const double L = p->boxlen;
    const long cbytes = (long)N * N * (N / 2 + 1) * 2 * sizeof(double);
    struct orc_grid grf, grid, pot, der;
    if (orc_grid_alloc(&grf, N, L) || orc_grid_alloc(&grid, N, L) || orc_grid_alloc(&pot, N, L) ||
        orc_grid_alloc(&der, N, L))
        return 5;

    /* src/mitos.c:216-227: noise, Hermitian symmetry, primordial power, to real space */
    orc_generate_grf(N, L, p->seed, grf.fbox);
    grf.momentum_space = 1;
    orc_enforce_hermiticity(N, grf.fbox);
    grid_kernel(&grf, &grf, ORC_K_POWER_NO_TRANSFER, &p->cosmo);
    if (o->grf) memcpy(o->grf, grf.fbox, cbytes);
    orc_grid_c2r(&grf);
    /* :300 back to momentum space */
    orc_grid_r2c(&grf);

    /* :357-367 generatePerturbationGrid (src/generate_grids.c:28-67) with z_source = z_ini */
    double log_tau_src = orc_log_tau_at_redshift(p->sp, p->z_ini);
    struct orc_transfer_params tp;
    tp.sp = p->sp;
    tp.index_src = p->index_src;
    orc_spline_find_tau(p->sp, log_tau_src, &tp.tau_index, &tp.u_tau);
    grid_kernel(&grid, &grf, ORC_K_TRANSFER, &tp);
    if (o->delta_k) memcpy(o->delta_k, grid.fbox, cbytes);
    orc_grid_c2r(&grid);
    /* :377 */
    orc_grid_r2c(&grid);

    /* :380-389 */
    if (p->ma_cycles > 0) {
        orc_solve_ma(&pot, &grid, &der, p->ma_cycles, o->ma_eps, NULL);
    } else if (p->lpt_order == 2) {
        orc_solve_2lpt(&pot, &grid, &der, 1.0, -3. / 7.);
    } else {
        grid_kernel(&pot, &grid, ORC_K_INV_POISSON, NULL);
    }
    if (o->phi_k) memcpy(o->phi_k, pot.fbox, cbytes);

    /* :425-490 the velocity grids (flux density of the velocity transfer function, its potential,
     * three derivatives), computed after the displacement grids below from a copy of pot */
    struct orc_hermite_params hp = {3, N, L};
    grid_kernel(&pot, &pot, ORC_K_UNDO_HERMITE, &hp);
    double *disp[3];
    static const int kid[3] = {ORC_K_DX, ORC_K_DY, ORC_K_DZ};
    for (int i = 0; i < 3; i++) {
        disp[i] = malloc(cbytes);
        grid_kernel(&der, &pot, kid[i], NULL);
        orc_grid_c2r(&der);
        memcpy(disp[i], der.box, cbytes);
        if (o->disp[i]) memcpy(o->disp[i], der.box, cbytes);
    }
    /* :419 */
    orc_grid_c2r(&pot);

    /* :425-490 velocity grids: generatePerturbationGrid with the velocity title (rescale 1 with
     * z_source = z_ini, :431-436), r2c (:451), 2LPT with the reference's velocity factors (:453-455)
     * or the inverse Poisson kernel (:457), TSC window undo (:461-467), three derivatives (:470-483) */
    double *vgrid[3] = {NULL, NULL, NULL};
    if (p->index_vel >= 0) {
        struct orc_transfer_params tv;
        tv.sp = p->sp;
        tv.index_src = p->index_vel;
        orc_spline_find_tau(p->sp, log_tau_src, &tv.tau_index, &tv.u_tau);
        grid_kernel(&grid, &grf, ORC_K_TRANSFER, &tv);
        orc_grid_c2r(&grid);
        orc_grid_r2c(&grid);
        if (p->lpt_order == 2 && p->ma_cycles <= 0)
            orc_solve_2lpt(&pot, &grid, &der, -0.001147273637728, 3.19354920304769E-05);
        else
            grid_kernel(&pot, &grid, ORC_K_INV_POISSON, NULL);
        struct orc_hermite_params hv = {3, N, L};
        grid_kernel(&pot, &pot, ORC_K_UNDO_HERMITE, &hv);
        for (int i = 0; i < 3; i++) {
            vgrid[i] = malloc(cbytes);
            grid_kernel(&der, &pot, kid[i], NULL);
            orc_grid_c2r(&der);
            memcpy(vgrid[i], der.box, cbytes);
        }
    }
    orc_grid_free(&grf);
    orc_grid_free(&grid);
    orc_grid_free(&pot);
    orc_grid_free(&der);

    /* particle stage: :794 lattice, :827-863 displacements, :1072-1077 wrap */
    const long np = (long)M * M * M;
    int thermal_err = 0;
    float *pos = malloc(sizeof(float) * 3 * np);
    orc_lattice(M, L, pos);
    for (int dir = 0; dir < 3; dir++) orc_displace(M, N, L, pos, disp[dir], dir);
    /* :865-908 velocities: the TSC gather of each velocity grid at the displaced (not yet wrapped)
     * position, stored as float */
    if (p->index_vel >= 0) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < np; i++) {
            const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
            for (int dir = 0; dir < 3; dir++) {
                const double v = orc_tsc_gather(vgrid[dir], N, L, x, y, z);
                if (o->vel) o->vel[3 * i + dir] = (float)v;
            }
        }
        for (int i = 0; i < 3; i++) free(vgrid[i]);
        /* :910-1064 thermal motion (no Firebolt) on top, from the stream the white noise left:
         * four draws a mode with k > 0 (src/grf.c:47-63), then those of earlier thermal species */
        if (p->thermal > 0 && o->vel) {
            uint64_t st[4];
            orc_rng_init(p->seed, st);
            orc_rng_advance(st, 4 * ((uint64_t)N * N * (N / 2 + 1) - 1) + p->thermal_draw_offset);
            struct orc_sampler ts;
            thermal_err = orc_sampler_init(&ts, p->thermal, p->thermal_T_eV, 0.0);
            if (!thermal_err)
                thermal_err = orc_thermal_velocities(&ts, st, np, p->thermal_M_eV, 1.0 / (1.0 + p->z_ini),
                                                     p->speed_of_light, o->vel, 3);
            orc_sampler_free(&ts);
        }
    }
    orc_wrap_positions(np, L, pos);
    for (int i = 0; i < 3; i++) free(disp[i]);
    if (o->pos) memcpy(o->pos, pos, sizeof(float) * 3 * np);

    /* analyse/src/mitos_read.c:278-419: CIC, overdensity, r2c, CIC undo, P(k) */
    double *rho = calloc((size_t)N * N * N, sizeof(double));
    float mass_f = (float)p->mass;
    double total_mass = orc_cic_deposit(np, pos, (double)mass_f, N, L, rho);
    free(pos);
    orc_overdensity(N, L, total_mass, rho);
    if (o->rho) memcpy(o->rho, rho, sizeof(double) * N * N * N);
    double *fbox = malloc(cbytes);
    orc_fft_r2c(N, L, rho, N, fbox);
    free(rho);
    struct orc_hermite_params hc = {2, N, L};
    orc_apply_kernel(N, L, fbox, fbox, ORC_K_UNDO_HERMITE, &hc);
    if (p->pk_linear)
        orc_powerspec_lin(N, L, fbox, fbox, p->pk_bins, o->pk_k, o->pk_p, o->pk_obs);
    else
        orc_powerspec_log(N, L, fbox, fbox, p->pk_bins, o->pk_k, o->pk_p, o->pk_obs);
    free(fbox);
    return thermal_err;
}
