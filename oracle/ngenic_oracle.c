/*
 * ngenic_oracle.c -- CPU restatement of generate_ngeniclike_grf (src/grf_ngeniclike.c:28-203) and
 * of the random generator it uses, GSL's gsl_rng_ranlxd1 (GSL version unpinned: the reference
 * links -lgsl, Makefile:9, with no lockfile).
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the GPU kernel).  PARITY UNPINNED: GSL is not on this
 * image and the reference ships no test of this path, so the generator below follows Luscher's
 * published double-precision RANLUX ("ranlxd", luxury level 1: 202 numbers per block of which
 * the last 12 are delivered) as described in M. Luscher, Comput. Phys. Commun. 79 (1994) 100 and
 * his ranlxd notes; it has not been compared with libgsl output.
 *
 * Generator restated here (all values integers in [0, 2^48), output x / 2^48):
 *   state: 12 words x[0..11], carry c in {0, 1}
 *   step (subtract with borrow, lags 5 and 12): y = x[j] - x[i] - c, c = (y < 0), y += 2^48 c,
 *        x[i] = y, i = i + 1 mod 12, j = j + 1 mod 12   (j = i - 5 mod 12)
 *   block: 202 steps; the delivered numbers are the state words in age order after the block
 *   seeding from s (s = 0 -> 1): a 31-bit shift register b[0..30] holds the low 31 bits of s;
 *        each of the 48 bits of each of the 12 words is 1 - b[p], and b[p] ^= b[p + 18 mod 31],
 *        p = p + 1 mod 31 (starting at p = 0); carry 0
 */
#include "ngenic_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define W48 (1ULL << 48)

void orc_ranlxd1_set(struct orc_ranlxd *r, unsigned long seed) {
    if (seed == 0) seed = 1;
    int b[31];
    unsigned long s = seed & 0xFFFFFFFFUL;
    for (int k = 0; k < 31; k++) {
        b[k] = (int)(s & 1);
        s >>= 1;
    }
    int p = 0, q = 18;
    for (int k = 0; k < 12; k++) {
        uint64_t x = 0;
        for (int l = 0; l < 48; l++) {
            x = 2 * x + (uint64_t)(1 - b[p]);
            b[p] = (b[p] + b[q]) % 2;
            p = (p + 1) % 31;
            q = (q + 1) % 31;
        }
        r->x[k] = x;
    }
    r->carry = 0;
    r->i = 0;      /* oldest word: the next step overwrites it */
    r->left = 0;   /* words still to deliver from the current block */
}

static void block(struct orc_ranlxd *r) {
    for (int k = 0; k < 202; k++) {
        const int i = r->i, j = (i + 7) % 12;
        int64_t y = (int64_t)r->x[j] - (int64_t)r->x[i] - (int64_t)r->carry;
        r->carry = y < 0;
        if (y < 0) y += (int64_t)W48;
        r->x[i] = (uint64_t)y;
        r->i = (i + 1) % 12;
    }
    r->left = 12;
}

double orc_ranlxd1_uniform(struct orc_ranlxd *r) {
    if (r->left == 0) block(r);
    /* age order: the oldest word sits at the next index to overwrite */
    const int k = (r->i + (12 - r->left)) % 12;
    r->left--;
    return (double)r->x[k] / (double)W48;
}

/* src/grf_ngeniclike.c:68-88: the seed table in the reference's mirrored fill order */
void orc_ngenic_seedtable(int N, unsigned long seed, unsigned int *table) {
    struct orc_ranlxd r;
    orc_ranlxd1_set(&r, seed);
    memset(table, 0, sizeof(unsigned int) * (size_t)N * N);
#define U ((unsigned int)(0x7fffffff * orc_ranlxd1_uniform(&r)))
    for (int i = 0; i < N / 2; i++) {
        for (int j = 0; j < i; j++) table[i * N + j] = U;
        for (int j = 0; j < i + 1; j++) table[j * N + i] = U;
        for (int j = 0; j < i; j++) table[(N - 1 - i) * N + j] = U;
        for (int j = 0; j < i + 1; j++) table[(N - 1 - j) * N + i] = U;
        for (int j = 0; j < i; j++) table[i * N + (N - 1 - j)] = U;
        for (int j = 0; j < i + 1; j++) table[j * N + (N - 1 - i)] = U;
        for (int j = 0; j < i; j++) table[(N - 1 - i) * N + (N - 1 - j)] = U;
        for (int j = 0; j < i + 1; j++) table[(N - 1 - j) * N + (N - 1 - i)] = U;
    }
#undef U
}

/* src/grf_ngeniclike.c:28-203 on one rank (NX = N, X0 = 0).  The reference repeats the whole
 * fill for three axes (:90) with identical results; it is done once here. */
int orc_ngeniclike_grf(int N, double boxlen, unsigned long seed, double *fbox) {
    const int H = N / 2 + 1;
    unsigned int *table = malloc(sizeof(unsigned int) * (size_t)N * N);
    if (!table) return 4;
    orc_ngenic_seedtable(N, seed, table);
    double fac = pow(boxlen, 1.5) / sqrt(2);  /* :60 */
    fac *= sqrt(2);                             /* :62 */
    memset(fbox, 0, sizeof(double) * 2 * (size_t)N * N * H);
    for (int i = 0; i < N; i++) {
        for (int j = 0; j < N; j++) {
            struct orc_ranlxd r;
            orc_ranlxd1_set(&r, table[i * N + j]);
            for (int k = 0; k < N / 2; k++) {
                const double phase = orc_ranlxd1_uniform(&r) * 2 * M_PI;
                double ampl;
                do ampl = orc_ranlxd1_uniform(&r);
                while (ampl == 0);
                if (i == N / 2 || j == N / 2 || k == N / 2) continue;
                if (i == 0 && j == 0 && k == 0) continue;
                const double delta = fac * sqrt(-log(ampl));  /* p_of_k = 1, Dplus = 1 */
                const double re = delta * sin(phase), im = delta * cos(phase);
                if (k > 0) {
                    double *c = fbox + 2 * (((size_t)i * N + j) * H + k);
                    c[0] = re;
                    c[1] = im;
                } else if (i == 0) {
                    if (j >= N / 2) continue;
                    const int jj = N - j;
                    double *c = fbox + 2 * (((size_t)i * N + j) * H);
                    c[0] = re;
                    c[1] = im;
                    c = fbox + 2 * (((size_t)i * N + jj) * H);
                    c[0] = re;
                    c[1] = -im;
                } else {
                    if (i >= N / 2) continue;
                    const int ii = N - i, jj = (N - j) % N;
                    double *c = fbox + 2 * (((size_t)i * N + j) * H);
                    c[0] = re;
                    c[1] = im;
                    c = fbox + 2 * (((size_t)ii * N + jj) * H);
                    c[0] = re;
                    c[1] = -im;
                }
            }
        }
    }
    free(table);
    return 0;
}
