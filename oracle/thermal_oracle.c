/*
 * thermal_oracle.c -- CPU restatement of the thermal-motion sampler of Mitos.  TEST
 * INFRASTRUCTURE: the checker for the GPU thermal velocities; nothing in the library links it.
 *
 *   orc_thermal_pdf         fd_pdf / be_pdf, src/random.c:52-71
 *   orc_sampler_init        initSampler, src/random.c:87-209, with numericalCDF (:74-84) and
 *                           splitInterval (:212-251); constants include/random.h:35-39
 *   orc_sampler_draw        samplerCustom, src/random.c:261-289
 *   orc_thermal_velocities  the thermal-motion loop of src/mitos.c:928-965 and :1054-1062 (the
 *                           branch without Firebolt: every draw accepted)
 *
 * The inverse CDF is cut into pieces until each holds at most 5% of the probability, then each
 * piece gets the cubic Hermite interpolant of x(F) from the CDF and the pdf at its ends and is
 * halved again while the interpolant is not monotone or misses the CDF by more than 1e-6 at the
 * midpoint.  Which pieces get cut depends only on each piece's own ends, so the final set does
 * not depend on the order of the walk.  Pieces end up sorted by Fl.
 *
 * Two properties of the reference draw are kept as they are:
 *   - the start table holds, for u_i = i / 1000, the piece with the largest right end among
 *     those with Fr < u_i (the piece BEFORE the one holding u_i);
 *   - the scan from there keeps the last consecutive piece with Fr < u, so a draw in piece j > 0
 *     usually evaluates piece j - 1's cubic beyond its right end (u~ > 1).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mitos_oracle.h"
#include "thermal_oracle.h"

#define CDF_SAMPLES 1000 /* NUMERICAL_CDF_SAMPLES */
#define TABLE_LEN 1000   /* SEARCH_TABLE_LENGTH */
#define P_MIN 1e-10      /* THERMAL_MIN_MOMENTUM, units of kT */
#define P_MAX 15.0       /* THERMAL_MAX_MOMENTUM, units of kT */

double orc_thermal_pdf(int kind, double T, double mu, double x) {
    if (x <= 0) return 0;
    const double e = exp((x - mu) / T);
    return x * x / (kind == ORC_BOSON ? e - 1 : e + 1);
}

/* midpoint rule on CDF_SAMPLES cells of [a, b] */
static double midpoint(const struct orc_sampler *s, double a, double b) {
    const double h = (b - a) / CDF_SAMPLES;
    double sum = 0;
    for (int i = 0; i < CDF_SAMPLES; i++) sum += h * orc_thermal_pdf(s->kind, s->T, s->mu, a + (i + 0.5) * h);
    return sum;
}

static double cdf(const struct orc_sampler *s, double x) { return s->norm * midpoint(s, s->xl, x); }

static int cut(struct orc_sampler *s, int *cap, int j) {
    if (s->n == *cap) {
        *cap *= 2;
        struct orc_piece *np = realloc(s->piece, sizeof(struct orc_piece) * (size_t)*cap);
        if (!np) return 1;
        s->piece = np;
    }
    struct orc_piece *p = &s->piece[j];
    const double m = p->l + 0.5 * (p->r - p->l);
    const double Fm = cdf(s, m);
    struct orc_piece *q = &s->piece[s->n];
    memset(q, 0, sizeof *q);
    q->l = m;
    q->r = p->r;
    q->Fl = Fm;
    q->Fr = p->Fr;
    q->next = p->next;
    p->r = m;
    p->Fr = Fm;
    p->next = s->n;
    s->n++;
    return 0;
}

static int by_Fl(const void *a, const void *b) {
    const double x = ((const struct orc_piece *)a)->Fl, y = ((const struct orc_piece *)b)->Fl;
    return (x > y) - (x < y);
}

int orc_sampler_init(struct orc_sampler *s, int kind, double T_eV, double mu_eV) {
    memset(s, 0, sizeof *s);
    if (kind != ORC_FERMION && kind != ORC_BOSON) return 1;
    s->kind = kind;
    s->T = T_eV;
    s->mu = mu_eV;
    s->xl = P_MIN * T_eV;
    s->xr = P_MAX * T_eV;
    s->norm = 1.0 / midpoint(s, s->xl, s->xr);
    int cap = 64;
    s->piece = calloc((size_t)cap, sizeof(struct orc_piece));
    if (!s->piece) return 1;
    s->n = 1;
    s->piece[0].l = s->xl;
    s->piece[0].r = s->xr;
    s->piece[0].Fl = 0.0;
    s->piece[0].Fr = 1.0;
    s->piece[0].next = -1;

    /* pass 1: at most 5% of the probability a piece */
    for (int j = 0;;) {
        struct orc_piece *p = &s->piece[j];
        if (p->Fr - p->Fl > 0.05) {
            if (cut(s, &cap, j)) return 1;
        } else if (p->r >= s->xr) {
            break;
        } else {
            j = p->next;
        }
    }
    /* pass 2: monotone cubic Hermite interpolants within 1e-6 at the midpoint */
    for (int j = 0;;) {
        struct orc_piece *p = &s->piece[j];
        const double fl = s->norm * orc_thermal_pdf(kind, T_eV, mu_eV, p->l);
        const double fr = s->norm * orc_thermal_pdf(kind, T_eV, mu_eV, p->r);
        const double dF = p->Fr - p->Fl;
        p->a0 = p->l;
        p->a1 = dF / fl;
        p->a2 = 3 * (p->r - p->l) - dF * (2. / fl + 1. / fr);
        p->a3 = 2 * (p->l - p->r) + dF * (1. / fl + 1. / fr);
        const double xmid = p->a0 + p->a1 * 0.5 + p->a2 * 0.25 + p->a3 * 0.125;
        const double miss = fabs(cdf(s, xmid) - 0.5 * (p->Fr + p->Fl));
        const double slope = dF / (p->r - p->l);
        const int monotone = slope <= 3 * fl && slope <= 3 * fr;
        if (miss > 1e-6 || !monotone) {
            if (cut(s, &cap, j)) return 1;
        } else if (p->r >= s->xr) {
            break;
        } else {
            j = p->next;
        }
    }
    qsort(s->piece, (size_t)s->n, sizeof(struct orc_piece), by_Fl);

    s->table_len = TABLE_LEN;
    s->table = malloc(sizeof(int) * TABLE_LEN);
    if (!s->table) return 1;
    for (int i = 0; i < TABLE_LEN; i++) {
        const double u = (double)i / TABLE_LEN;
        double rmax = 0;
        int best = 0;
        for (int j = 0; j < s->n; j++)
            if (s->piece[j].Fr < u && s->piece[j].r > rmax) {
                rmax = s->piece[j].r;
                best = j;
            }
        s->table[i] = best;
    }
    return 0;
}

void orc_sampler_free(struct orc_sampler *s) {
    free(s->piece);
    free(s->table);
    memset(s, 0, sizeof *s);
}

double orc_sampler_draw(const struct orc_sampler *s, uint64_t st[4]) {
    const uint64_t w = orc_rng_next(st);
    const double u = (double)w / (double)UINT64_MAX; /* (double)UINT64_MAX is 2^64 */
    const int t = (int)floor(u * s->table_len);
    int j = s->table[t < s->table_len ? t : s->table_len - 1];
    int pick = j;
    double rmax = 0;
    for (; j < s->n && s->piece[j].Fr < u && s->piece[j].r > rmax; j++) {
        rmax = s->piece[j].r;
        pick = j;
    }
    const struct orc_piece *p = &s->piece[pick];
    const double v = (u - p->Fl) / (p->Fr - p->Fl);
    return p->a0 + p->a1 * v + p->a2 * v * v + p->a3 * v * v * v;
}

int orc_thermal_velocities(const struct orc_sampler *s, uint64_t st[4], long n, double M_eV,
                           double a_ini, double speed_of_light, float *vel, long stride) {
    for (long i = 0; i < n; i++) {
        const double p = orc_sampler_draw(s, st) / a_ini; /* momentum at a_ini */
        if (isnan(p) || p <= 0) return 1;
        const double V = p / M_eV * speed_of_light;
        double d[3];
        for (int c = 0; c < 3; c++) d[c] = orc_sample_norm(st);
        const double len = hypot(d[0], hypot(d[1], d[2]));
        if (len > 0)
            for (int c = 0; c < 3; c++) d[c] /= len;
        float *v = vel + i * stride;
        for (int c = 0; c < 3; c++) v[c] = (float)(v[c] + d[c] * V);
    }
    return 0;
}

int orc_sampler_table(int kind, double T_eV, int max, double *rows, int *table, double *norm) {
    struct orc_sampler s;
    if (orc_sampler_init(&s, kind, T_eV, 0.0)) {
        orc_sampler_free(&s);
        return -1;
    }
    const int n = s.n;
    for (int j = 0; j < n && j < max; j++) {
        const struct orc_piece *p = &s.piece[j];
        const double r[8] = {p->l, p->r, p->Fl, p->Fr, p->a0, p->a1, p->a2, p->a3};
        memcpy(rows + 8 * j, r, sizeof r);
    }
    if (table) memcpy(table, s.table, sizeof(int) * TABLE_LEN);
    if (norm) *norm = s.norm;
    orc_sampler_free(&s);
    return n;
}

int orc_sampler_draws(int kind, double T_eV, const uint64_t st0[4], long n, double *out) {
    struct orc_sampler s;
    if (orc_sampler_init(&s, kind, T_eV, 0.0)) {
        orc_sampler_free(&s);
        return 1;
    }
    uint64_t st[4];
    memcpy(st, st0, sizeof st);
    for (long i = 0; i < n; i++) out[i] = orc_sampler_draw(&s, st);
    orc_sampler_free(&s);
    return 0;
}

int orc_thermal(int kind, double T_eV, double M_eV, double a_ini, double speed_of_light,
                const uint64_t st0[4], long n, float *vel, long stride) {
    struct orc_sampler s;
    if (orc_sampler_init(&s, kind, T_eV, 0.0)) {
        orc_sampler_free(&s);
        return 1;
    }
    uint64_t st[4];
    memcpy(st, st0, sizeof st);
    const int e = orc_thermal_velocities(&s, st, n, M_eV, a_ini, speed_of_light, vel, stride);
    orc_sampler_free(&s);
    return e;
}
