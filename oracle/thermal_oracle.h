/*
 * thermal_oracle.h -- CPU restatement of the thermal-motion sampler of Mitos.  TEST
 * INFRASTRUCTURE: the checker for the GPU thermal velocities; nothing in the library links it.
 */
#ifndef THERMAL_ORACLE_H
#define THERMAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_FERMION 1 /* Fermi-Dirac, src/random.c:52-60 */
#define ORC_BOSON 2   /* Bose-Einstein, src/random.c:63-71 */

/* one piece of the inverse CDF: x(u~) = a0 + a1 u~ + a2 u~^2 + a3 u~^3 on [Fl, Fr] */
struct orc_piece {
    double l, r, Fl, Fr;
    double a0, a1, a2, a3;
    int next; /* right neighbour while building; unused once sorted */
};

struct orc_sampler {
    int kind;
    double T, mu, xl, xr, norm;
    int n;                   /* pieces, sorted by Fl */
    struct orc_piece *piece;
    int table_len;           /* 1000 */
    int *table;              /* piece to start the scan from, per u = i / table_len */
};

double orc_thermal_pdf(int kind, double T, double mu, double x);
int orc_sampler_init(struct orc_sampler *s, int kind, double T_eV, double mu_eV);
void orc_sampler_free(struct orc_sampler *s);
double orc_sampler_draw(const struct orc_sampler *s, uint64_t st[4]);
/* n particles in id order: vel[i*stride + c] += (float) n_c V, 7 draws a particle from st.
 * Returns 0, or 1 for an invalid momentum (src/mitos.c:939-942). */
int orc_thermal_velocities(const struct orc_sampler *s, uint64_t st[4], long n, double M_eV,
                           double a_ini, double speed_of_light, float *vel, long stride);

/* flat exports for ctypes: pieces as rows [l r Fl Fr a0 a1 a2 a3] */
int orc_sampler_table(int kind, double T_eV, int max, double *rows, int *table, double *norm);
int orc_sampler_draws(int kind, double T_eV, const uint64_t st0[4], long n, double *out);
int orc_thermal(int kind, double T_eV, double M_eV, double a_ini, double speed_of_light,
                const uint64_t st0[4], long n, float *vel, long stride);

#ifdef __cplusplus
}
#endif
#endif
