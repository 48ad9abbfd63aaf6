/*
 * mitos_oracle.h -- CPU restatement (FP64) of the Mitos initial-condition hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path: only the
 * test-suite, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may
 * load it.  The GPU library never links or calls it.
 *
 * Every function restates one piece of the reference (wullm/mitos) and cites the file and
 * line it follows.  Complex arrays are interleaved (re, im) doubles in the reference layout
 * N x N x (N/2+1); padded real arrays are N x N x (N+2) doubles (the layout of
 * struct distributed_grid, include/distributed_grid.h:29-60); unpadded real arrays are N^3.
 * All loops assume one rank (NX = N, X0 = 0).
 */
#ifndef MITOS_ORACLE_H
#define MITOS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- random numbers: include/random_xorshift.h, src/random.c --------------------- */
void     orc_rng_init(uint64_t seed, uint64_t s[4]);
uint64_t orc_rng_next(uint64_t s[4]);
void     orc_rng_advance(uint64_t s[4], uint64_t n);
double   orc_sample_uniform(uint64_t s[4]);
double   orc_sample_norm(uint64_t s[4]);
void     orc_draws(uint64_t seed, int64_t n, uint64_t *out);
void     orc_norms(uint64_t seed, int64_t n, double *out);

/* ---- white noise: src/grf.c ------------------------------------------------------- */
int orc_generate_grf(int N, double boxlen, uint64_t seed, double *fbox);
int orc_enforce_hermiticity(int N, double *fbox);

/* ---- FFT with FFTW conventions (unnormalised) and the Mitos normalisation ---------- */
/* rpitch = row length of the real array: N (serial FFTW arrays) or N+2 (padded grids) */
int orc_dft_r2c_3d(int N, const double *in, long rpitch, double *out);
int orc_dft_c2r_3d(int N, double *in_destroyed, double *out, long rpitch);
int orc_fft_r2c(int N, double boxlen, const double *box, long rpitch, double *fbox);
int orc_fft_c2r(int N, double boxlen, double *fbox_destroyed, double *box, long rpitch);
int orc_fft_1d(int n, int sign, double *data); /* complex, in place, unnormalised */

/* ---- perturbation table + spline: include/perturb_data.h, src/perturb_spline.c ---- */
struct orc_perturb {
    int k_size, tau_size, n_functions;
    const double *k, *log_tau, *redshift, *D_growth, *f_growth, *H_Hubble;
    const double *delta; /* [n_functions][tau_size][k_size] */
    int k_acc_size;
    double *k_acc;       /* acceleration table (indices stored as double, as the reference does) */
};
int    orc_spline_init(struct orc_perturb *sp, int k_acc_size);
void   orc_spline_free(struct orc_perturb *sp);
void   orc_spline_find_tau(const struct orc_perturb *sp, double log_tau, int *index, double *u);
void   orc_spline_find_k(const struct orc_perturb *sp, double k, int *index, double *u);
double orc_spline_interp(const struct orc_perturb *sp, int k_index, int tau_index, double u_k,
                         double u_tau, int index_src);
double orc_log_tau_at_redshift(const struct orc_perturb *sp, double z);
double orc_growth_at_log_tau(const struct orc_perturb *sp, double log_tau);

/* ---- k-space kernels: include/fft_kernels.h + src/fft.c:257-302 -------------------- */
enum orc_kernel_id {
    ORC_K_CONSTANT = 0, ORC_K_LOWPASS, ORC_K_HIPASS, ORC_K_TOPHAT, ORC_K_ELLIPTIC_TOPHAT,
    ORC_K_TRANSLATE, ORC_K_GAUSSIAN, ORC_K_GAUSSIAN_INV, ORC_K_INV_POISSON, ORC_K_DX,
    ORC_K_DY, ORC_K_DZ, ORC_K_POWER_NO_TRANSFER, ORC_K_TRANSFER, ORC_K_INV_TRANSFER,
    ORC_K_UNDO_HERMITE
};
struct orc_cosmo { double A_s, n_s, k_pivot; };
struct orc_transfer_params { const struct orc_perturb *sp; int index_src; int tau_index; double u_tau; };
struct orc_hermite_params { int order; int N; double boxlen; };
void   orc_wavevector(int x, int y, int z, int N, double dk, double *kx, double *ky, double *kz,
                      double *k);
double orc_primordial_power(double k, const struct orc_cosmo *c);
int    orc_apply_kernel(int N, double boxlen, double *write, const double *read, int kernel_id,
                        const void *params);

/* ---- solvers: src/poisson.c, src/2lpt.c, src/monge_ampere.c ------------------------ */
/* Grids: fbox (complex) + box (padded real), momentum-space flags as the reference.    */
struct orc_grid { int N; double boxlen; int momentum_space; double *fbox; double *box; };
int orc_grid_alloc(struct orc_grid *g, int N, double boxlen);
void orc_grid_free(struct orc_grid *g);
int orc_grid_r2c(struct orc_grid *g);
int orc_grid_c2r(struct orc_grid *g);
int orc_solve_poisson(struct orc_grid *g);
int orc_solve_2lpt(struct orc_grid *pot, struct orc_grid *dens, struct orc_grid *work,
                   double f1, double f2);
int orc_solve_ma(struct orc_grid *pot, struct orc_grid *dens, struct orc_grid *work, int cycles,
                 double *eps_out /* [cycles] reference eps, may be NULL */,
                 double *rel_out /* [cycles] sqrt(sum res^2 / sum rho^2) over cells, may be NULL */);

/* ---- particles, interpolation, CIC: src/particle.c, src/grids_interp.c,
 *      src/mitos.c:827-863,1072-1077, analyse/src/mitos_read.c:278-376 -------------- */
void   orc_lattice(int M, double boxlen, float *pos /* M^3 x 3 */);
double orc_tsc_gather(const double *box, int N, double boxlen, double x, double y, double z);
void   orc_displace(int M, int N, double boxlen, float *pos, const double *dbox, int dir);
void   orc_wrap_positions(long n, double boxlen, float *pos);
double orc_cic_deposit(long n, const float *pos, double mass, int N, double boxlen,
                       double *rho /* N^3 unpadded, accumulated into */);
void   orc_overdensity(int N, double boxlen, double total_mass, double *rho);

/* ---- power spectrum: src/calc_powerspec.c:32-90 and linear shells ------------------ */
void orc_powerspec_log(int N, double boxlen, const double *f1, const double *f2, int bins,
                       double *k_in_bins, double *power_in_bins, long *obs_in_bins);
void orc_powerspec_lin(int N, double boxlen, const double *f1, const double *f2, int bins,
                       double *k_in_bins, double *power_in_bins, long *obs_in_bins);
int  orc_lin_bin(int N, int bins, long n2);
/* calc_cross_powerspec_float_mpi (src/calc_powerspec.c:152-217) on one rank: float boxes holding
 * the x-slab X0 .. X0+NX-1, log bins over that slab's modes */
void orc_powerspec_float_slab(long N, long X0, long NX, double boxlen, const float *box1, const float *box2,
                              int bins, double *k_in_bins, double *power_in_bins, long *obs_in_bins);
void orc_bispectrum(int N, double boxlen, const double *fbox, int bins, int bins3, double *k1_in_bins,
                    double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode, int type,
                    double theta, double k3);
int  orc_log_bin(int N, double boxlen, int bins, long n2);

/* ---- the whole initial-condition pipeline (src/mitos.c:205-422,794-863 followed by
 *      analyse/src/mitos_read.c:278-419) ------------------------------------------------ */
struct orc_ic_params {
    int N, M;
    double boxlen;
    uint64_t seed;
    struct orc_cosmo cosmo;
    const struct orc_perturb *sp;
    int index_src;
    double z_ini;
    int lpt_order;      /* 1 = Zel'dovich, 2 = 2LPT */
    int ma_cycles;      /* > 0: Monge-Ampere instead of 2LPT */
    int pk_bins;
    int pk_linear;      /* 1 = linear shells to k_Nyquist, 0 = reference log bins */
    double mass;        /* particle mass (cancels in the overdensity) */
    int index_vel;      /* velocity transfer function (src/mitos.c:425-490), < 0: no velocities */
    int thermal;        /* thermal motion (src/mitos.c:910-1064): 0 none, 1 fermion, 2 boson */
    double thermal_T_eV, thermal_M_eV, speed_of_light;
    uint64_t thermal_draw_offset; /* draws of earlier thermal species after the white noise */
};
struct orc_ic_out {
    double *grf;        /* complex, after hermiticity + primordial power (optional) */
    double *delta_k;    /* complex density after the transfer function (optional) */
    double *phi_k;      /* complex potential after the solver, before the TSC undo (optional) */
    double *disp[3];    /* padded real displacement grids (optional) */
    float  *pos;        /* M^3 x 3 particle positions after wrap (optional) */
    double *rho;        /* N^3 CIC overdensity (optional) */
    double *pk_k, *pk_p; long *pk_obs; /* bins (required) */
    double *ma_eps;     /* per-cycle reference eps (optional, ma_cycles entries) */
    float  *vel;        /* M^3 x 3 particle velocities (optional; index_vel >= 0) */
};
int orc_ic_pipeline(const struct orc_ic_params *p, struct orc_ic_out *o);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
