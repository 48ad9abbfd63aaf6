// grids.cuh -- whole-grid transforms shared by the entry points (api.cu), the fused pipeline
// (pipeline.cu) and the Monge-Ampere solver (ma.cu).
#pragma once

#include "context.cuh"

namespace mitos {

// fbox (destroyed) -> box (pitch N + 2), FFTW c2r order and the 1/V normalisation (src/fft.c:110-125)
int grid_c2r(const GridGeom &g, int prec, double boxlen, void *fbox, void *box);
// box (pitch rp, transformed on load as x * rho_a + rho_b) -> fbox, x V/N^3 (src/fft.c:91-106)
int grid_r2c(const GridGeom &g, int prec, double boxlen, const void *box, int rp, double rho_a, double rho_b,
             void *fbox);
// six Hessian components of phi (k space) through the fused X / Y / Z passes into out (real);
// ZOP_HESS_2LPT writes the second-order source, ZOP_HESS_MA the Monge-Ampere residual (and, when
// out2 is given, the second-order source too)
// (zero / zero_bytes: a region the 2LPT-source Z pass clears on the side)
int grid_hessian(const GridGeom &g, int prec, double boxlen, const void *phi, int zop, const void *rho, void *out,
                 double *red, int window_order, void *out2 = nullptr, int batch = 1, size_t bstride = 0,
                 void *zero = nullptr, size_t zero_bytes = 0);
int axpby(int prec, long n, double a, const void *x, double b, const void *y, void *out);
inline size_t csize(int prec) { return prec == MITOS_FP32 ? 8 : 16; }

// options of one pipeline run (pipeline.cu): acc, when set, receives the P(k) accumulators
// (3 * pk_bins + 2 doubles: k sums, power sums, counts); graph = a run inside a stream capture (no
// host copies or synchronisation; the transfer rows an earlier run of the workspace set uploaded)
struct PipeOpts {
    double *acc;
    bool graph;
    // batch > 1: that many realisations of cfg, realisation b started at states[4 b .. 4 b + 3]
    // (device; seed_state of its seed), its P(k) sums at acc + b (3 pk_bins + 2); one launch per pass
    int batch = 1;
    const uint64_t *states = nullptr;
    double *dtab = nullptr;      // device transfer rows of this run (3 k_size), or the workspace's
    int async_slot = -1;         // >= 0: an ic_pipeline_submit run in staging slot 0 or 1
    double *acc_host = nullptr;  // async: pinned host buffer for the power sums
    int *iters = nullptr;        // async: Monge-Ampere cycles and residual, filled on the host
    double *last_rel = nullptr;
};
// calc_bispectrum on a device field of the precision (fbox may be null in volume mode)
int bispectrum_run(int N, double boxlen, int prec, const void *fbox, int bins, int bins3, double *k1_in_bins,
                   double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode, int type,
                   double theta, double k3);
// the xoshiro256** start state of a seed (splitmix64, as the reference seeds Seed + rank 0)
void seed_state(uint64_t seed, uint64_t st[4]);
// thermal motion of one species (thermal.cu): n particles from the stream of seed_state advanced by
// `skip` draws, added to the device velocities (n x stride floats); *derr (device) gets bit 0 for an
// invalid momentum
int thermal_add(int prec, long n, const uint64_t seed_state[4], unsigned long long skip, int kind, double T_eV,
                double M_eV, double a_ini, double c, float *dvel, long stride, int *derr);
int pipeline_table(const struct ic_config *cfg, int k_size, int tau_size, int n_functions, const double *k,
                   const double *log_tau, const double *redshift, const double *D_growth, const double *delta,
                   struct ic_result *res, const PipeOpts *opt);
int pipeline_spline(const struct ic_config *cfg, const struct perturb_spline *spline, struct ic_result *res,
                    const PipeOpts *opt);

}  // namespace mitos
