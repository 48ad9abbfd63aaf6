/*
 * mitos_gb300.h -- C ABI of the GB300 (sm_103a) initial-condition library.
 *
 * The library replaces the FFTW-MPI hot path of Mitos (wullm/mitos) on one GPU.  It exports
 * the reference's own entry points with the reference's signatures, so the reference driver
 * (src/mitos.c) and analysis code (analyse/src/mitos_read.c) call it unchanged once they are
 * compiled against this header instead of the reference headers named beside each item.
 * A few entry points are new; each says so.
 *
 * Differences from the reference, all deliberate:
 *   - struct distributed_grid keeps the reference fields in the reference order and appends
 *     private fields; fbox and box are DEVICE pointers (use dg_copy_to_host/_from_host).
 *   - A grid is FP64 (complex128 / double, as the reference) or FP32 (complex64 / float);
 *     alloc_local_grid uses the precision set by mitos_set_precision (default FP64).
 *   - One rank: NX = N, X0 = 0.  MPI_Comm is kept as an opaque pointer-sized type.
 *   - Functions return an int status instead of exiting: 0 ok, 1 shape mismatch, 2 not in
 *     momentum space, 3 unsupported kernel callback or size, 4 CUDA error, 5 out of memory,
 *     6 bounded wait timed out, 7 no convergence, 8 invalid value drawn.  mitos_last_error()
 *     describes the last one.
 *   - Every entry point is synchronous on return (its work on the library stream is done),
 *     unless the calling thread chose asynchronous mode with mitos_set_stream.
 */
#ifndef MITOS_GB300_H
#define MITOS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- types kept from the reference headers ------------------------------------------- */
#if !defined(MPI_VERSION) && !defined(ORC_SHIM_MPI_H)
typedef struct mitos_comm_opaque *MPI_Comm; /* pointer-sized, as OpenMPI's MPI_Comm */
#define MPI_COMM_WORLD ((MPI_Comm)0)
#endif

#if defined(FFTW3_H)
typedef fftw_complex mitos_c128;
typedef fftwf_complex mitos_c64;
#else
typedef double mitos_c128[2]; /* layout of fftw_complex */
typedef float mitos_c64[2];   /* layout of fftwf_complex */
#endif

#define MITOS_FP64 0
#define MITOS_FP32 1

/* include/distributed_grid.h:29-60, fields in the reference order, private fields appended */
struct distributed_grid {
    int N;
    double boxlen;
    MPI_Comm comm;
    char momentum_space;
    long int NX;
    long int X0;
    long int local_size; /* complex elements: NX * N * (N/2 + 1) */
    mitos_c128 *fbox;    /* device; complex64 storage when precision == MITOS_FP32 */
    double *box;         /* device; float storage when precision == MITOS_FP32, padded to N+2 */
    /* ---- appended (not in the reference) ---- */
    int precision;
    int flags;
    void *priv;
};

/* include/random_xorshift.h:11-13 + include/random.h:25 */
struct xoshiro256ss_state {
    uint64_t s[4];
};
typedef struct xoshiro256ss_state rng_state;

/* include/fft.h:31-39 */
struct kernel {
    double kx, ky, kz;
    double k;
    double kern[2]; /* double complex in the reference; same layout */
    const void *params;
};

/* include/input.h:127-141 */
struct cosmology {
    double h;
    double n_s;
    double A_s;
    double k_pivot;
    double z_ini;
    double log_tau_ini;
    double rho_crit;
    double z_source;
    double log_tau_source;
};

/* include/perturb_data.h:28-53 */
struct perturb_data {
    int k_size;
    int tau_size;
    int n_functions;
    double *delta; /* [n_functions][tau_size][k_size] */
    double *k;
    double *log_tau;
    double *redshift;
    double *D_growth;
    double *f_growth;
    double *H_Hubble;
    char **titles;
    double *Omega;
};

/* include/perturb_spline.h:27-36 */
struct perturb_spline {
    const struct perturb_data *ptdat;
    double *k_acc_table;
    int k_acc_table_size;
};

/* include/fft_kernels.h:123-128 */
struct spline_params {
    const struct perturb_spline *spline;
    int index_src;
    int tau_index;
    double u_tau;
};

/* include/fft_kernels.h:189-193 */
struct Hermite_kern_params {
    int order;
    int N;
    double boxlen;
};

/* ---- grids: replaces src/distributed_grid.c (include/distributed_grid.h:74-77) -------- */
int alloc_local_grid(struct distributed_grid *dg, int N, double boxlen, MPI_Comm comm);
int free_local_grid(struct distributed_grid *dg);
int free_local_real_grid(struct distributed_grid *dg);
int free_local_complex_grid(struct distributed_grid *dg);

/* ---- FFT + k-space kernels: replaces src/fft.c:29-35,219-302 (include/fft.h:92-116) --- */
void fft_wavevector(int x, int y, int z, int N, double delta_k, double *kx, double *ky,
                    double *kz, double *k);
int fft_r2c_dg(struct distributed_grid *dg);
int fft_c2r_dg(struct distributed_grid *dg);
int fft_apply_kernel_dg(struct distributed_grid *dg_write, const struct distributed_grid *dg_read,
                        void (*compute)(struct kernel *the_kernel), const void *params);

/* Kernel callbacks of include/fft_kernels.h:28-219.  The reference defines them static inline
 * in a header, so their addresses differ per translation unit; here they are defined once in
 * the library (host functions with the reference arithmetic) and fft_apply_kernel_dg
 * recognises them by address.  Any other callback returns status 3 (there is no CPU path). */
void kernel_constant(struct kernel *the_kernel);
void kernel_lowpass(struct kernel *the_kernel);
void kernel_hipass(struct kernel *the_kernel);
void kernel_tophat(struct kernel *the_kernel);
void kernel_elliptic_tophat(struct kernel *the_kernel);
void kernel_translate(struct kernel *the_kernel);
void kernel_gaussian(struct kernel *the_kernel);
void kernel_gaussian_inv(struct kernel *the_kernel);
void kernel_inv_poisson(struct kernel *the_kernel);
void kernel_dx(struct kernel *the_kernel);
void kernel_dy(struct kernel *the_kernel);
void kernel_dz(struct kernel *the_kernel);
void kernel_power_no_transfer(struct kernel *the_kernel);
void kernel_transfer_function(struct kernel *the_kernel);
void kernel_inv_transfer_function(struct kernel *the_kernel);
void kernel_undo_Hermite_window(struct kernel *the_kernel);

/* ---- white noise: replaces src/grf.c:26-175 (include/grf.h:30-31) --------------------- */
/* Advances *state past every draw, as the sequential reference does. */
int generate_complex_grf(struct distributed_grid *dg, rng_state *state);
int enforce_hermiticity(struct distributed_grid *dg);
/* src/grf_ngeniclike.c:28-203 (include/grf_ngeniclike.h:29-30): the N-GenIC-style field (RANLUX
 * ranlxd1 seed table, per-column reseeding, amplitude sqrt(-ln U), kz = 0 conjugate fill).  fbox:
 * device buffer of NX*N*(N/2+1) complex doubles (the rows X0 .. X0+NX-1); block_size unused, as in
 * the reference.  Returns 0, 1 (invalid grid) or 4 (seed table allocation). */
int generate_ngeniclike_grf(mitos_c128 *fbox, int N, int NX, int X0, long block_size, double boxlen,
                            long seed);
/* the same into a grid of either precision (its N, NX, X0, boxlen), left in momentum space */
int generate_ngeniclike_grf_dg(struct distributed_grid *grf, long seed);
/* the first n uniforms of ranlxd1 seeded with seed (host; the generator of the two above) */
int mitos_ranlxd1_uniforms(unsigned long seed, long n, double *out);

/* ---- perturbation grid, Poisson, 2LPT, Monge-Ampere ----------------------------------- */
/* src/generate_grids.c:28-67 (include/generate_grids.h:29-34).  fname is not written: field
 * files are host I/O outside this library; copy the grid out with dg_copy_to_host. */
int generatePerturbationGrid(const struct cosmology *cosmo, const struct perturb_spline *spline,
                             struct distributed_grid *grf, struct distributed_grid *grid,
                             const char *transfer_func_title, const char *fname,
                             const double rescale_factor);
/* src/poisson.c:58-70 (include/poisson.h:30) */
int solvePoisson_dg(struct distributed_grid *dg);
/* src/2lpt.c:38-143 (include/2lpt.h:27-29) */
int solve2LPT(struct distributed_grid *potential, struct distributed_grid *density,
              struct distributed_grid *workspace, double factor1, double factor2);
/* src/monge_ampere.c:50-183 (include/monge_ampere.h:27-29) */
int solveMongeAmpere(struct distributed_grid *potential, struct distributed_grid *density,
                     struct distributed_grid *workspace, int cycles);

/* ---- power spectra: replaces src/calc_powerspec.c:32-217 (include/calc_powerspec.h:26-36) */
/* box1/box2 may be host or device pointers; bins are host arrays. */
void calc_cross_powerspec(int N, double boxlen, const mitos_c128 *box1, const mitos_c128 *box2,
                          int bins, double *k_in_bins, double *power_in_bins, int *obs_in_bins);
void calc_cross_powerspec_float(int N, double boxlen, const mitos_c64 *box1,
                                const mitos_c64 *box2, int bins, double *k_in_bins,
                                double *power_in_bins, int *obs_in_bins);
/* box1/box2 hold the x-slab X0 .. X0+NX-1 of the grid (NX*N*(N/2+1) elements, as each rank of the
 * reference holds); the bins average that slab's modes (the reference's MPI_Allreduce over ranks,
 * src/calc_powerspec.c:203-205, is the identity on one rank) */
void calc_cross_powerspec_float_mpi(long int N, long int X0, long int NX, double boxlen,
                                    const mitos_c64 *box1, const mitos_c64 *box2, int bins,
                                    double *k_in_bins, double *power_in_bins,
                                    long int *obs_in_bins);
/* src/calc_powerspec.c:295-508 (include/calc_powerspec.h:40-43): the bispectrum B(k1, k2, k3),
 * k1 = k2 in each of `bins` log bins, k3 from theta (type 0) or the value k3 (type 1) in `bins3`
 * log bins; volume_mode 1 masks ones (fbox ignored) for the bin volumes.  fbox may be a host or
 * device pointer; outputs are host arrays; nothing is printed. */
void calc_bispectrum(int N, double boxlen, const mitos_c128 *fbox, int bins, int bins3,
                     double *k1_in_bins, double *k2_in_bins, double *k3_in_bins, double *bispectrum,
                     int volume_mode, int type, double theta, double k3);

/* ==== entry points with no reference counterpart ====================================== */

/* Precision used by alloc_local_grid (MITOS_FP64 by default). */
int mitos_set_precision(int precision);
int mitos_get_precision(void);
int alloc_local_grid_prec(struct distributed_grid *dg, int N, double boxlen, MPI_Comm comm,
                          int precision);

/* Copy a grid between host and device.  which = 0: fbox (N*N*(N/2+1) complex),
 * which = 1: box (N*N*(N+2) reals).  Element type follows dg->precision. */
int dg_copy_to_host(const struct distributed_grid *dg, int which, void *host);
/* The /Field/Field dataset of writeFieldFile_dg (src/output_mpi.c:52-141): the real-space grid as
 * N x N x (N + 2) doubles, padding included, from a grid of either precision (no reference
 * counterpart; the HDF5 calls stay with the caller).  Returns 2 for a grid in momentum space, as
 * the reference refuses it (:81-84). */
int dg_field_to_host(const struct distributed_grid *dg, double *host);
int dg_copy_from_host(struct distributed_grid *dg, int which, const void *host);

/* The attribute values of the snapshot's /Header, /Cosmology and /Units groups, as
 * writeHeaderAttributes (src/header.c:26-175) writes them; the file, group and attribute calls
 * stay with the caller's HDF5 writer (host I/O).  The particle numbers come from the types whose
 * export name is "PartType0" .. "PartType6" (summed per name, as the reference does). */
struct snapshot_header {
    double BoxSize[3];                /* /Header */
    int Dimension;
    double Redshift;
    int Flag_Entropy_ICs;
    int NumFilesPerSnapshot;
    long NumPart_Total[7];
    long NumPart_Total_HighWord[7];
    double MassTable[7];
    double Cosmology_Redshift;        /* /Cosmology */
    double Unit_mass_cgs;             /* /Units: "Unit mass in cgs (U_M)" and the rest */
    double Unit_length_cgs;
    double Unit_time_cgs;
    double Unit_temperature_cgs;
    double Unit_current_cgs;
};
/* boxlen (pars->BoxLen), z_ini (cosmo->z_ini); per particle type its ExportName and
 * TotalNumber; the unit system (us->UnitMassKilogram, UnitLengthMetres, UnitTimeSeconds,
 * UnitTemperatureKelvin, UnitCurrentAmpere).  Host only; returns 0, or 1 for invalid arguments. */
int snapshot_header_attributes(double boxlen, double z_ini, int num_types, const char *const *export_names,
                               const long long *total_numbers, double unit_mass_kg, double unit_length_m,
                               double unit_time_s, double unit_temperature_K, double unit_current_A,
                               struct snapshot_header *out);

/* Description of the last failure (empty when none), and the number of kernels launched. */
const char *mitos_last_error(void);
long mitos_launch_count(void);
/* Release every cached plan, table and workspace. */
int mitos_release_all(void);
/* Timing on the library stream: CUDA events around everything launched in between. */
int mitos_timer_start(void);
double mitos_timer_stop(void);
int mitos_sync(void);
/* Per-launch timing (off by default): on = 1 clears and starts recording; mitos_kernel_times
 * returns up to max (name, milliseconds) pairs of the launches since. */
int mitos_kernel_timing(int on);
int mitos_kernel_times(const char **names, double *ms, int max);
/* Stage times (ms) of the last ic_pipeline_run made with MITOS_PROFILE set in the environment. */
int mitos_stage_times(double *ms, int max);
/* Per-cycle reference eps and relative rms residual of the last solveMongeAmpere. */
int mitos_ma_history(double *eps, double *rel, int max);
/* Host-only helpers (no GPU work): the xoshiro256** state n draws after s (jump-ahead), and
 * the start state of noise column c of an N grid. */
int mitos_rng_jump(uint64_t s[4], unsigned long long n);
int mitos_noise_column_state(int N, long c, const uint64_t s0[4], uint64_t out[4]);
/* Host copies of the FP64 white noise's arithmetic (no reference counterpart; the device kernel
 * performs the same operations): the correctly rounded log (x > 0) and cos (|y| < 8), and
 * sampleNorm (src/random.c:34-49) of the draws A, B with them.  mitos_cr_steps gives the two steps
 * of the evaluation separately (fn 0: log, 1: cos): the fast step's rounding, NaN when it cannot
 * decide, and the accurate step's. */
double mitos_cr_log(double x);
double mitos_cr_cos(double y);
double mitos_sample_norm_cr(uint64_t A, uint64_t B);
int mitos_cr_steps(int fn, double x, double *fast, double *accurate);

/* CIC mass assignment of n particles (float x,y,z triples, host or device pointer) onto the
 * real part of rho (padded layout), accumulated on top of its contents:
 * analyse/src/mitos_read.c:278-334 as a library call.  Returns the summed mass in *total. */
int cic_deposit_dg(struct distributed_grid *rho, const float *pos, long n, double mass,
                   double *total_mass);

/* Fused initial-condition pipeline on the device: white noise -> primordial power and
 * transfer function -> Zel'dovich / 2LPT / Monge-Ampere potential -> TSC window undo ->
 * displacement grids -> lattice displacement (TSC gather) -> CIC -> overdensity -> r2c ->
 * CIC window undo -> P(k).  Follows src/mitos.c:205-422,794-863,1072-1077 and
 * analyse/src/mitos_read.c:278-419 with z_source = z_ini. */
#define MITOS_METHOD_ZELDOVICH 1
#define MITOS_METHOD_2LPT 2
#define MITOS_METHOD_MONGE_AMPERE 3
struct ic_config {
    int N;              /* grid size */
    int M;              /* cube root of the particle number */
    double boxlen;
    uint64_t seed;      /* Seed (+ rank 0), src/mitos.c:148 */
    double A_s, n_s, k_pivot;
    double z_ini;
    int index_src;      /* transfer function index (findTitle of the density title) */
    int method;
    int ma_cycles;      /* Monge-Ampere: maximum cycles */
    double ma_tol;      /* Monge-Ampere: stop when sqrt(sum res^2 / sum rho^2) <= ma_tol (0: run all cycles) */
    int pk_bins;
    int pk_linear;      /* 1: linear shells to k_Nyquist; 0: the reference log bins */
    int precision;      /* MITOS_FP32 or MITOS_FP64 */
    int keep_outputs;   /* 1: keep the displacement grids, positions and density on the device */
    int index_vel;      /* velocity transfer function (TransferFunctionVelocity, src/mitos.c:425-490);
                           used when res->vel is set */
    /* thermal motion on top of the velocities (ThermalMotionType, src/mitos.c:910-1064, the branch
     * without Firebolt); used when res->vel is set */
    int thermal;                /* 0 none, 1 "fermion" (fd_pdf), 2 "boson" (be_pdf) */
    double thermal_M_eV;        /* MicroscopicMass_eV */
    double thermal_T_eV;        /* MicroscopyTemperature * kBoltzmann / ElectronVolt */
    double speed_of_light;      /* us.SpeedOfLight in internal units */
    uint64_t thermal_draw_offset; /* draws taken after the white noise by earlier thermal species */
    /* snapshot datasets (ic_result.coords / vels / masses / ids) */
    double particle_mass;        /* ptype->Mass (stored as float in struct particle, src/particle.c:104) */
    long long id_first_particle; /* ptype->FirstID */
};
struct ic_result {
    double *pk_k;       /* host [pk_bins] */
    double *pk_p;       /* host [pk_bins] */
    long *pk_obs;       /* host [pk_bins] */
    float *pos;         /* optional host [M^3 * 3]: positions after the wrap */
    int ma_iterations;  /* Monge-Ampere cycles run */
    double ma_residual; /* last sqrt(sum res^2 / sum rho^2) */
    float *vel;         /* optional host [M^3 * 3]: particle velocities (src/mitos.c:865-908): the TSC
                           gather of the velocity grids at the displaced positions; the velocity
                           potential from 2LPT with the reference's velocity factors (:453-455) for
                           2LPT configurations, else the inverse Poisson kernel (:457); plus the
                           thermal motion when cfg->thermal is set */
    /* optional host arrays: the particle datasets of the snapshot as src/mitos.c:1106-1117 hands them
     * to H5Dwrite (Coordinates, Velocities [M^3 * 3] and Masses [M^3] as double, ParticleIDs [M^3]),
     * made on the device from the wrapped positions and the velocities; vels needs index_vel */
    double *coords;
    double *vels;
    double *masses;
    long long *ids;
};
int ic_pipeline_run(const struct ic_config *cfg, const struct perturb_spline *spline,
                    struct ic_result *res);
/* Asynchronous form of ic_pipeline_run (no reference counterpart), for callers producing many ICs:
 * it enqueues the IC and returns.  The particle positions travel to res->pos on a copy stream while
 * later submissions compute; with res->pos in pinned (page-locked) host memory that transfer
 * overlaps the next IC's compute, otherwise the call waits for it.  At most two ICs are in flight:
 * a third submission first completes the oldest.  res and the arrays it points to must stay valid
 * until ic_pipeline_wait (or the submission after next) returns; ic_pipeline_wait completes every
 * submitted IC and fills its P(k) and Monge-Ampere fields. */
int ic_pipeline_submit(const struct ic_config *cfg, const struct perturb_spline *spline,
                       struct ic_result *res);
int ic_pipeline_wait(void);
/* The same on caller-provided host table arrays (convenience for bindings without structs). */
int ic_pipeline_run_table(const struct ic_config *cfg, int k_size, int tau_size,
                          int n_functions, const double *k, const double *log_tau,
                          const double *redshift, const double *D_growth, const double *delta,
                          struct ic_result *res);

/* calc_bispectrum on a momentum-space grid of either precision (no reference counterpart);
 * returns 0, or 1 (no grid), 2 (not in momentum space), 3, 4, 5. */
int calc_bispectrum_dg(const struct distributed_grid *dg, int bins, int bins3, double *k1_in_bins,
                       double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode,
                       int type, double theta, double k3);

/* ---- thermal motion: src/random.c:87-289 and the loop of src/mitos.c:928-1064 ---------------- */
#ifndef RANDOM_H
/* include/random.h:43-81 */
typedef double (*pdf)(double x, void *params);
struct interval {
    int id;
    double l, r;
    double Fl, Fr;
    double a0, a1, a2, a3;
    double error;
    int nid;
};
struct sampler {
    double norm;
    double xl, xr;
    pdf f;
    void *params;
    struct interval *intervals;
    int intervalNum;
    int I_max;
    double *index;
};
#endif
/* The thermal-motion loop of src/mitos.c:928-965,1054-1062 (without Firebolt) on the GPU, for n
 * particles of one species in id order: seven draws a particle from *state (samplerCustom of s,
 * then three sampleNorm), vel[i*stride + c] += n_c p / (a_ini M_eV) speed_of_light.  s is a sampler
 * made by the reference's initSampler (its pieces in order, as initSampler leaves them) or by
 * thermal_sampler_init.  vel is host or device memory (n particles, `stride` floats apart: 3 for
 * packed velocities, 10 for the v_X of struct particle).  *state advances by 7 n draws, as the
 * reference loop leaves it.  Every draw is the reference's; FP64 (mitos_set_precision) evaluates
 * it with the reference's operations.  Returns 0, 1, 3 (a sampler not in order), 5, or 8 (an
 * invalid momentum, where the reference exits). */
int thermal_velocities(const struct sampler *s, rng_state *state, long n, double M_eV, double a_ini,
                       double speed_of_light, float *vel, long stride);
/* initSampler (src/random.c:87-209) for fd_pdf (kind 1) or be_pdf (kind 2) on the domain
 * src/mitos.c:645-668 sets up ([1e-10, 15] T_eV, mu = 0), built on the host; no reference
 * counterpart under this name.  f and params are left NULL; free with thermal_sampler_free (or the
 * reference's cleanSampler). */
int thermal_sampler_init(struct sampler *s, int kind, double T_eV);
int thermal_sampler_free(struct sampler *s);
/* Host-only check (no GPU): the piece thermal_velocities' kernel takes for each 64-bit draw w[i]
 * (exact integer thresholds on u = w / 2^64, no reference counterpart); returns 0 or 3. */
int mitos_thermal_pieces(const struct sampler *s, const uint64_t *w, long n, int *piece);

/* P(k) binning that allocates no device memory.  No counterpart in the reference: for callers
 * that must not allocate device memory in their loop, because another allocator already holds
 * the device's memory or because cudaMalloc / cudaFree would synchronise a streaming pipeline.
 * dev_box1 / dev_box2 are device complex grids (N*N*(N/2+1), FP64 or FP32 per `precision`, on the
 * library's device: the device current at the library's first call; another device gives status
 * 3); linear = 0 gives the reference log bins of calc_cross_powerspec, 1 linear shells to
 * k_Nyquist, each mode in the bin the regular entry points give it.  Outputs are host arrays.
 * Scratch: a fixed device array for at most 4096 bins (128 KB) that the GPU holds until the
 * process exits; more bins return status 3.  The array is shared by all calls and keeps the last
 * call's contents; every call clears what it sums into, so calls whose GPU work overlaps race.
 * Set-up: the first call looks up the array's device address (cudaGetSymbolAddress).  Under
 * CUDA's lazy module loading (the default) the array is also reserved on the device then, so make
 * the first call -- N = 0 with both grids NULL does the set-up alone and returns 0 -- before
 * another allocator reserves the device's memory, and before any stream capture. */
int calc_cross_powerspec_noalloc(int N, double boxlen, const void *dev_box1, const void *dev_box2,
                                 int precision, int bins, int linear, double *k_in_bins,
                                 double *power_in_bins, long *obs_in_bins);

/* ---- Learned Monge-Ampere warm start (no reference counterpart) ----------------------------
 * A 3D convolutional network: 4 periodic 3x3x3 layers, channels 3 -> 16 -> 16 -> 16 -> 1, ReLU
 * after the first three; BF16 weights and activations on the tensor cores with FP32 accumulation.
 * Inputs: delta(x), the 1LPT potential phi_1(x) = c2r(-delta/k^2) and the 2LPT potential
 * phi_2(x) = c2r(-S(k)/k^2) (S the 2LPT source, src/2lpt.c:111-112).  Output: a source-space
 * correction sigma(x); the warm start adds G(k) r2c(sigma) to phi(k) after the first cycle.
 * Grids are FP32 device arrays of row pitch `pitch` (N for packed, N + 2 for the padded real
 * grids of struct distributed_grid); N must be a multiple of 32. */
#define MANET_PARAMS 27712 /* 4 x (27 * 16 * 16 weights + 16 biases), channel padded */
struct manet {
    float scale_in[3]; /* delta, phi_1, phi_2 are divided by these before the first layer */
    float scale_out;   /* the network output is multiplied by this */
    int steps;         /* Adam steps taken */
    void *priv;        /* device parameters, gradients and Adam moments */
};
/* He-normal initial weights from a splitmix64 stream of `seed`; scales 1 */
int manet_init(struct manet *net, unsigned long long seed);
int manet_free(struct manet *net);
/* FP32 parameters, layer by layer: w[t][ci][co] (27 x 16 x 16, taps t = (dx+1)*9 + (dy+1)*3 +
 * (dz+1)) then b[16]; entries of padded channels are zero */
int manet_get_params(const struct manet *net, float *host);
int manet_set_params(struct manet *net, const float *host);
/* gradients of the last manet_loss_grad / manet_train_step, same layout */
int manet_get_grads(const struct manet *net, float *host);
/* loss = mean over voxels of (net(inputs) - target / scale_out)^2 and its gradients */
int manet_loss_grad(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                    const float *phi2, const float *target, double *loss);
/* manet_loss_grad followed by one Adam step (beta 0.9 / 0.999) of learning rate lr */
int manet_train_step(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                     const float *phi2, const float *target, float lr, double *loss);
/* out = scale_out * net(inputs) */
int manet_infer(struct manet *net, int N, int pitch, const float *delta, const float *phi1,
                const float *phi2, float *out);
/* The grid the warm start of solveMongeAmpereTol runs the network on: 0 (default) the solve's own
 * grid; Nw < N a coarser grid of the same box: the inputs are the solve's fields with the modes
 * above Nw's Nyquist frequency dropped, and the correction enters phi(k) at those low modes only
 * (the iteration then fixes the rest).  Nw must be a multiple of 32; returns 0 or 1. */
int manet_set_warm_grid(struct manet *net, int Nw);

/* Monge-Ampere to a tolerance (no reference counterpart; the cycle of src/monge_ampere.c:50-183
 * with phi kept in k space: phi(k) += G(k) r2c(res)(k)).  Stops when the relative rms residual
 * rel = sqrt(sum res^2 / sum rho^2) is <= tol; the reference's eps (src/monge_ampere.c:177) is
 * rel / N^(3/2).  dens: density in momentum space with rho(x) in its box (as solveMongeAmpere);
 * pot->fbox receives phi(k).  warm: NULL for the reference's Zel'dovich start
 * (src/monge_ampere.c:87), or a trained network whose correction is added after the first
 * update (FP32 grids).  Returns 0, or 7 when max_cycles updates leave rel above tol. */
struct ma_stats {
    int cycles;         /* phi updates applied (the network correction not counted) */
    int evaluations;    /* residual evaluations (six-Hessian passes) */
    double rel;         /* last relative rms residual */
    double eps;         /* the reference's eps of the last evaluation: rel / N^(3/2) */
    double rel_first;   /* residual of the Zel'dovich start */
    double rel_second;  /* residual after the first update (and the network correction, if warm) */
    double ms;          /* device time of the call (CUDA events) */
    double ms_warm;     /* of which the warm start: 2LPT potential, network inference, correction */
};
int solveMongeAmpereTol(struct distributed_grid *potential, struct distributed_grid *density,
                        struct distributed_grid *workspace, double tol, int max_cycles,
                        struct manet *warm, struct ma_stats *stats);
/* One training pair for the network from a density (FP32 grids): the cold iteration runs
 * `cycles` updates; outputs are device FP32 real grids of N*N*(N+2) floats (pitch N+2):
 * delta(x), phi_1(x), phi_2(x) (the inputs) and sigma(x) = lap(phi_final - phi_after_first_update),
 * the source-space correction the network learns. */
int manet_training_pair(struct distributed_grid *potential, struct distributed_grid *density,
                        struct distributed_grid *workspace, int cycles, float *delta, float *phi1,
                        float *phi2, float *sigma, struct ma_stats *stats);

/* ---- Ensembles of realisations in one CUDA graph (no reference counterpart: the reference runs
 * one realisation per process) -------------------------------------------------------------------
 * ic_ensemble_create runs every configuration once (workspaces, tables), then captures all of
 * them into one graph over `streams` concurrent streams (largest work first).  Configurations
 * that differ only in the seed (Zel'dovich or 2LPT, lattice-aligned) form batched units: one
 * launch per pass covers the whole unit.  A replay (ic_ensemble_run) recomputes the same
 * realisations; *ms receives its device time.  ic_ensemble_result fills P(k) of configuration i
 * (pos is not produced). */
struct ic_ensemble;
int ic_ensemble_create(struct ic_ensemble **ens, const struct ic_config *cfgs, int n,
                       const struct perturb_spline *spline, int streams);
/* The same with at most max_batch realisations per unit (1: no batching; 0: as many as fit in
 * 2^25 grid cells, the ic_ensemble_create default). */
int ic_ensemble_create_batched(struct ic_ensemble **ens, const struct ic_config *cfgs, int n,
                               const struct perturb_spline *spline, int streams, int max_batch);
int ic_ensemble_run(struct ic_ensemble *ens, double *ms);
int ic_ensemble_result(struct ic_ensemble *ens, int i, struct ic_result *res);
int ic_ensemble_launches(const struct ic_ensemble *ens); /* kernel launches in one replay */
int ic_ensemble_units(const struct ic_ensemble *ens);    /* batched pipeline runs in one replay */
int ic_ensemble_destroy(struct ic_ensemble *ens);
/* FFT schedule autotuner: times the IC of cfg (best of three) over the radix schedules of the
 * length-N transforms (X / Y passes), then of the length-N/2 transforms (Z passes), then over
 * every fitting pair of X/Y pencils per block and Z rows per block; keeps the fastest for
 * (N, precision) in this process and returns its tile (mitos_get_radix gives its radices). */
int mitos_autotune(const struct ic_config *cfg, const struct perturb_spline *spline, int *p_xy,
                   int *p_z, double *ms);
int mitos_set_tiles(int N, int precision, int p_xy, int p_z);
int mitos_get_tiles(int N, int precision, int *p_xy, int *p_z);
/* Radix schedules, first stage first: radices 2, 3, 4 or 8 that divide the elements a thread holds
 * (8 for N = 2^k, 12 for 3 2^k), with product N (X / Y) and N/2 (Z); at most 11 stages.  Returns 1
 * for a schedule that does not fit.  Any schedule but the default runs the FP32 sizes 256, 512
 * and 1024 on the runtime-plan kernels instead of their compile-time ones.  mitos_get_radix fills
 * arrays of at least 12 ints. */
int mitos_set_radix(int N, int precision, const int *rad_n, int stages_n, const int *rad_h, int stages_h);
int mitos_get_radix(int N, int precision, int *rad_n, int *stages_n, int *rad_h, int *stages_h);
/* The r2c's Z and Y steps in one thread-block-cluster pass (the x-plane held in the cluster's
 * distributed shared memory), for FP32 N = 256 and 512 where the device fits the cluster.  mode 0
 * (the default): off, the Z r2c and Y passes; 1: clusters of 16 CTAs of 512 threads (N = 256: 8),
 * two column buffers; 2: 16 CTAs of 256 threads (N = 256: 8), one buffer; 3: 8 CTAs of 512 threads
 * (N = 256: 4), one buffer.  Other values turn it off.  Returns the previous mode.  No reference
 * counterpart (a switch of this library's FFT; fft_r2c_dg, src/fft.c:219-236, is the transform
 * either way). */
int mitos_set_cluster_fft(int mode);
/* Staging of the lattice deposit's displacement tiles: 1 (the default) stages the bricks off the box's
 * x and y faces with tensor copies (cp.async.bulk.tensor, one thread a brick), 0 stages every brick
 * with 16-byte cp.async.  The results are identical.  Returns the previous setting.  No reference
 * counterpart. */
int mitos_set_lattice_tma(int on);
/* The stream the calling thread's entry points launch on: a caller's cudaStream_t, or NULL for the
 * library's own stream (the default).  async = 1 with a caller's stream: the entry points that only
 * transform device grids enqueue their work and return without synchronising (the *_async form of
 * the reference entry points, e.g. for capture into the caller's CUDA graph): fft_r2c_dg,
 * fft_c2r_dg, fft_apply_kernel_dg (any kernel but the transfer functions, whose spline rows come
 * from the host), solvePoisson_dg, solve2LPT, generate_complex_grf, enforce_hermiticity,
 * cic_deposit_dg (device positions).  Entry points that return host results or upload host data (the grid copies,
 * P(k), the transfer-function kernels, the IC pipeline) still synchronise, so they cannot be
 * captured.  The first call of an entry point for a grid size allocates its workspace and tables:
 * make it once outside a capture.  Per thread; returns 0. */
int mitos_set_stream(void *stream, int async);
/* Order in which the lattice deposit's blocks walk its 8 x 8 x 32 bricks: 1 (the default, where the
 * bricks tile into them) by regions of 8 x 8 x 4 bricks, so that the bricks in flight share their
 * halo tiles and flushed density sectors in L2; 0 by rows (x fastest, then y, then z).  FP32 output
 * is identical (fixed-point sums); FP64 sums may differ in the last bits (their atomics' order).
 * Returns the previous setting.  No reference counterpart. */
int mitos_set_lattice_order(int regions);

#ifdef __cplusplus
}
#endif
#endif /* MITOS_GB300_H */
