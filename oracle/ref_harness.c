/*
 * ref_harness.c -- drives the reference's own hot-path functions (compiled unmodified from
 * the reference sources against ref_shim/) in the order src/mitos.c:205-422,794-863 and
 * analyse/src/mitos_read.c:278-419 call them, so the oracle restatement can be pinned
 * against the reference code.  TEST INFRASTRUCTURE ONLY; built into oracle/_ref/.
 *
 * The CIC deposit and the overdensity exist in the reference only inside main()
 * (analyse/src/mitos_read.c:278-376); for those two steps this harness calls the oracle's
 * line-by-line restatement.  Linear P(k) shells are an extension with no reference code.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mitos.h"
#include "../../oracle/mitos_oracle.h"

/* one external definition of the C99 inline sinc of include/fft_kernels.h:187 */
extern inline double sinc(double x);

void ref_draws(uint64_t seed, int64_t n, uint64_t *out) {
    rng_state s = rand_uint64_init(seed);
    for (int64_t i = 0; i < n; i++) out[i] = rand_uint64(&s);
}

void ref_norms(uint64_t seed, int64_t n, double *out) {
    rng_state s = rand_uint64_init(seed);
    for (int64_t i = 0; i < n; i++) out[i] = sampleNorm(&s);
}

/* generate_complex_grf + enforce_hermiticity, src/mitos.c:216-221 */
int ref_grf(int N, double boxlen, uint64_t seed, int hermitian, double *out) {
    struct distributed_grid grf;
    alloc_local_grid(&grf, N, boxlen, MPI_COMM_WORLD);
    rng_state s = rand_uint64_init(seed);
    generate_complex_grf(&grf, &s);
    if (hermitian) enforce_hermiticity(&grf);
    memcpy(out, grf.fbox, sizeof(fftw_complex) * grf.local_size);
    free_local_grid(&grf);
    return 0;
}

/* one r2c or c2r of a padded grid through fft_r2c_dg / fft_c2r_dg */
int ref_fft_dg(int N, double boxlen, int to_momentum, double *real_padded, double *complex_half) {
    struct distributed_grid g;
    alloc_local_grid(&g, N, boxlen, MPI_COMM_WORLD);
    size_t n = sizeof(fftw_complex) * g.local_size;
    if (to_momentum) {
        memcpy(g.box, real_padded, n);
        fft_r2c_dg(&g);
        memcpy(complex_half, g.fbox, n);
    } else {
        memcpy(g.fbox, complex_half, n);
        g.momentum_space = 1;
        fft_c2r_dg(&g);
        memcpy(real_padded, g.box, n);
    }
    free_local_grid(&g);
    return 0;
}

static char *g_titles[64];

/* the thermal-motion loop of src/mitos.c:928-965,1054-1062 (the branch without Firebolt, every draw
 * accepted), calling the reference's samplerCustom and sampleNorm; the loop itself is inline in the
 * reference's main() */
static int thermal_loop(struct sampler *ts, rng_state *seed, struct particle *parts, long long n,
                        double M_eV, double a_ini, double speed_of_light) {
    for (long long i = 0; i < n; i++) {
        double p0_eV = samplerCustom(ts, seed);
        double p_eV = p0_eV / a_ini;
        if (isnan(p_eV) || p_eV <= 0) return 1;
        double V = p_eV / M_eV * speed_of_light;
        double nx = sampleNorm(seed);
        double ny = sampleNorm(seed);
        double nz = sampleNorm(seed);
        double length = hypot(nx, hypot(ny, nz));
        if (length > 0) {
            nx /= length;
            ny /= length;
            nz /= length;
        }
        parts[i].v_X += nx * V;
        parts[i].v_Y += ny * V;
        parts[i].v_Z += nz * V;
    }
    return 0;
}

/* the reference sampler (src/random.c:87-289) for kind 1 (fd_pdf) or 2 (be_pdf) on
 * [THERMAL_MIN_MOMENTUM, THERMAL_MAX_MOMENTUM] kT, as src/mitos.c:641-668 sets it up: the pieces as
 * rows [l r Fl Fr a0 a1 a2 a3], the search table, the normalisation */
int ref_sampler_table(int kind, double T_eV, int max, double *rows, int *table, double *norm) {
    double tp[2] = {T_eV, 0};
    struct sampler s;
    if (initSampler(&s, kind == 2 ? be_pdf : fd_pdf, THERMAL_MIN_MOMENTUM * T_eV, THERMAL_MAX_MOMENTUM * T_eV, tp))
        return -1;
    for (int j = 0; j < s.intervalNum && j < max; j++) {
        const struct interval *iv = &s.intervals[j];
        const double r[8] = {iv->l, iv->r, iv->Fl, iv->Fr, iv->a0, iv->a1, iv->a2, iv->a3};
        memcpy(rows + 8 * j, r, sizeof r);
    }
    for (int i = 0; i < s.I_max && table; i++) table[i] = (int)s.index[i];
    if (norm) *norm = s.norm;
    const int n = s.intervalNum;
    cleanSampler(&s);
    return n;
}

int ref_sampler_draws(int kind, double T_eV, const uint64_t st0[4], long n, double *out) {
    double tp[2] = {T_eV, 0};
    struct sampler s;
    if (initSampler(&s, kind == 2 ? be_pdf : fd_pdf, THERMAL_MIN_MOMENTUM * T_eV, THERMAL_MAX_MOMENTUM * T_eV, tp))
        return 1;
    rng_state st;
    memcpy(st.s, st0, sizeof st.s);
    for (long i = 0; i < n; i++) out[i] = samplerCustom(&s, &st);
    cleanSampler(&s);
    return 0;
}

/* n particles (velocities n x 3 in/out) through the thermal loop from state st0 */
int ref_thermal(int kind, double T_eV, double M_eV, double a_ini, double speed_of_light,
                const uint64_t st0[4], long n, float *vel) {
    double tp[2] = {T_eV, 0};
    struct sampler s;
    if (initSampler(&s, kind == 2 ? be_pdf : fd_pdf, THERMAL_MIN_MOMENTUM * T_eV, THERMAL_MAX_MOMENTUM * T_eV, tp))
        return 1;
    struct particle *parts = calloc((size_t)n, sizeof(struct particle));
    for (long i = 0; i < n; i++) {
        parts[i].v_X = vel[3 * i];
        parts[i].v_Y = vel[3 * i + 1];
        parts[i].v_Z = vel[3 * i + 2];
    }
    rng_state st;
    memcpy(st.s, st0, sizeof st.s);
    const int e = thermal_loop(&s, &st, parts, n, M_eV, a_ini, speed_of_light);
    for (long i = 0; i < n; i++) {
        vel[3 * i] = parts[i].v_X;
        vel[3 * i + 1] = parts[i].v_Y;
        vel[3 * i + 2] = parts[i].v_Z;
    }
    free(parts);
    cleanSampler(&s);
    return e;
}

int ref_ic_pipeline(int N, int M, double L, uint64_t seed, double A_s, double n_s, double k_pivot,
                    int k_size, int tau_size, int n_functions, const double *kv,
                    const double *log_tau, const double *redshift, const double *Dg,
                    const double *fg, const double *Hh, const double *delta, int index_src,
                    double z_ini, int lpt_order, int ma_cycles, int pk_bins, int pk_linear,
                    double mass, double *out_grf, double *out_delta_k, double *out_phi_k,
                    double *out_d0, double *out_d1, double *out_d2, float *out_pos,
                    double *out_rho, double *pk_k, double *pk_p, long *pk_obs, int index_vel,
                    float *out_vel, int thermal_kind, double T_eV, double M_eV,
                    double speed_of_light, uint64_t thermal_draw_offset) {
    if (n_functions > 64) return 1;
    for (int i = 0; i < n_functions; i++) {
        if (!g_titles[i]) {
            g_titles[i] = malloc(16);
            snprintf(g_titles[i], 16, "f%d", i);
        }
    }
    struct perturb_data ptdat;
    memset(&ptdat, 0, sizeof ptdat);
    ptdat.k_size = k_size;
    ptdat.tau_size = tau_size;
    ptdat.n_functions = n_functions;
    ptdat.delta = (double *)delta;
    ptdat.k = (double *)kv;
    ptdat.log_tau = (double *)log_tau;
    ptdat.redshift = (double *)redshift;
    ptdat.D_growth = (double *)Dg;
    ptdat.f_growth = (double *)fg;
    ptdat.H_Hubble = (double *)Hh;
    ptdat.titles = g_titles;
    struct perturb_spline spline;
    initPerturbSpline(&spline, DEFAULT_K_ACC_TABLE_SIZE, &ptdat);

    struct cosmology cosmo;
    memset(&cosmo, 0, sizeof cosmo);
    cosmo.A_s = A_s;
    cosmo.n_s = n_s;
    cosmo.k_pivot = k_pivot;
    cosmo.z_ini = z_ini;
    cosmo.z_source = z_ini;

    /* src/mitos.c:148-177 */
    rng_state seed_state = rand_uint64_init(seed + 0);
    cosmo.log_tau_ini = perturbLogTauAtRedshift(&spline, cosmo.z_ini);
    cosmo.log_tau_source = perturbLogTauAtRedshift(&spline, cosmo.z_source);
    const double D_source = perturbGrowthFactorAtLogTau(&spline, cosmo.log_tau_source);
    const double D_ini = perturbGrowthFactorAtLogTau(&spline, cosmo.log_tau_ini);

    /* :206-227 */
    struct distributed_grid grf;
    alloc_local_grid(&grf, N, L, MPI_COMM_WORLD);
    generate_complex_grf(&grf, &seed_state);
    enforce_hermiticity(&grf);
    fft_apply_kernel_dg(&grf, &grf, kernel_power_no_transfer, &cosmo);
    const size_t cb = sizeof(fftw_complex) * grf.local_size;
    if (out_grf) memcpy(out_grf, grf.fbox, cb);
    fft_c2r_dg(&grf);
    /* :300 */
    fft_r2c_dg(&grf);

    /* :308-317 */
    struct distributed_grid grid, potential, derivative;
    alloc_local_grid(&grid, N, L, MPI_COMM_WORLD);
    alloc_local_grid(&potential, N, L, MPI_COMM_WORLD);
    alloc_local_grid(&derivative, N, L, MPI_COMM_WORLD);

    /* :356-377 */
    double rescale_factor = (cosmo.z_ini != cosmo.z_source) ? D_ini / D_source : 1.0;
    char title[16];
    snprintf(title, sizeof title, "f%d", index_src);
    int err = generatePerturbationGrid(&cosmo, &spline, &grf, &grid, title, "", rescale_factor);
    if (err) return err;
    if (out_delta_k) {
        /* the transfer-function product before the c2r; recompute it the same way */
        struct distributed_grid tmp;
        alloc_local_grid(&tmp, N, L, MPI_COMM_WORLD);
        int tau_index; double u_tau;
        perturbSplineFindTau(&spline, cosmo.log_tau_source, &tau_index, &u_tau);
        struct spline_params sp = {&spline, index_src, tau_index, u_tau};
        fft_apply_kernel_dg(&tmp, &grf, kernel_transfer_function, &sp);
        memcpy(out_delta_k, tmp.fbox, cb);
        free_local_grid(&tmp);
    }
    fft_r2c_dg(&grid);

    /* :380-389 */
    if (ma_cycles > 0) err = solveMongeAmpere(&potential, &grid, &derivative, ma_cycles);
    else if (lpt_order == 2) err = solve2LPT(&potential, &grid, &derivative, 1.0, -3. / 7.);
    else fft_apply_kernel_dg(&potential, &grid, kernel_inv_poisson, NULL);
    if (err) return err;
    if (out_phi_k) memcpy(out_phi_k, potential.fbox, cb);

    /* :395-416 */
    struct Hermite_kern_params Hkp;
    Hkp.order = 3;
    Hkp.N = N;
    Hkp.boxlen = L;
    fft_apply_kernel_dg(&potential, &potential, kernel_undo_Hermite_window, &Hkp);
    const kernel_func derivative_kernels[] = {kernel_dx, kernel_dy, kernel_dz};
    double *disp[3];
    double *outs[3] = {out_d0, out_d1, out_d2};
    for (int i = 0; i < 3; i++) {
        fft_apply_kernel_dg(&derivative, &potential, derivative_kernels[i], NULL);
        fft_c2r_dg(&derivative);
        disp[i] = malloc(cb);
        memcpy(disp[i], derivative.box, cb);
        if (outs[i]) memcpy(outs[i], derivative.box, cb);
    }
    fft_c2r_dg(&potential);

    /* :425-490 velocity grids, with z_source = z_ini (rescale 1, :431-436) */
    double *vgrid[3] = {NULL, NULL, NULL};
    if (index_vel >= 0) {
        snprintf(title, sizeof title, "f%d", index_vel);
        err = generatePerturbationGrid(&cosmo, &spline, &grf, &grid, title, "", 1.0);
        if (err) return err;
        fft_r2c_dg(&grid);
        if (lpt_order == 2 && ma_cycles <= 0)
            err = solve2LPT(&potential, &grid, &derivative, -0.001147273637728, 3.19354920304769E-05);
        else
            fft_apply_kernel_dg(&potential, &grid, kernel_inv_poisson, NULL);
        if (err) return err;
        fft_apply_kernel_dg(&potential, &potential, kernel_undo_Hermite_window, &Hkp);
        for (int i = 0; i < 3; i++) {
            fft_apply_kernel_dg(&derivative, &potential, derivative_kernels[i], NULL);
            fft_c2r_dg(&derivative);
            vgrid[i] = malloc(cb);
            memcpy(vgrid[i], derivative.box, cb);
        }
    }
    free_local_grid(&grf);
    free_local_grid(&grid);
    free_local_grid(&potential);
    free_local_grid(&derivative);

    /* :772-863 particle lattice and TSC displacement (one rank) */
    struct params pars;
    memset(&pars, 0, sizeof pars);
    pars.BoxLen = L;
    struct particle_type ptype;
    memset(&ptype, 0, sizeof ptype);
    ptype.TotalNumber = (long long)M * M * M;
    ptype.CubeRootNumber = M;
    ptype.Mass = mass;
    long long chunk_size = (long long)M * M * M;
    struct particle *parts = malloc(chunk_size * sizeof(struct particle));
    genParticlesFromGrid_local(&parts, &pars, NULL, &cosmo, &ptype, M, 0, 0, 0);
    for (int dir = 0; dir < 3; dir++) {
        struct left_right_slice lrs;
        lrs.local_slice = disp[dir];
        lrs.local_NX = N;
        lrs.local_X0 = 0;
        lrs.left_slice = disp[dir];
        lrs.left_NX = 0;
        lrs.left_X0 = 0;
        lrs.right_slice = disp[dir];
        lrs.right_NX = 0;
        lrs.right_X0 = 0;
#pragma omp parallel for
        for (long long i = 0; i < chunk_size; i++) {
            double x = parts[i].X;
            double y = parts[i].Y;
            double z = parts[i].Z;
            double d = gridTSC_dg(&lrs, x, y, z, L, N);
            if (dir == 0) parts[i].X -= d;
            else if (dir == 1) parts[i].Y -= d;
            else parts[i].Z -= d;
        }
    }
    /* :865-908 velocities at the displaced positions */
    if (index_vel >= 0) {
        for (int dir = 0; dir < 3; dir++) {
            struct left_right_slice lrs;
            lrs.local_slice = vgrid[dir];
            lrs.local_NX = N;
            lrs.local_X0 = 0;
            lrs.left_slice = vgrid[dir];
            lrs.left_NX = 0;
            lrs.left_X0 = 0;
            lrs.right_slice = vgrid[dir];
            lrs.right_NX = 0;
            lrs.right_X0 = 0;
#pragma omp parallel for
            for (long long i = 0; i < chunk_size; i++) {
                double vel = gridTSC_dg(&lrs, parts[i].X, parts[i].Y, parts[i].Z, L, N);
                if (dir == 0) parts[i].v_X = vel;
                else if (dir == 1) parts[i].v_Y = vel;
                else parts[i].v_Z = vel;
            }
        }
        for (int i = 0; i < 3; i++) free(vgrid[i]);
        /* :910-1064 thermal motion (no Firebolt), from the stream the white noise left (:148, :220) */
        if (thermal_kind > 0) {
            for (uint64_t d = 0; d < thermal_draw_offset; d++) (void)rand_uint64(&seed_state);
            double tp[2] = {T_eV, 0};
            struct sampler ts;
            if (initSampler(&ts, thermal_kind == 2 ? be_pdf : fd_pdf, THERMAL_MIN_MOMENTUM * T_eV,
                            THERMAL_MAX_MOMENTUM * T_eV, tp))
                return 1;
            const double a_ini = 1.0 / (1.0 + cosmo.z_ini);
            err = thermal_loop(&ts, &seed_state, parts, chunk_size, M_eV, a_ini, speed_of_light);
            cleanSampler(&ts);
            if (err) return err;
        }
        if (out_vel)
            for (long long i = 0; i < chunk_size; i++) {
                out_vel[3 * i] = parts[i].v_X;
                out_vel[3 * i + 1] = parts[i].v_Y;
                out_vel[3 * i + 2] = parts[i].v_Z;
            }
    }
    /* :1072-1077 */
    for (long long i = 0; i < chunk_size; i++) {
        parts[i].X = fwrap(parts[i].X, L);
        parts[i].Y = fwrap(parts[i].Y, L);
        parts[i].Z = fwrap(parts[i].Z, L);
    }
    for (int i = 0; i < 3; i++) free(disp[i]);
    float *pos = malloc(sizeof(float) * 3 * chunk_size);
    for (long long i = 0; i < chunk_size; i++) {
        pos[3 * i] = parts[i].X;
        pos[3 * i + 1] = parts[i].Y;
        pos[3 * i + 2] = parts[i].Z;
    }
    float pmass = parts[0].mass;
    free(parts);
    if (out_pos) memcpy(out_pos, pos, sizeof(float) * 3 * chunk_size);

    /* analyse/src/mitos_read.c:278-419 */
    double *box = calloc((size_t)N * N * N, sizeof(double));
    double total_mass = orc_cic_deposit(chunk_size, pos, (double)pmass, N, L, box);
    free(pos);
    orc_overdensity(N, L, total_mass, box);
    if (out_rho) memcpy(out_rho, box, sizeof(double) * N * N * N);
    fftw_complex *fbox = fftw_malloc((size_t)N * N * (N / 2 + 1) * sizeof(fftw_complex));
    fftw_plan r2c = fftw_plan_dft_r2c_3d(N, N, N, box, fbox, FFTW_ESTIMATE);
    fft_execute(r2c);
    fft_normalize_r2c(fbox, N, L);
    undoCICWindow(fbox, N, L);
    if (pk_linear) {
        orc_powerspec_lin(N, L, (double *)fbox, (double *)fbox, pk_bins, pk_k, pk_p, pk_obs);
    } else {
        int *obs = calloc(pk_bins, sizeof(int));
        calc_cross_powerspec(N, L, fbox, fbox, pk_bins, pk_k, pk_p, obs);
        for (int i = 0; i < pk_bins; i++) pk_obs[i] = obs[i];
        free(obs);
    }
    fftw_destroy_plan(r2c);
    fftw_free(fbox);
    free(box);
    cleanPerturbSpline(&spline);
    return 0;
}

/* writeHeaderAttributes (src/header.c:26-175) of a run with the given box, redshift, particle
 * types (ExportName, TotalNumber) and units; the attributes it writes are recorded by the HDF5
 * stand-in (orc_h5_count / orc_h5_get) */
void orc_h5_reset(void);
int ref_header_attributes(double boxlen, double z_ini, int ntypes, const char **export_names,
                          const long long *total_numbers, const double *units5) {
    struct params pars;
    struct cosmology cosmo;
    struct units us;
    memset(&pars, 0, sizeof pars);
    memset(&cosmo, 0, sizeof cosmo);
    memset(&us, 0, sizeof us);
    pars.BoxLen = boxlen;
    pars.NumParticleTypes = ntypes;
    cosmo.z_ini = z_ini;
    us.UnitMassKilogram = units5[0];
    us.UnitLengthMetres = units5[1];
    us.UnitTimeSeconds = units5[2];
    us.UnitTemperatureKelvin = units5[3];
    us.UnitCurrentAmpere = units5[4];
    struct particle_type *types = calloc(ntypes > 0 ? ntypes : 1, sizeof *types);
    for (int i = 0; i < ntypes; i++) {
        types[i].ExportName = (char *)export_names[i];
        types[i].TotalNumber = total_numbers[i];
    }
    orc_h5_reset();
    int err = writeHeaderAttributes(&pars, &cosmo, &us, &types, (hid_t)1);
    free(types);
    return err;
}
