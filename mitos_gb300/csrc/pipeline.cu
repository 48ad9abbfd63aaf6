// pipeline.cu -- the fused initial-condition pipeline (ic_pipeline_run).
//
// Stage order (src/mitos.c:205-422,794-863,1072-1077 then analyse/src/mitos_read.c:278-419), with
// the reference's redundant c2r -> r2c round trips removed (exact in exact arithmetic):
//   S1  noise x sqrt(P_prim) x T(k, tau_src) x rescale x (-1/k^2)  -> phi1(k)   [+ Hermitian planes]
//   S2  six Hessians of phi1 (X, Y, Z passes) with the 2LPT source and its z r2c fused into the Z pass
//   S3  the Y and X steps of the S r2c; the X pass forms phi = f1 phi1 - f2 S/k^2 and undoes the TSC window
//       (Monge-Ampere: S2/S3 iterate residual -> phi += -res/k^2 until the tolerance)
//   S4  three displacement grids (X, Y, Z passes)
//   S5  lattice + TSC displacement + wrap + CIC deposit
//   S6  density r2c; the last X pass undoes the CIC window and bins P(k)
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "context.cuh"
#include "grids.cuh"
#include "kspace.cuh"
#include "particles.cuh"

using namespace mitos;

// filter per squared integer wavevector norm: include/fft_kernels.h:116-155 (power, transfer),
// rescale, and optionally the inverse Poisson kernel (:96-99)
template <typename T>
__global__ void k_filter(long n2max, double dk, double A_s, double n_s, double k_pivot,
                         const double *__restrict__ tab, int k_size, double u_tau, double rescale,
                         int poisson, T *__restrict__ out) {
    for (long n2 = (long)blockIdx.x * blockDim.x + threadIdx.x; n2 <= n2max; n2 += (long)gridDim.x * blockDim.x) {
        if (n2 == 0) { out[0] = 0; continue; }
        const double k = sqrt((double)n2) * dk;
        double v = sqrt(A_s * pow(k / k_pivot, n_s - 1.) * k * (2. * M_PI * M_PI));
        v *= transfer_at<double>(tab, tab + k_size, tab + 2 * k_size, k_size, k, u_tau);
        v *= rescale;
        if (poisson) v *= -1.0 / k / k;
        out[n2] = (T)v;
    }
}

// The same table for FP32 grids in FP32 arithmetic (the FP64 pipe runs at a small fraction of the
// FP32 rate): the node search runs on the double table with k rounded to float; the power law,
// the interpolation weights and the products in float (a few ulp of the FP64 table's values).
__global__ void k_filter32(int n2max, float dk, float A_s, float ns1, float inv_kp, const double *__restrict__ tab,
                           int k_size, float u_tau, float rescale, int poisson, float *__restrict__ out) {
    for (int n2 = blockIdx.x * blockDim.x + threadIdx.x; n2 <= n2max; n2 += gridDim.x * blockDim.x) {
        if (n2 == 0) { out[0] = 0; continue; }
        const float k = sqrtf((float)n2) * dk;
        float v = sqrtf(A_s * powf(k * inv_kp, ns1) * k * (float)(2. * M_PI * M_PI));
        // transfer_at with the search on doubles (kspace.cuh)
        const double *kt = tab, *lo = tab + k_size, *hi = tab + 2 * k_size;
        const double kd = (double)k;
        int i;
        float u;
        if (kd > kt[k_size - 1]) {
            i = k_size - 2;
            u = 1.f;
        } else {
            int a = 0, b = k_size - 1;
            while (b - a > 1) {
                const int m = (a + b) >> 1;
                if (kt[m] <= kd) a = m; else b = m;
            }
            i = a;
            u = (float)(kd - kt[i]) / (float)(kt[i + 1] - kt[i]);
        }
        const float T11 = (float)lo[i], T21 = (float)lo[i + 1], T12 = (float)hi[i], T22 = (float)hi[i + 1];
        v *= (1.f - u_tau) * ((1.f - u) * T11 + u * T21) + u_tau * ((1.f - u) * T12 + u * T22);
        v *= rescale;
        if (poisson) v *= -1.f / k / k;
        out[n2] = v;
    }
}

static double g_stage_ms[16];
static int g_nstages = 0;

extern "C" int mitos_stage_times(double *ms, int max) {
    for (int i = 0; i < g_nstages && i < max; i++) ms[i] = g_stage_ms[i];
    return g_nstages;
}

struct StageTimer {
    bool on;
    std::vector<cudaEvent_t> ev;
    explicit StageTimer(bool enable) : on(enable) {}
    void mark() {
        if (!on) return;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, stream());
        ev.push_back(e);
    }
    void finish() {
        if (!on) return;
        cudaEventSynchronize(ev.back());
        g_nstages = 0;
        for (size_t i = 1; i < ev.size() && i <= 16; i++) {
            float m = 0;
            cudaEventElapsedTime(&m, ev[i - 1], ev[i]);
            g_stage_ms[g_nstages++] = m;
        }
        for (auto e : ev) cudaEventDestroy(e);
    }
};

// pinned host staging of the transfer rows, one buffer per slot (0, 1: ic_pipeline_submit, 2: the
// synchronous entry point); a slot's buffer is rewritten only after its previous IC completed
static double *table_pinned(int slot, size_t n) {
    static double *buf[3] = {nullptr, nullptr, nullptr};
    static size_t cap[3] = {0, 0, 0};
    if (cap[slot] < n) {
        if (buf[slot]) cudaFreeHost(buf[slot]);
        buf[slot] = nullptr;
        cap[slot] = 0;
        if (cudaMallocHost((void **)&buf[slot], sizeof(double) * n) != cudaSuccess) {
            cudaGetLastError();
            set_error(5, "out of pinned host memory for the transfer table");
            return nullptr;
        }
        cap[slot] = n;
    }
    return buf[slot];
}

__global__ void k_copy_table(const double *__restrict__ src, double *__restrict__ dst, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}
__global__ void k_flag_out(const int *__restrict__ flag, double *__restrict__ dst) { *dst = (double)*flag; }

// the copy stream of the position transfers and the events of the two staging slots:
// pos_event(s, 0) = positions ready on the device, pos_event(s, 1) = their copy done (buffer free)
static cudaStream_t copy_stream() {
    static cudaStream_t s = nullptr;
    if (!s) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    return s;
}
static cudaEvent_t pos_event(int slot, int which) {
    static cudaEvent_t ev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    if (!ev[slot][which]) cudaEventCreateWithFlags(&ev[slot][which], cudaEventDisableTiming);
    return ev[slot][which];
}
static cudaEvent_t acc_event(int slot) {
    static cudaEvent_t ev[2] = {nullptr, nullptr};
    if (!ev[slot]) cudaEventCreateWithFlags(&ev[slot], cudaEventDisableTiming);
    return ev[slot];
}

// splitmix64 seeding (include/random_xorshift.h:38-59) of Seed + rank 0
void mitos::seed_state(uint64_t seed, uint64_t st[4]) {
    uint64_t s = seed;
    for (int i = 0; i < 4; i++) {
        uint64_t r = s;
        s = r + 0x9E3779B97f4A7C15ULL;
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ULL;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBULL;
        st[i] = r ^ (r >> 31);
    }
}

// the reference's 2LPT factors of the velocity potential (src/mitos.c:453-455)
static const double F1_VEL = -0.001147273637728, F2_VEL = 3.19354920304769E-05;

template <typename T>
static int run_pipeline(const struct ic_config *cfg, const double *ktab, const double *tlo, const double *thi,
                        const double *tvlo, const double *tvhi, int k_size, double u_tau, struct ic_result *res,
                        const PipeOpts *opt) {
    const int prec = cfg->precision;
    const int N = cfg->N, M = cfg->M;
    const double L = cfg->boxlen;
    const GridGeom *gp = geom(N, prec);
    if (!gp) return 3;
    const GridGeom &g = *gp;
    const size_t gb1 = (size_t)g.cells * sizeof(cplx<T>);
    const double V = L * L * L;
    const double dk = 2 * M_PI / L;
    // displacement grids: row pitch N + 4 on the lattice-aligned path (16-byte aligned rows for
    // the staged tile copies of the deposit), the reference's N + 2 otherwise
    const bool aligned = lattice_aligned(N, M, L);
    const int disp_pitch = aligned ? N + 4 : N + 2;
    const size_t db1 = (size_t)N * N * disp_pitch * sizeof(T);
    // batched runs (the ensemble): B realisations of cfg with their own start states, every grid
    // of realisation b at b * bs bytes from the first; one launch per pass covers all of them
    const int B = (opt && opt->batch > 1) ? opt->batch : 1;
    const size_t bs = B > 1 ? ((std::max(gb1, db1) + 255) & ~(size_t)255) : 0;
    const bool want_snap = res && (res->coords || res->vels || res->masses || res->ids);
    if (B > 1 && (!opt->states || !opt->acc || cfg->method == MITOS_METHOD_MONGE_AMPERE || !aligned ||
                  (res && res->pos) || want_snap)) {
        set_error(3, "batched runs need device start states and accumulators, a lattice-aligned "
                     "Zel'dovich or 2LPT configuration and no positions");
        return 3;
    }
    const size_t gb = B > 1 ? B * bs : gb1, db = B > 1 ? B * bs : db1;
    const bool want_vel = res && (res->vel || res->vels);
    if (want_vel && (!tvlo || !tvhi || B > 1)) {
        set_error(1, "velocities need a velocity transfer function (ic_config.index_vel) and an unbatched run");
        return 1;
    }
    if (cfg->thermal && (!want_vel || (cfg->thermal != 1 && cfg->thermal != 2) || !(cfg->thermal_M_eV > 0) ||
                         !(cfg->thermal_T_eV > 0))) {
        set_error(1, "thermal motion needs velocities (ic_result.vel), kind 1 or 2, and positive mass and temperature");
        return 1;
    }
    const int acc_stride = 3 * cfg->pk_bins + 2;
    auto reset = [&](PassArgs &x) {
        memset(&x, 0, sizeof x);
        x.batch = B;
        x.bstride = (long long)bs;
        x.acc_stride = acc_stride;
    };
    StageTimer tim(getenv("MITOS_PROFILE") != nullptr);
    tim.mark();

    void *phi = workspace(gb, 0), *S = workspace(gb, 10), *Sk = workspace(gb, 11), *rho = workspace(gb, 12);
    void *A0 = workspace(gb, 1), *A1 = workspace(gb, 2);
    void *B0 = workspace(gb, 4), *B1 = workspace(gb, 5), *B2 = workspace(gb, 6);
    void *D0 = workspace(db, 7), *D1 = workspace(db, 8), *D2 = workspace(db, 9);
    if (!phi || !S || !Sk || !rho || !A0 || !A1 || !B0 || !B1 || !B2 || !D0 || !D1 || !D2) return 5;
    const long n2max = 3L * (N / 2) * (N / 2);
    T *filt = (T *)workspace(sizeof(T) * (n2max + 1), 106);
    // transfer rows [k, lo, hi] of the density function, then (velocities) those of the velocity one
    const int tab_rows = want_vel ? 6 : 3;
    double *dtab = (opt && opt->dtab) ? opt->dtab : (double *)workspace(sizeof(double) * tab_rows * k_size, 107);
    double *acc = (opt && opt->acc) ? opt->acc : (double *)workspace(sizeof(double) * acc_stride, 104);
    if (!filt || !dtab || !acc) return 5;
    double *red = acc + 3 * cfg->pk_bins;

    // inputs: the transfer table rows of the source time (host -> device).  Ensemble runs upload
    // them with a copy once per workspace set (a graph-mode run reuses them: no pageable copies in a
    // capture).  Other runs place them in a pinned buffer of their slot and a small kernel reads
    // them over the link, so no copy engine is involved: the positions of a previous submission may
    // still occupy one for milliseconds.
    if (opt && (opt->graph || opt->acc)) {
        if (!opt->graph) {
            MITOS_CUDA(cudaMemcpyAsync(dtab, ktab, sizeof(double) * k_size, cudaMemcpyHostToDevice, stream()));
            MITOS_CUDA(cudaMemcpyAsync(dtab + k_size, tlo, sizeof(double) * k_size, cudaMemcpyHostToDevice, stream()));
            MITOS_CUDA(cudaMemcpyAsync(dtab + 2 * k_size, thi, sizeof(double) * k_size, cudaMemcpyHostToDevice, stream()));
        }
    } else {
        const int tslot = (opt && opt->async_slot >= 0) ? opt->async_slot : 2;
        double *ht = table_pinned(tslot, (size_t)tab_rows * k_size);
        if (!ht) return 5;
        memcpy(ht, ktab, sizeof(double) * k_size);
        memcpy(ht + k_size, tlo, sizeof(double) * k_size);
        memcpy(ht + 2 * k_size, thi, sizeof(double) * k_size);
        if (want_vel) {
            memcpy(ht + 3 * k_size, ktab, sizeof(double) * k_size);
            memcpy(ht + 4 * k_size, tvlo, sizeof(double) * k_size);
            memcpy(ht + 5 * k_size, tvhi, sizeof(double) * k_size);
        }
        double *hd = nullptr;
        MITOS_CUDA(cudaHostGetDevicePointer((void **)&hd, ht, 0));
        launch_begin("table_in");
        k_copy_table<<<8, 256, 0, stream()>>>(hd, dtab, tab_rows * k_size);
        count_launch();
        MITOS_LAUNCH_CHECK("transfer table upload");
    }
    const bool ma = cfg->method == MITOS_METHOD_MONGE_AMPERE;
    // filter per |n|^2 from the rows at tab, with (poisson = 1) or without the -1/k^2 kernel
    auto filter_launch = [&](const double *tab, int poisson, T *out) {
        int blocks = (int)((n2max + 256) / 256);
        if (blocks > 4096) blocks = 4096;
        launch_begin("filter");
        if constexpr (sizeof(T) == 4)
            k_filter32<<<blocks, 256, 0, stream()>>>((int)n2max, (float)dk, (float)cfg->A_s, (float)(cfg->n_s - 1.),
                                                     (float)(1. / cfg->k_pivot), tab, k_size, (float)u_tau, 1.f,
                                                     poisson, (float *)out);
        else
            k_filter<T><<<blocks, 256, 0, stream()>>>(n2max, dk, cfg->A_s, cfg->n_s, cfg->k_pivot, tab, k_size,
                                                      u_tau, 1.0, poisson, out);
        count_launch();
        const cudaError_t ce = cudaGetLastError();
        return ce == cudaSuccess ? 0 : check_cuda(ce, "filter table");
    };
    if (int fe = filter_launch(dtab, ma ? 0 : 1, filt)) return fe;
    tim.mark();

    // S1: noise (src/mitos.c:148,220-224 + generatePerturbationGrid)
    uint64_t st[4];
    seed_state(cfg->seed, st);
    int e;
    void *dens_k = ma ? Sk : phi;  // Monge-Ampere keeps delta(k) to build rho(x)
    // the lattice-aligned deposit's density grid (row pitch N + 4), cleared on the side by the
    // 2LPT-source Z pass (latency-bound, with HBM bandwidth to spare) or else by the noise kernel
    const int rho_pitch = aligned ? N + 4 : N + 2;
    const size_t rho_bytes = B > 1 ? db : (size_t)N * N * rho_pitch * (sizeof(T));
    void *rhoA = aligned ? workspace(rho_bytes, 15) : nullptr;
    if (aligned && !rhoA) return 5;
    const bool clear_in_z = aligned && cfg->method == MITOS_METHOD_2LPT;
    e = noise_generate(g, prec, L, st, filt, dens_k, B > 1 ? opt->states : nullptr, B, bs,
                       clear_in_z ? nullptr : rhoA, aligned && !clear_in_z ? rho_bytes : 0);
    if (!e) e = hermitian_planes(g, prec, dens_k, B, bs);
    if (e) return e;
    tim.mark();

    PassArgs a;
    int win_disp = 3;
    bool fused_disp_x = false;
    int iters = 0;
    double last_rel = 0;
    if (cfg->method == MITOS_METHOD_2LPT) {
        // S2: Hessians + source, and the source's r2c along z in the same Z pass
        e = grid_hessian(g, prec, L, phi, ZOP_HESS_2LPT_K, nullptr, Sk, nullptr, 0, nullptr, B, bs,
                         clear_in_z ? rhoA : nullptr, clear_in_z ? rho_bytes : 0);
        if (e) return e;
        tim.mark();
        // S3: the rest of the S r2c -> phi = f1 phi1 + f2 (-1/k^2) S, TSC window undone
        // (src/2lpt.c:125-136)
        reset(a);
        a.dk = dk;
        a.scale = 1.0;
        a.in[0] = Sk;
        a.out[0] = Sk;
        e = launch_y<T>(g, YOP_PLAIN, -1, a);
        a.in2 = phi;
        a.scale = V / ((double)N * N * N);
        a.f1 = 1.0;
        a.f2 = -3. / 7.;  // src/mitos.c:385
        a.window_order = 3;
        fused_disp_x = true;  // the X pass of the displacement grids runs inside this one
        a.out[0] = A0;
        a.out[1] = A1;
        a.stencil = lattice_aligned(N, M, L) ? stencil_table(N, prec) : nullptr;
        if (!e) e = launch_x<T>(g, XOP_COMBINE_DISP, -1, a);
        if (e) return e;
        win_disp = 0;
        tim.mark();
    } else if (ma) {
        // rho(x) = c2r(delta(k)) and phi = -delta/k^2 (src/monge_ampere.c:87-90)
        void *rhoR = workspace(gb, 13);
        void *tmp = workspace(gb, 14);
        if (!rhoR || !tmp) return 5;
        KernelParams kp;
        memset(&kp, 0, sizeof kp);
        kp.id = KID_INV_POISSON;
        e = apply_kernel_launch(N, L, prec, kp, Sk, phi);
        if (!e) { MITOS_CUDA(cudaMemcpyAsync(tmp, Sk, gb, cudaMemcpyDeviceToDevice, stream())); }
        if (!e) e = grid_c2r(g, prec, L, tmp, rhoR);
        if (e) return e;
        tim.mark();
        const int maxc = cfg->ma_cycles > 0 ? cfg->ma_cycles : 1;
        for (int it = 0; it < maxc; it++) {
            MITOS_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(double), stream()));
            // the residual with its z r2c in the Z pass (into Sk), then the Y and X steps
            e = grid_hessian(g, prec, L, phi, ZOP_HESS_MA_K, rhoR, Sk, red, 0);
            if (e) return e;
            reset(a);
            a.dk = dk;
            a.scale = 1.0;
            a.in[0] = Sk;
            a.out[0] = Sk;
            e = launch_y<T>(g, YOP_PLAIN, -1, a);
            a.in2 = phi;
            a.out[0] = phi;
            a.scale = V / ((double)N * N * N);
            if (!e) e = launch_x<T>(g, XOP_ADD_POISSON, -1, a);
            if (e) return e;
            double h[2];
            MITOS_CUDA(cudaMemcpyAsync(h, red, sizeof h, cudaMemcpyDeviceToHost, stream()));
            MITOS_CUDA(cudaStreamSynchronize(stream()));
            iters = it + 1;
            last_rel = sqrt(h[0] / h[1]);
            if (cfg->ma_tol > 0 && last_rel <= cfg->ma_tol) break;
        }
        tim.mark();
    } else {
        tim.mark();
        tim.mark();
    }

    // S4: displacement grids d_i = c2r(i k_i phi W^-3) (src/mitos.c:395-416)
    reset(a);
    a.dk = dk;
    a.scale = 1.0;
    a.window_order = win_disp;
    a.stencil = aligned ? stencil_table(N, prec) : nullptr;
    if (aligned && !a.stencil) return 5;
    a.in[0] = phi;
    a.out[0] = A0;
    a.out[1] = A1;
    if (!fused_disp_x) e = launch_x<T>(g, XOP_DISP, +1, a);
    if (e) return e;
    a.window_order = 0;
    // Y: [B0, B1, B2] = [A1, i ky A0, A0], the y stencil on the d_x and d_y chains (B0, B1)
    a.in[0] = A0;
    a.out[0] = B1;
    a.out[1] = B2;
    e = launch_y<T>(g, YOP_DISP_A, +1, a);
    a.in[0] = A1;
    a.out[0] = B0;
    if (!e) e = launch_y<T>(g, YOP_STN, +1, a);
    if (e) return e;
    a.in[0] = B0;
    a.in[1] = B1;
    a.in[2] = B2;
    a.out[0] = D0;
    a.out[1] = D1;
    a.out[2] = D2;
    a.rp_out = disp_pitch;
    a.scale = 1.0 / V;
    e = launch_z_c2r<T>(g, ZOP_DISP, a);
    if (e) return e;
    tim.mark();

    // S5: particles + CIC.  The positions are staged in a device buffer of the run's slot (for the
    // caller's res->pos and for the snapshot datasets) and copied to the caller on the copy stream as
    // soon as the deposit ends, under the P(k) passes (and, for ic_pipeline_submit, under the next
    // IC); the buffer is reused once its last copy is done.
    float *dpos = nullptr, *dposraw = nullptr;
    const int pslot = (opt && opt->async_slot >= 0) ? opt->async_slot : 0;
    const size_t pos_bytes = sizeof(float) * 3 * (size_t)M * M * M;
    if (res && (res->pos || want_snap)) {
        dpos = (float *)workspace(pos_bytes, 108 + pslot);
        if (!dpos) return 5;
    }
    if (want_vel) {
        dposraw = (float *)workspace(pos_bytes, 112);  // the velocity gather's unwrapped positions
        if (!dposraw) return 5;
    }
    // the slot's staging buffers are free once their previous copies are done
    if (dpos || want_vel) MITOS_CUDA(cudaStreamWaitEvent(stream(), pos_event(pslot, 1), 0));
    int *therr = nullptr;  // thermal motion: bit 0 set for an invalid momentum
    // the aligned deposit uses a row pitch of N + 4 reals (16-byte aligned rows for vector
    // reductions) into the grid the noise kernel cleared; the general path into rho
    void *rhoD = aligned ? rhoA : rho;
    if (!rhoD) return 5;
    if (!aligned) MITOS_CUDA(cudaMemsetAsync(rhoD, 0, rho_bytes, stream()));
    e = aligned ? lattice_deposit(N, L, prec, D0, D1, D2, disp_pitch, rhoD, rho_pitch, dpos, B, bs, dposraw)
                : displace_and_deposit(N, M, L, prec, D0, D1, D2, rhoD, dpos, dposraw);
    if (e) return e;
    if (res && res->pos) {
        MITOS_CUDA(cudaEventRecord(pos_event(pslot, 0), stream()));
        MITOS_CUDA(cudaStreamWaitEvent(copy_stream(), pos_event(pslot, 0), 0));
        MITOS_CUDA(cudaMemcpyAsync(res->pos, dpos, pos_bytes, cudaMemcpyDeviceToHost, copy_stream()));
        MITOS_CUDA(cudaEventRecord(pos_event(pslot, 1), copy_stream()));
    }
    tim.mark();

    // Velocities (src/mitos.c:425-490, :865-908): the same noise through the velocity transfer
    // function (z_source = z_ini: rescale 1, :431-436) and the -1/k^2 kernel, the velocity potential
    // by 2LPT with the reference's velocity factors for 2LPT configurations (:453-455) or that first
    // order potential otherwise (:457), the TSC window undone (:461-467), three derivative grids
    // (:470-483, pitch N + 2, no on-node stencil: the gather is at displaced positions), and the
    // TSC gather of each at the unwrapped positions.  Every workspace of S1-S4 is free again here.
    float *dvel = nullptr;
    if (want_vel) {
        T *filtv = (T *)workspace(sizeof(T) * (n2max + 1), 116);
        // velocity grids: pitch N + 4 for the lattice-aligned gather (16-byte aligned rows for its
        // tile staging), N + 2 otherwise
        const int vpitch = aligned ? N + 4 : N + 2;
        const size_t vb = (size_t)N * N * vpitch * sizeof(T);
        void *V0 = workspace(vb, 19), *V1 = workspace(vb, 20), *V2 = workspace(vb, 21);
        dvel = (float *)workspace(pos_bytes, 110 + pslot);
        if (!filtv || !V0 || !V1 || !V2 || !dvel) return 5;
        if ((e = filter_launch(dtab + 3 * k_size, 1, filtv))) return e;
        e = noise_generate(g, prec, L, st, filtv, phi);
        if (!e) e = hermitian_planes(g, prec, phi);
        if (e) return e;
        if (cfg->method == MITOS_METHOD_2LPT) {
            e = grid_hessian(g, prec, L, phi, ZOP_HESS_2LPT_K, nullptr, Sk, nullptr, 0);
            if (e) return e;
            reset(a);
            a.dk = dk;
            a.scale = 1.0;
            a.in[0] = Sk;
            a.out[0] = Sk;
            e = launch_y<T>(g, YOP_PLAIN, -1, a);
            a.in2 = phi;
            a.scale = V / ((double)N * N * N);
            a.f1 = F1_VEL;
            a.f2 = F2_VEL;
            a.window_order = 3;
            a.out[0] = A0;
            a.out[1] = A1;
            a.stencil = nullptr;
            if (!e) e = launch_x<T>(g, XOP_COMBINE_DISP, -1, a);
        } else {
            reset(a);
            a.dk = dk;
            a.scale = 1.0;
            a.window_order = 3;
            a.in[0] = phi;
            a.out[0] = A0;
            a.out[1] = A1;
            e = launch_x<T>(g, XOP_DISP, +1, a);
        }
        if (e) return e;
        reset(a);
        a.dk = dk;
        a.scale = 1.0;
        a.in[0] = A0;
        a.out[0] = B1;
        a.out[1] = B2;
        e = launch_y<T>(g, YOP_DISP_A, +1, a);
        a.in[0] = A1;
        a.out[0] = B0;
        if (!e) e = launch_y<T>(g, YOP_STN, +1, a);
        if (e) return e;
        a.in[0] = B0;
        a.in[1] = B1;
        a.in[2] = B2;
        a.out[0] = V0;
        a.out[1] = V1;
        a.out[2] = V2;
        a.rp_out = vpitch;
        a.scale = 1.0 / V;
        e = launch_z_c2r<T>(g, ZOP_DISP, a);
        if (!e) e = velocity_gather((long)M * M * M, N, vpitch, L, prec, dposraw, V0, V1, V2, dvel);
        if (e) return e;
        // thermal motion (src/mitos.c:910-1064) from the stream the white noise left: four draws a
        // mode with k > 0 (src/grf.c:47-63), then those of earlier thermal species
        if (cfg->thermal) {
            therr = (int *)workspace(sizeof(int), 153 + pslot);
            if (!therr) return 5;
            MITOS_CUDA(cudaMemsetAsync(therr, 0, sizeof(int), stream()));
            const unsigned long long skip = 4ULL * ((unsigned long long)N * N * (N / 2 + 1) - 1) + cfg->thermal_draw_offset;
            e = thermal_add(prec, (long)M * M * M, st, skip, cfg->thermal, cfg->thermal_T_eV, cfg->thermal_M_eV,
                            1.0 / (1.0 + cfg->z_ini), cfg->speed_of_light, dvel, 3, therr);
            if (e) return e;
        }
        // to the caller on the copy stream, behind the positions (pos_event(pslot, 1) then covers both)
        if (res->vel) {
            MITOS_CUDA(cudaEventRecord(pos_event(pslot, 0), stream()));
            MITOS_CUDA(cudaStreamWaitEvent(copy_stream(), pos_event(pslot, 0), 0));
            MITOS_CUDA(cudaMemcpyAsync(res->vel, dvel, pos_bytes, cudaMemcpyDeviceToHost, copy_stream()));
            MITOS_CUDA(cudaEventRecord(pos_event(pslot, 1), copy_stream()));
        }
    }

    // the particle datasets of the snapshot (src/mitos.c:1106-1117), made on the device from the
    // wrapped positions and the velocities, to the caller on the copy stream behind the rest
    if (want_snap) {
        const long np = (long)M * M * M;
        double *dc = res->coords ? (double *)workspace(2 * pos_bytes, 160 + 4 * pslot) : nullptr;
        double *dv = res->vels ? (double *)workspace(2 * pos_bytes, 161 + 4 * pslot) : nullptr;
        double *dm = res->masses ? (double *)workspace(sizeof(double) * np, 162 + 4 * pslot) : nullptr;
        long long *di = res->ids ? (long long *)workspace(sizeof(long long) * np, 163 + 4 * pslot) : nullptr;
        if ((res->coords && !dc) || (res->vels && !dv) || (res->masses && !dm) || (res->ids && !di)) return 5;
        e = snapshot_arrays(np, dpos, dvel, (float)cfg->particle_mass, cfg->id_first_particle, dc, dv, dm, di);
        if (e) return e;
        MITOS_CUDA(cudaEventRecord(pos_event(pslot, 0), stream()));
        MITOS_CUDA(cudaStreamWaitEvent(copy_stream(), pos_event(pslot, 0), 0));
        if (dc) MITOS_CUDA(cudaMemcpyAsync(res->coords, dc, 2 * pos_bytes, cudaMemcpyDeviceToHost, copy_stream()));
        if (dv) MITOS_CUDA(cudaMemcpyAsync(res->vels, dv, 2 * pos_bytes, cudaMemcpyDeviceToHost, copy_stream()));
        if (dm) MITOS_CUDA(cudaMemcpyAsync(res->masses, dm, sizeof(double) * np, cudaMemcpyDeviceToHost, copy_stream()));
        if (di) MITOS_CUDA(cudaMemcpyAsync(res->ids, di, sizeof(long long) * np, cudaMemcpyDeviceToHost, copy_stream()));
        MITOS_CUDA(cudaEventRecord(pos_event(pslot, 1), copy_stream()));
    }

    // the deposit's and the velocity gather's tile-copy fault flag to the host (read after the
    // final synchronisation)
    if (aligned && !(opt && opt->graph)) {
        e = lattice_fault_fetch();
        if (e) return e;
    }
    // S6: overdensity r2c, CIC window undo, P(k) (analyse/src/mitos_read.c:364-419)
    const int *bins = bin_table(N, cfg->pk_bins, cfg->pk_linear, L);
    if (!bins) return 5;
    MITOS_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * ((size_t)(B - 1) * acc_stride + 3 * cfg->pk_bins), stream()));
    reset(a);
    a.dk = dk;
    a.scale = 1.0;
    a.in[0] = rhoD;
    a.out[0] = Sk;
    a.rp_in = rho_pitch;
    a.rho_a = 1.0;
    a.rho_b = -1.0;
    e = grid_r2c_zy(g, sizeof(T) == 4 ? MITOS_FP32 : MITOS_FP64, a);
    a.in[0] = Sk;
    a.rho_a = 1.0;
    a.rho_b = 0.0;
    a.out[0] = nullptr;
    a.scale = V / ((double)N * N * N);
    a.window_order = 2;
    a.bin_of_n2 = bins;
    a.nbins = cfg->pk_bins;
    a.bin_k = acc;
    a.bin_p = acc + cfg->pk_bins;
    a.bin_n = (long long *)(acc + 2 * cfg->pk_bins);
    if (!e) e = launch_x<T>(g, XOP_PK, -1, a);
    if (e) return e;
    tim.mark();
    if (opt && opt->graph) return 0;  // results stay in opt->acc
    if (opt && opt->async_slot >= 0) {
        // the power sums go to the slot's pinned buffer through a kernel's stores, not a copy
        // engine (which the positions may occupy); the host finishes the bins at wait time
        double *hd = nullptr;
        MITOS_CUDA(cudaHostGetDevicePointer((void **)&hd, opt->acc_host, 0));
        launch_begin("pk_out");
        k_copy_table<<<1, 256, 0, stream()>>>(acc + cfg->pk_bins, hd, cfg->pk_bins);
        count_launch();
        MITOS_LAUNCH_CHECK("P(k) sums to the host");
        opt->acc_host[cfg->pk_bins] = 0;
        if (therr) {
            launch_begin("flag_out");
            k_flag_out<<<1, 1, 0, stream()>>>(therr, hd + cfg->pk_bins);
            count_launch();
            MITOS_LAUNCH_CHECK("thermal flag to the host");
        }
        MITOS_CUDA(cudaEventRecord(acc_event(opt->async_slot), stream()));
        if (opt->iters) *opt->iters = iters;
        if (opt->last_rel) *opt->last_rel = last_rel;
        return 0;
    }

    if (res) {
        const double *ksum;
        const long long *count;
        e = bin_geometry(N, cfg->pk_bins, cfg->pk_linear, L, &ksum, &count);
        if (e) return e;
        std::vector<double> h(cfg->pk_bins);
        MITOS_CUDA(cudaMemcpyAsync(h.data(), acc + cfg->pk_bins, sizeof(double) * cfg->pk_bins,
                                   cudaMemcpyDeviceToHost, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
        if (dpos || want_vel) MITOS_CUDA(cudaEventSynchronize(pos_event(pslot, 1)));
        if ((e = lattice_fault_check())) return e;
        if (therr) {
            int h = 0;
            MITOS_CUDA(cudaMemcpy(&h, therr, sizeof(int), cudaMemcpyDeviceToHost));
            if (h) {
                set_error(8, "thermal motion: invalid thermal momentum drawn");
                return 8;
            }
        }
        for (int i = 0; i < cfg->pk_bins; i++) {
            const double n = (double)count[i];
            if (res->pk_obs) res->pk_obs[i] = (long)count[i];
            if (res->pk_k) res->pk_k[i] = ksum[i] / n;
            if (res->pk_p) res->pk_p[i] = h[i] / n / V;
        }
        res->ma_iterations = iters;
        res->ma_residual = last_rel;
    } else {
        MITOS_CUDA(cudaStreamSynchronize(stream()));
        if ((e = lattice_fault_check())) return e;
    }
    tim.finish();
    return 0;
}

int mitos::pipeline_table(const struct ic_config *cfg, int k_size, int tau_size, int n_functions, const double *k,
                          const double *log_tau, const double *redshift, const double *D_growth, const double *delta,
                          struct ic_result *res, const PipeOpts *opt) {
    if (!cfg || cfg->N < 16 || cfg->M < 1 || cfg->boxlen <= 0 || cfg->pk_bins < 1) {
        set_error(1, "invalid ic_config");
        return 1;
    }
    if (cfg->index_src < 0 || cfg->index_src >= n_functions) {
        set_error(1, "transfer function index %d out of range", cfg->index_src);
        return 1;
    }
    struct perturb_data pd;
    memset(&pd, 0, sizeof pd);
    pd.k_size = k_size;
    pd.tau_size = tau_size;
    pd.n_functions = n_functions;
    pd.k = (double *)k;
    pd.log_tau = (double *)log_tau;
    pd.redshift = (double *)redshift;
    pd.D_growth = (double *)D_growth;
    pd.delta = (double *)delta;
    // src/mitos.c:151-153 with z_source = z_ini (rescale factor 1, :357-362)
    const double lt = log_tau_at_z_h(&pd, cfg->z_ini);
    int tau_index;
    double u_tau;
    find_tau_h(&pd, lt, &tau_index, &u_tau);
    const double *arr = delta + (long)cfg->index_src * k_size * tau_size;
    const double *tlo = arr + (long)k_size * tau_index, *thi = arr + (long)k_size * (tau_index + 1);
    // the velocity transfer function's rows at the same time (used when res->vel or res->vels is set)
    const double *tvlo = nullptr, *tvhi = nullptr;
    if (cfg->index_vel >= 0 && cfg->index_vel < n_functions) {
        const double *va = delta + (long)cfg->index_vel * k_size * tau_size;
        tvlo = va + (long)k_size * tau_index;
        tvhi = va + (long)k_size * (tau_index + 1);
    }
    if (cfg->precision == MITOS_FP32) return run_pipeline<float>(cfg, k, tlo, thi, tvlo, tvhi, k_size, u_tau, res, opt);
    if (cfg->precision == MITOS_FP64) return run_pipeline<double>(cfg, k, tlo, thi, tvlo, tvhi, k_size, u_tau, res, opt);
    set_error(3, "unknown precision %d", cfg->precision);
    return 3;
}

extern "C" int ic_pipeline_run_table(const struct ic_config *cfg, int k_size, int tau_size, int n_functions,
                                     const double *k, const double *log_tau, const double *redshift,
                                     const double *D_growth, const double *delta, struct ic_result *res) {
    return pipeline_table(cfg, k_size, tau_size, n_functions, k, log_tau, redshift, D_growth, delta, res, nullptr);
}

int mitos::pipeline_spline(const struct ic_config *cfg, const struct perturb_spline *spline, struct ic_result *res,
                           const PipeOpts *opt) {
    if (!spline || !spline->ptdat) {
        set_error(1, "missing perturbation spline");
        return 1;
    }
    const struct perturb_data *pd = spline->ptdat;
    return pipeline_table(cfg, pd->k_size, pd->tau_size, pd->n_functions, pd->k, pd->log_tau, pd->redshift,
                          pd->D_growth, pd->delta, res, opt);
}

extern "C" int ic_pipeline_run(const struct ic_config *cfg, const struct perturb_spline *spline,
                               struct ic_result *res) {
    return pipeline_spline(cfg, spline, res, nullptr);
}

// ---- asynchronous submission: two ICs in flight, the positions of one travelling under the
// compute of the next --------------------------------------------------------------------------
namespace {
struct AsyncSlot {
    bool busy = false;
    struct ic_config cfg;
    struct ic_result *res = nullptr;
    double *acc_host = nullptr;
    int acc_cap = 0;
    int iters = 0;
    double last_rel = 0;
    long order = 0;
};
AsyncSlot g_slot[2];
int g_next = 0;
long g_order = 0;

int finish_slot(int k) {
    AsyncSlot &s = g_slot[k];
    if (!s.busy) return 0;
    s.busy = false;
    MITOS_CUDA(cudaEventSynchronize(acc_event(k)));
    if (s.res && (s.res->pos || s.res->vel || s.res->coords || s.res->vels || s.res->masses || s.res->ids))
        MITOS_CUDA(cudaEventSynchronize(pos_event(k, 1)));
    if (const int f = lattice_fault_check()) return f;
    if (!s.res) return 0;
    const double *ksum;
    const long long *count;
    int e = bin_geometry(s.cfg.N, s.cfg.pk_bins, s.cfg.pk_linear, s.cfg.boxlen, &ksum, &count);
    if (e) return e;
    const double V = s.cfg.boxlen * s.cfg.boxlen * s.cfg.boxlen;
    for (int i = 0; i < s.cfg.pk_bins; i++) {
        const double n = (double)count[i];
        if (s.res->pk_obs) s.res->pk_obs[i] = (long)count[i];
        if (s.res->pk_k) s.res->pk_k[i] = ksum[i] / n;
        if (s.res->pk_p) s.res->pk_p[i] = s.acc_host[i] / n / V;
    }
    s.res->ma_iterations = s.iters;
    s.res->ma_residual = s.last_rel;
    if (s.acc_host[s.cfg.pk_bins] != 0) {
        set_error(8, "thermal motion: invalid thermal momentum drawn");
        return 8;
    }
    return 0;
}
}  // namespace

extern "C" int ic_pipeline_submit(const struct ic_config *cfg, const struct perturb_spline *spline,
                                  struct ic_result *res) {
    if (!cfg || cfg->pk_bins < 1) {
        set_error(1, "invalid ic_config");
        return 1;
    }
    const int k = g_next;
    int e = finish_slot(k);  // the slot's previous IC (submitted two calls ago)
    if (e) return e;
    AsyncSlot &s = g_slot[k];
    if (s.acc_cap < cfg->pk_bins) {
        if (s.acc_host) cudaFreeHost(s.acc_host);
        s.acc_host = nullptr;
        s.acc_cap = 0;
        // P(k) sums, then the thermal-motion flag
        if (cudaMallocHost(&s.acc_host, sizeof(double) * (cfg->pk_bins + 1)) != cudaSuccess) {
            cudaGetLastError();
            set_error(5, "out of pinned host memory for the P(k) sums");
            return 5;
        }
        s.acc_cap = cfg->pk_bins;
    }
    PipeOpts o;
    o.acc = nullptr;
    o.graph = false;
    o.async_slot = k;
    o.acc_host = s.acc_host;
    o.iters = &s.iters;
    o.last_rel = &s.last_rel;
    e = pipeline_spline(cfg, spline, res, &o);
    if (e) return e;
    s.busy = true;
    s.cfg = *cfg;
    s.res = res;
    s.order = g_order++;
    g_next = k ^ 1;
    return 0;
}

extern "C" int ic_pipeline_wait(void) {
    const int first = (g_slot[0].busy && g_slot[1].busy && g_slot[1].order < g_slot[0].order) ? 1 : 0;
    int e = finish_slot(first);
    const int e2 = finish_slot(first ^ 1);
    return e ? e : e2;
}
