// ma.cu -- Monge-Ampere iteration to a tolerance (src/monge_ampere.c:50-183 with the update kept
// in k space) and its learned warm start.
//
// One cycle: the six Hessian components of phi(k) through the fused X / Y / Z passes, the residual
// res = (1 + rho) - det(I + H) with FP64 sums of res^2 and rho^2 in the last pass
// (src/monge_ampere.c:96-145), then phi(k) += G(k) r2c(res)(k) with G = -1/k^2 (DC 1,
// include/fft_kernels.h:96-99).  The reference applies the same update through real space
// (solvePoisson_dg, c2r(phi), phi += res', r2c(phi), src/monge_ampere.c:154-165); in FP32 that round
// trip of phi leaves a residual floor near 5e-5 (white round-off in phi, amplified by k^2 in the
// Hessian), while the k-space update follows the FP64 iteration down to 1e-6.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "context.cuh"
#include "grids.cuh"
#include "kspace.cuh"

namespace mitos {

// out(k) = -|k|^2 (a(k) - b(k))  (the Laplacian of a difference of potentials)
template <typename T>
__global__ void k_lap_diff(int N, T dk, const cplx<T> *__restrict__ a, const cplx<T> *__restrict__ b,
                           cplx<T> *__restrict__ out) {
    const int H = N / 2 + 1;
    const long n = (long)N * N * H;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int kz = (int)(i % H), y = (int)((i / H) % N), x = (int)(i / ((long)H * N));
        const T kx = (T)kint(x, N) * dk, ky = (T)kint(y, N) * dk, kzz = (T)kz * dk;
        const T f = -(kx * kx + ky * ky + kzz * kzz);
        const cplx<T> d = csub<T>(a[i], b[i]);
        out[i] = cscale<T>(d, f);
    }
}

template <typename T>
static int lap_diff(const GridGeom &g, double boxlen, const void *a, const void *b, void *out) {
    const long n = g.cells;
    const unsigned blocks = (unsigned)std::min<long>((n + 255) / 256, 152L * 16);
    launch_begin("lap_diff");
    k_lap_diff<T><<<blocks, 256, 0, stream()>>>(g.N, (T)(2 * M_PI / boxlen), (const cplx<T> *)a, (const cplx<T> *)b,
                                               (cplx<T> *)out);
    count_launch();
    MITOS_LAUNCH_CHECK("laplacian of a difference");
    return 0;
}

// phi(k) += G(k) r2c(src)(k): src real (pitch N + 2); Sk complex scratch
static int add_poisson(const GridGeom &g, int prec, double boxlen, const void *src, void *phi, void *Sk) {
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.dk = 2 * M_PI / boxlen;
    a.scale = 1.0;
    a.in[0] = src;
    a.out[0] = Sk;
    a.rp_in = g.N + 2;
    a.rho_a = 1.0;
    int e = prec == MITOS_FP32 ? launch_z_r2c<float>(g, a) : launch_z_r2c<double>(g, a);
    if (e) return e;
    a.in[0] = Sk;
    e = prec == MITOS_FP32 ? launch_y<float>(g, YOP_PLAIN, -1, a) : launch_y<double>(g, YOP_PLAIN, -1, a);
    if (e) return e;
    a.in2 = phi;
    a.out[0] = phi;
    a.scale = boxlen * boxlen * boxlen / ((double)g.N * g.N * g.N);
    return prec == MITOS_FP32 ? launch_x<float>(g, XOP_ADD_POISSON, -1, a) : launch_x<double>(g, XOP_ADD_POISSON, -1, a);
}

// real out (pitch N + 2) = c2r(G(k) r2c(src)(k)): the potential of a source
static int poisson_real(const GridGeom &g, int prec, double boxlen, const void *src, void *Sk, void *out) {
    int e = grid_r2c(g, prec, boxlen, src, g.N + 2, 1.0, 0.0, Sk);
    if (e) return e;
    KernelParams kp;
    memset(&kp, 0, sizeof kp);
    kp.id = KID_INV_POISSON;
    e = apply_kernel_launch(g.N, boxlen, prec, kp, Sk, Sk);
    if (e) return e;
    return grid_c2r(g, prec, boxlen, Sk, out);
}

struct MAFields {
    // training-pair capture (device FP32 real grids, pitch N + 2), or null
    float *delta, *phi1, *phi2, *sigma;
};

// the iteration; warm (optional) applies the network's correction after the first update;
// cap (optional) captures a training pair; returns 0, 7 (tolerance not reached) or an error
static int ma_run(struct distributed_grid *pot, struct distributed_grid *dens, struct distributed_grid *work,
                  double tol, int max_cycles, struct manet *warm, struct ma_stats *st, const MAFields *cap) {
    const int N = dens->N, prec = dens->precision;
    const double L = dens->boxlen;
    const GridGeom *gp = geom(N, prec);
    if (!gp) return 3;
    const GridGeom &g = *gp;
    if ((warm || cap) && prec != MITOS_FP32) {
        set_error(3, "the network warm start and its training pairs run on FP32 grids");
        return 3;
    }
    const size_t gb = (size_t)g.cells * csize(prec);
    void *Sk = workspace(gb, 30), *S = workspace(gb, 31);
    double *red = (double *)workspace(2 * sizeof(double), 103);
    if (!Sk || !S || !red) return 5;
    cudaEvent_t ev[3];
    for (int i = 0; i < 3; i++) MITOS_CUDA(cudaEventCreate(&ev[i]));
    MITOS_CUDA(cudaEventRecord(ev[0], stream()));
    memset(st, 0, sizeof *st);

    // phi = -delta/k^2 (Zel'dovich, src/monge_ampere.c:87) and the reference's r2c of the density
    // (src/monge_ampere.c:90; the box, rho(x), is preserved)
    KernelParams kp;
    memset(&kp, 0, sizeof kp);
    kp.id = KID_INV_POISSON;
    int e = apply_kernel_launch(N, L, prec, kp, dens->fbox, pot->fbox);
    if (!e) e = fft_r2c_dg(dens);
    pot->momentum_space = 1;
    void *phi1k = nullptr, *phi_first = nullptr;
    if (!e && cap) {
        phi1k = workspace(gb, 32);
        phi_first = workspace(gb, 33);
        if (!phi1k || !phi_first) e = 5;
        else MITOS_CUDA(cudaMemcpyAsync(phi1k, pot->fbox, gb, cudaMemcpyDeviceToDevice, stream()));
    }
    const double n15 = pow((double)N, 1.5);
    int status = 0;
    for (int it = 0; !e; it++) {
        MITOS_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(double), stream()));
        const bool want_S = it == 0 && (warm || cap);
        e = grid_hessian(g, prec, L, pot->fbox, ZOP_HESS_MA, dens->box, work->box, red, 0, want_S ? S : nullptr);
        if (e) break;
        double h[2];
        MITOS_CUDA(cudaMemcpyAsync(h, red, sizeof h, cudaMemcpyDeviceToHost, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
        const double rel = sqrt(h[0] / h[1]);
        st->evaluations++;
        st->rel = rel;
        st->eps = rel / n15;  // src/monge_ampere.c:177
        if (it == 0) st->rel_first = rel;
        if (it == 1) st->rel_second = rel;
        if (rel <= tol && !cap) break;
        if (st->cycles >= max_cycles) {
            if (!cap) status = 7;
            break;
        }
        e = add_poisson(g, prec, L, work->box, pot->fbox, Sk);
        if (e) break;
        st->cycles++;
        if (it == 0 && (warm || cap)) {
            // network inputs: delta(x) (the density box), phi_1(x), phi_2(x) = c2r(G S(k))
            MITOS_CUDA(cudaEventRecord(ev[1], stream()));
            float *d1 = cap ? cap->phi1 : (float *)workspace(gb, 34);
            float *d2 = cap ? cap->phi2 : (float *)workspace(gb, 35);
            float *sg = (float *)workspace(gb, 36);
            void *tmp = workspace(gb, 37);
            if (!d1 || !d2 || !sg || !tmp) { e = 5; break; }
            e = apply_kernel_launch(N, L, prec, kp, dens->fbox, tmp);  // phi_1(k) = -delta/k^2
            if (!e) e = grid_c2r(g, prec, L, tmp, d1);
            if (!e) e = poisson_real(g, prec, L, S, Sk, d2);
            if (e) break;
            if (cap) {
                MITOS_CUDA(cudaMemcpyAsync(cap->delta, dens->box, gb, cudaMemcpyDeviceToDevice, stream()));
                MITOS_CUDA(cudaMemcpyAsync(phi_first, pot->fbox, gb, cudaMemcpyDeviceToDevice, stream()));
            } else {
                e = manet_infer(warm, N, N + 2, (const float *)dens->box, d1, d2, sg);
                if (!e) e = add_poisson(g, prec, L, sg, pot->fbox, Sk);
                if (e) break;
            }
            MITOS_CUDA(cudaEventRecord(ev[2], stream()));
            MITOS_CUDA(cudaEventSynchronize(ev[2]));
            float wms = 0;
            cudaEventElapsedTime(&wms, ev[1], ev[2]);
            st->ms_warm = wms;
        }
    }
    if (!e && cap) {
        // sigma = lap(phi_final - phi_after_first_update)
        e = lap_diff<float>(g, L, pot->fbox, phi_first, Sk);
        if (!e) e = grid_c2r(g, prec, L, Sk, cap->sigma);
    }
    MITOS_CUDA(cudaEventRecord(ev[2], stream()));
    MITOS_CUDA(cudaEventSynchronize(ev[2]));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[0], ev[2]);
    st->ms = ms;
    for (int i = 0; i < 3; i++) cudaEventDestroy(ev[i]);
    (void)phi1k;
    return e ? e : status;
}

}  // namespace mitos

using namespace mitos;

static int check_ma_grids(struct distributed_grid *p, struct distributed_grid *d, struct distributed_grid *w) {
    if (!p || !d || !w || p->N != d->N || d->N != w->N || p->precision != d->precision ||
        d->precision != w->precision) {
        set_error(1, "grids differ in size or precision");
        return 1;
    }
    if (p->box == d->box || w->box == d->box || p->box == w->box) {
        set_error(1, "potential, density and workspace must be distinct grids");
        return 1;
    }
    if (d->momentum_space != 1) {
        set_error(1, "Density grid is not in momentum space");
        return 1;
    }
    return 0;
}

extern "C" int solveMongeAmpereTol(struct distributed_grid *pot, struct distributed_grid *dens,
                                   struct distributed_grid *work, double tol, int max_cycles, struct manet *warm,
                                   struct ma_stats *stats) {
    struct ma_stats local;
    if (!stats) stats = &local;
    int e = check_ma_grids(pot, dens, work);
    if (e) return e;
    e = ma_run(pot, dens, work, tol, max_cycles, warm, stats, nullptr);
    if (e == 7) set_error(7, "Monge-Ampere residual %.3e above the tolerance %.3e after %d cycles", stats->rel, tol,
                          stats->cycles);
    return e;
}

extern "C" int manet_training_pair(struct distributed_grid *pot, struct distributed_grid *dens,
                                   struct distributed_grid *work, int cycles, float *delta, float *phi1, float *phi2,
                                   float *sigma, struct ma_stats *stats) {
    struct ma_stats local;
    if (!stats) stats = &local;
    int e = check_ma_grids(pot, dens, work);
    if (e) return e;
    if (!delta || !phi1 || !phi2 || !sigma || cycles < 1) return 1;
    MAFields cap = {delta, phi1, phi2, sigma};
    return ma_run(pot, dens, work, 0.0, cycles, nullptr, stats, &cap);
}
