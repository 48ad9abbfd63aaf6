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

// ---- the warm start on a coarser grid ------------------------------------------------------
// The modes of an Ns grid are the modes of the N grid (same box) with |k_i| <= Ns/2 in units of the
// fundamental: Ns index xs <-> N index of the wavevector kint(xs, Ns).  The Ns grid's Nyquist modes
// (an index at Ns/2) are left out in both directions: their mirror on the N grid is a different
// mode, and their share of the correction is negligible.
__device__ __forceinline__ int mode_index(int k, int N) { return k < 0 ? k + N : k; }

// out (Ns modes) = in (N modes) at the shared wavevectors, zero at the Ns Nyquist modes
template <typename T>
__global__ void k_modes_down(int N, int Ns, const cplx<T> *__restrict__ in, cplx<T> *__restrict__ out) {
    const int Hs = Ns / 2 + 1, H = N / 2 + 1;
    const long n = (long)Ns * Ns * Hs;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int zs = (int)(i % Hs);
        const long xy = i / Hs;
        const int ys = (int)(xy % Ns), xs = (int)(xy / Ns);
        if (xs == Ns / 2 || ys == Ns / 2 || zs == Ns / 2) {
            out[i] = mk<T>(0, 0);
            continue;
        }
        const int x = mode_index(kint(xs, Ns), N), y = mode_index(kint(ys, Ns), N);
        out[i] = in[((long)x * N + y) * H + zs];
    }
}

// phi (N modes) += G(k) s(k) at the Ns modes but the Nyquist ones; G = -1/k^2, 1 at k = 0
// (kernel_inv_poisson, include/fft_kernels.h:96-99)
template <typename T>
__global__ void k_add_poisson_up(int N, int Ns, T dk, const cplx<T> *__restrict__ s, cplx<T> *__restrict__ phi) {
    const int Hs = Ns / 2 + 1, H = N / 2 + 1;
    const long n = (long)Ns * Ns * Hs;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int zs = (int)(i % Hs);
        const long xy = i / Hs;
        const int ys = (int)(xy % Ns), xs = (int)(xy / Ns);
        if (xs == Ns / 2 || ys == Ns / 2 || zs == Ns / 2) continue;
        const int kx = kint(xs, Ns), ky = kint(ys, Ns);
        const T k2 = ((T)kx * kx + (T)ky * ky + (T)zs * zs) * dk * dk;
        const T G = k2 > 0 ? -1 / k2 : (T)1;
        const long j = ((long)mode_index(kx, N) * N + mode_index(ky, N)) * H + zs;
        const cplx<T> v = s[i];
        phi[j] = mk<T>(phi[j].x + G * v.x, phi[j].y + G * v.y);
    }
}

template <typename T>
static int modes_down(int N, int Ns, const void *in, void *out) {
    const long n = (long)Ns * Ns * (Ns / 2 + 1);
    launch_begin("modes_down");
    k_modes_down<T><<<(unsigned)std::min<long>((n + 255) / 256, 152L * 16), 256, 0, stream()>>>(
        N, Ns, (const cplx<T> *)in, (cplx<T> *)out);
    count_launch();
    MITOS_LAUNCH_CHECK("coarse-grid modes");
    return 0;
}

template <typename T>
static int add_poisson_up(int N, int Ns, double boxlen, const void *s, void *phi) {
    const long n = (long)Ns * Ns * (Ns / 2 + 1);
    launch_begin("add_poisson_up");
    k_add_poisson_up<T><<<(unsigned)std::min<long>((n + 255) / 256, 152L * 16), 256, 0, stream()>>>(
        N, Ns, (T)(2 * M_PI / boxlen), (const cplx<T> *)s, (cplx<T> *)phi);
    count_launch();
    MITOS_LAUNCH_CHECK("coarse-grid correction");
    return 0;
}

int manet_warm_grid(const struct manet *net);

// the network correction on the Ns grid: inputs delta, phi_1 = G delta and phi_2 = G r2c(S) reduced
// to the Ns modes and back to real space there, inference, r2c, and phi(k) += G sigma(k) at those
// modes (FP32 grids)
static int warm_coarse(const GridGeom &g, int Ns, double L, struct manet *net, const void *dens_k, const void *S,
                       void *Sk, void *phi) {
    const int N = g.N, prec = MITOS_FP32;
    const GridGeom *gsp = geom(Ns, prec);
    if (!gsp) return 3;
    const GridGeom &gs = *gsp;
    const size_t sb = (size_t)gs.cells * csize(prec);
    void *ck = workspace(sb, 40);
    float *ds = (float *)workspace(sb, 41), *p1 = (float *)workspace(sb, 42), *p2 = (float *)workspace(sb, 43),
          *sg = (float *)workspace(sb, 44);
    if (!ck || !ds || !p1 || !p2 || !sg) return 5;
    KernelParams kp;
    memset(&kp, 0, sizeof kp);
    kp.id = KID_INV_POISSON;
    int e = modes_down<float>(N, Ns, dens_k, ck);
    if (!e) e = grid_c2r(gs, prec, L, ck, ds);
    if (!e) e = modes_down<float>(N, Ns, dens_k, ck);
    if (!e) e = apply_kernel_launch(Ns, L, prec, kp, ck, ck);
    if (!e) e = grid_c2r(gs, prec, L, ck, p1);
    if (!e) e = grid_r2c(g, prec, L, S, N + 2, 1.0, 0.0, Sk);
    if (!e) e = modes_down<float>(N, Ns, Sk, ck);
    if (!e) e = apply_kernel_launch(Ns, L, prec, kp, ck, ck);
    if (!e) e = grid_c2r(gs, prec, L, ck, p2);
    if (!e) e = manet_infer(net, Ns, Ns + 2, ds, p1, p2, sg);
    if (!e) e = grid_r2c(gs, prec, L, sg, Ns + 2, 1.0, 0.0, ck);
    if (!e) e = add_poisson_up<float>(N, Ns, L, ck, phi);
    return e;
}

// phi(k) += G(k) r2c(src)(k) for a source whose z r2c the Z pass already made (Sk: complex, the Y
// and X steps remain)
static int add_poisson_zk(const GridGeom &g, int prec, double boxlen, void *Sk, void *phi) {
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.dk = 2 * M_PI / boxlen;
    a.scale = 1.0;
    a.in[0] = Sk;
    a.out[0] = Sk;
    int e = prec == MITOS_FP32 ? launch_y<float>(g, YOP_PLAIN, -1, a) : launch_y<double>(g, YOP_PLAIN, -1, a);
    if (e) return e;
    a.in2 = phi;
    a.out[0] = phi;
    a.scale = boxlen * boxlen * boxlen / ((double)g.N * g.N * g.N);
    return prec == MITOS_FP32 ? launch_x<float>(g, XOP_ADD_POISSON, -1, a) : launch_x<double>(g, XOP_ADD_POISSON, -1, a);
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
    int e = grid_r2c_zy(g, prec, a);
    if (e) return e;
    a.in[0] = Sk;
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
        // the residual leaves the Z pass already transformed along z (into Sk)
        e = grid_hessian(g, prec, L, pot->fbox, want_S ? ZOP_HESS_MA_KS : ZOP_HESS_MA_K, dens->box, Sk, red, 0,
                         want_S ? S : nullptr);
        if (e) break;
        double h[2];
        MITOS_CUDA(cudaMemcpyAsync(h, red, sizeof h, cudaMemcpyDeviceToHost, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
        if ((e = zrow_fault_check())) break;
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
        e = add_poisson_zk(g, prec, L, Sk, pot->fbox);
        if (e) break;
        st->cycles++;
        const int Nw = warm && !cap ? manet_warm_grid(warm) : 0;
        if (it == 0 && Nw > 0 && Nw < N) {
            // the network on the coarser grid
            MITOS_CUDA(cudaEventRecord(ev[1], stream()));
            e = warm_coarse(g, Nw, L, warm, dens->fbox, S, Sk, pot->fbox);
            if (e) break;
            MITOS_CUDA(cudaEventRecord(ev[2], stream()));
            MITOS_CUDA(cudaEventSynchronize(ev[2]));
            float wms = 0;
            cudaEventElapsedTime(&wms, ev[1], ev[2]);
            st->ms_warm = wms;
        } else if (it == 0 && (warm || cap)) {
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
