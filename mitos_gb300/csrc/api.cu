// api.cu -- the reference entry points (include/mitos_gb300.h) over device grids.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "context.cuh"
#include "grids.cuh"
#include "kspace.cuh"
#include "particles.cuh"

using namespace mitos;

static int g_default_precision = MITOS_FP64;

static inline size_t grid_bytes(const struct distributed_grid *dg) {
    return (size_t)dg->local_size * csize(dg->precision);
}

// the end of a synchronous entry point; a caller's stream in asynchronous mode (mitos_set_stream)
// gets the work enqueued only
static int sync_all() {
    if (async_mode()) {
        const cudaError_t ce = cudaGetLastError();
        return ce == cudaSuccess ? 0 : check_cuda(ce, "an asynchronous entry point");
    }
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    return 0;
}

static bool is_device_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

namespace mitos {
// passes over whole grids, shared with pipeline.cu
int grid_c2r(const GridGeom &g, int prec, double boxlen, void *fbox, void *box) {
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.dk = 2 * M_PI / boxlen;
    a.scale = 1.0;
    a.in[0] = fbox;
    a.out[0] = fbox;
    int e = prec == MITOS_FP32 ? launch_x<float>(g, XOP_PLAIN, +1, a) : launch_x<double>(g, XOP_PLAIN, +1, a);
    if (e) return e;
    e = prec == MITOS_FP32 ? launch_y<float>(g, YOP_PLAIN, +1, a) : launch_y<double>(g, YOP_PLAIN, +1, a);
    if (e) return e;
    a.out[0] = box;
    a.scale = 1.0 / (boxlen * boxlen * boxlen);  // src/fft.c:110-125
    a.rp_out = g.N + 2;
    return prec == MITOS_FP32 ? launch_z_c2r<float>(g, ZOP_C2R, a) : launch_z_c2r<double>(g, ZOP_C2R, a);
}

// the Z and Y steps of an r2c from a.in[0] (real, pitch a.rp_in) into a.out[0]: one cluster pass
// where it applies (fft_cluster.cu), else the Z r2c pass and the in-place Y pass
int grid_r2c_zy(const GridGeom &g, int prec, const PassArgs &a) {
    int e = launch_zy_r2c(g, prec, a);
    if (e != -1) return e;
    e = prec == MITOS_FP32 ? launch_z_r2c<float>(g, a) : launch_z_r2c<double>(g, a);
    if (e) return e;
    PassArgs b = a;
    b.in[0] = a.out[0];
    return prec == MITOS_FP32 ? launch_y<float>(g, YOP_PLAIN, -1, b) : launch_y<double>(g, YOP_PLAIN, -1, b);
}

int grid_r2c(const GridGeom &g, int prec, double boxlen, const void *box, int rp, double rho_a,
             double rho_b, void *fbox) {
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.dk = 2 * M_PI / boxlen;
    a.scale = 1.0;
    a.in[0] = box;
    a.out[0] = fbox;
    a.rp_in = rp;
    a.rho_a = rho_a;
    a.rho_b = rho_b;
    int e = grid_r2c_zy(g, prec, a);
    if (e) return e;
    a.in[0] = fbox;
    a.scale = boxlen * boxlen * boxlen / ((double)g.N * g.N * g.N);  // src/fft.c:91-106
    return prec == MITOS_FP32 ? launch_x<float>(g, XOP_PLAIN, -1, a) : launch_x<double>(g, XOP_PLAIN, -1, a);
}

// six Hessian components of phi (k space) through the fused X / Y / Z passes into out (real);
// ZOP_HESS_2LPT writes the second-order source, ZOP_HESS_MA the Monge-Ampere residual
int grid_hessian(const GridGeom &g, int prec, double boxlen, const void *phi, int zop,
                 const void *rho, void *out, double *red, int window_order, void *out2, int batch,
                 size_t bstride, void *zero, size_t zero_bytes) {
    // batched (batch > 1): every grid holds batch realisations bstride bytes apart
    const size_t gb = batch > 1 ? (size_t)batch * bstride : (size_t)g.cells * csize(prec);
    void *A[3], *B[6];
    for (int i = 0; i < 3; i++) if (!(A[i] = workspace(gb, 1 + i))) return 5;
    for (int i = 0; i < 6; i++) if (!(B[i] = workspace(gb, 4 + i))) return 5;
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.batch = batch;
    a.bstride = batch > 1 ? (long long)bstride : 0;
    a.dk = 2 * M_PI / boxlen;
    a.scale = 1.0;
    a.window_order = window_order;
    a.in[0] = phi;
    for (int i = 0; i < 3; i++) a.out[i] = A[i];
    int e = prec == MITOS_FP32 ? launch_x<float>(g, XOP_HESS, +1, a) : launch_x<double>(g, XOP_HESS, +1, a);
    if (e) return e;
    a.window_order = 0;
    for (int i = 0; i < 6; i++) a.out[i] = B[i];
    // Y: one pass per X output, [xx, xy, xz, yy, yz, zz] = [A2, i ky A1, A1, -ky^2 A0, i ky A0, A0]
    // (single-input passes fit three 256-thread blocks an SM where one three-input pass needs 128
    // registers and runs two; the plain pass of A2 runs the wider 512-thread tiles)
    {
        auto ly = [&](YOp op) { return prec == MITOS_FP32 ? launch_y<float>(g, op, +1, a) : launch_y<double>(g, op, +1, a); };
        a.in[0] = A[0];
        a.out[0] = B[3];
        a.out[1] = B[4];
        a.out[2] = B[5];
        e = ly(YOP_HESS_A);
        a.in[0] = A[1];
        a.out[0] = B[1];
        a.out[1] = B[2];
        if (!e) e = ly(YOP_HESS_B);
        a.in[0] = A[2];
        a.out[0] = B[0];
        if (!e) e = ly(YOP_PLAIN);
    }
    if (e) return e;
    for (int i = 0; i < 6; i++) a.in[i] = B[i];
    a.out[0] = out;
    a.out[1] = out2;
    a.in2 = rho;
    a.red = red;
    a.rp_in = g.N + 2;
    a.rp_out = g.N + 2;
    a.scale = 1.0 / (boxlen * boxlen * boxlen);
    if (zop == ZOP_HESS_2LPT_K) {
        a.zero = zero;
        a.zero_bytes = zero_bytes;
    }
    return prec == MITOS_FP32 ? launch_z_c2r<float>(g, (ZOp)zop, a) : launch_z_c2r<double>(g, (ZOp)zop, a);
}

template <typename T>
__global__ void k_axpby(long n, T a, const T *x, T b, const T *y, T *out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = x[i] * a + b * y[i];
}

int axpby(int prec, long n, double a, const void *x, double b, const void *y, void *out) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    launch_begin("axpby");
    if (prec == MITOS_FP32)
        k_axpby<float><<<blocks, 256, 0, stream()>>>(n, (float)a, (const float *)x, (float)b, (const float *)y, (float *)out);
    else
        k_axpby<double><<<blocks, 256, 0, stream()>>>(n, a, (const double *)x, b, (const double *)y, (double *)out);
    count_launch();
    MITOS_LAUNCH_CHECK("axpby");
    return 0;
}

// cross power of two complex grids into log or linear bins (device accumulators)
template <typename T>
__global__ void k_bin_cross(int N, int x0, int nx, double dk, const cplx<T> *f1, const cplx<T> *f2,
                            const int *bin_of_n2, int nbins, double *bk, double *bp, unsigned long long *bn) {
    extern __shared__ double shb[];
    double *sk = shb, *sp = shb + nbins;
    unsigned long long *sn = (unsigned long long *)(shb + 2 * nbins);
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) { sk[i] = 0; sp[i] = 0; sn[i] = 0; }
    __syncthreads();
    const int H = N / 2 + 1;
    const long total = (long)nx * N * H;  // the rows x0 .. x0 + nx - 1 (a slab, or the whole grid)
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int y = (int)(xy % N), x = x0 + (int)(xy / N);
        const int jx = kint(x, N), jy = kint(y, N);
        const long n2 = (long)jx * jx + (long)jy * jy + (long)z * z;
        const int b = bin_of_n2[n2];
        if (b < 0) continue;
        const cplx<T> a = f1[id], c = f2[id];
        const double pw = (double)a.x * (double)c.x + (double)a.y * (double)c.y;
        const int mult = (z == 0 || z == N / 2) ? 1 : 2;
        const double kx = __dmul_rn((double)jx, dk), ky = __dmul_rn((double)jy, dk), kz = __dmul_rn((double)z, dk);
        const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
        atomicAdd(sk + b, mult * k);
        atomicAdd(sp + b, mult * pw);
        atomicAdd(sn + b, (unsigned long long)mult);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
        if (sn[i]) {
            atomicAdd(bk + i, sk[i]);
            atomicAdd(bp + i, sp[i]);
            atomicAdd(bn + i, sn[i]);
        }
    }
}

int bin_cross(int N, int x0, int nx, double boxlen, int prec, const void *f1, const void *f2, int bins, int linear,
              double *k_out, double *p_out, long long *n_out) {
    const int *tab = bin_table(N, bins, linear, boxlen);
    if (!tab) return 5;
    double *acc = (double *)workspace(sizeof(double) * 3 * (size_t)bins, 101);
    if (!acc) return 5;
    MITOS_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * bins, stream()));
    const size_t smem = sizeof(double) * 3 * bins;
    const long total = (long)nx * N * (N / 2 + 1);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    const double dk = 2 * M_PI / boxlen;
    launch_begin("bin_cross");
    if (prec == MITOS_FP32)
        k_bin_cross<float><<<blocks, 256, smem, stream()>>>(N, x0, nx, dk, (const float2 *)f1, (const float2 *)f2, tab,
                                                            bins, acc, acc + bins, (unsigned long long *)(acc + 2 * bins));
    else
        k_bin_cross<double><<<blocks, 256, smem, stream()>>>(N, x0, nx, dk, (const double2 *)f1, (const double2 *)f2, tab,
                                                             bins, acc, acc + bins, (unsigned long long *)(acc + 2 * bins));
    count_launch();
    MITOS_LAUNCH_CHECK("power spectrum binning");
    std::vector<double> h(3 * bins);
    MITOS_CUDA(cudaMemcpyAsync(h.data(), acc, sizeof(double) * 3 * bins, cudaMemcpyDeviceToHost, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    for (int i = 0; i < bins; i++) {
        k_out[i] = h[i];
        p_out[i] = h[bins + i];
        memcpy(&n_out[i], &h[2 * bins + i], sizeof(long long));
    }
    return 0;
}
}  // namespace mitos

// ==== grids ==============================================================================
extern "C" int mitos_set_precision(int precision) {
    if (precision != MITOS_FP32 && precision != MITOS_FP64) {
        set_error(3, "unknown precision %d", precision);
        return 3;
    }
    g_default_precision = precision;
    return 0;
}
extern "C" int mitos_get_precision(void) { return g_default_precision; }

extern "C" int alloc_local_grid_prec(struct distributed_grid *dg, int N, double boxlen, MPI_Comm comm,
                                     int precision) {
    if (!dg) return 1;
    if (!geom(N, precision)) return 3;
    // fftw_mpi_local_size_3d on one rank: NX = N, X0 = 0 (src/distributed_grid.c:23-42)
    dg->N = N;
    dg->boxlen = boxlen;
    dg->comm = comm;
    dg->momentum_space = 0;
    dg->NX = N;
    dg->X0 = 0;
    dg->local_size = (long)N * N * (N / 2 + 1);
    dg->precision = precision;
    dg->flags = 0;
    dg->priv = nullptr;
    dg->fbox = nullptr;
    dg->box = nullptr;
    const size_t b = grid_bytes(dg);
    void *f = nullptr, *r = nullptr;
    if (cudaMalloc(&f, b) != cudaSuccess || cudaMalloc(&r, b) != cudaSuccess) {
        cudaGetLastError();
        if (f) cudaFree(f);
        set_error(5, "out of device memory allocating a grid of N = %d", N);
        return 5;
    }
    cudaMemsetAsync(f, 0, b, stream());
    cudaMemsetAsync(r, 0, b, stream());
    dg->fbox = (mitos_c128 *)f;
    dg->box = (double *)r;
    MITOS_CUDA(cudaStreamSynchronize(stream()));  // the grid is ready for any stream
    return 0;
}

extern "C" int alloc_local_grid(struct distributed_grid *dg, int N, double boxlen, MPI_Comm comm) {
    return alloc_local_grid_prec(dg, N, boxlen, comm, g_default_precision);
}

extern "C" int free_local_real_grid(struct distributed_grid *dg) {
    if (dg && dg->box) { cudaFree(dg->box); dg->box = nullptr; }
    return 0;
}
extern "C" int free_local_complex_grid(struct distributed_grid *dg) {
    if (dg && dg->fbox) { cudaFree(dg->fbox); dg->fbox = nullptr; }
    return 0;
}
extern "C" int free_local_grid(struct distributed_grid *dg) {
    free_local_real_grid(dg);
    free_local_complex_grid(dg);
    return 0;
}

extern "C" int dg_copy_to_host(const struct distributed_grid *dg, int which, void *host) {
    const void *src = which == 0 ? (const void *)dg->fbox : (const void *)dg->box;
    if (!src) { set_error(1, "grid part not allocated"); return 1; }
    MITOS_CUDA(cudaMemcpyAsync(host, src, grid_bytes(dg), cudaMemcpyDeviceToHost, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));  // host memory: synchronous in either mode
    return 0;
}
// writeHeaderAttributes (src/header.c:26-175): the values of its attributes, without the HDF5 calls
extern "C" int snapshot_header_attributes(double boxlen, double z_ini, int num_types, const char *const *export_names,
                                          const long long *total_numbers, double unit_mass_kg, double unit_length_m,
                                          double unit_time_s, double unit_temperature_K, double unit_current_A,
                                          struct snapshot_header *out) {
    if (!out || num_types < 0 || (num_types > 0 && (!export_names || !total_numbers))) {
        mitos::set_error(1, "snapshot_header_attributes: invalid arguments");
        return 1;
    }
    memset(out, 0, sizeof *out);
    for (int c = 0; c < 3; c++) out->BoxSize[c] = boxlen;  // :38-40
    out->Dimension = 3;
    out->Redshift = z_ini;
    out->Flag_Entropy_ICs = 0;
    out->NumFilesPerSnapshot = 1;
    // :79-92: types whose export name is PartType<i> add their total number to entry i; the high
    // words and the mass table are written as zeros
    for (int i = 0; i < 7; i++) {
        char want[40];
        snprintf(want, sizeof want, "PartType%d", i);
        for (int t = 0; t < num_types; t++)
            if (export_names[t] && strcmp(export_names[t], want) == 0) out->NumPart_Total[i] += (long)total_numbers[t];
    }
    out->Cosmology_Redshift = z_ini;  // :119-121
    // :136-141: SI to cgs
    out->Unit_mass_cgs = unit_mass_kg * 1000;
    out->Unit_length_cgs = unit_length_m * 100;
    out->Unit_time_cgs = unit_time_s;
    out->Unit_temperature_cgs = unit_temperature_K;
    out->Unit_current_cgs = unit_current_A;
    return 0;
}

extern "C" int dg_field_to_host(const struct distributed_grid *dg, double *host) {
    if (!dg || !dg->box || !host) { set_error(1, "grid part not allocated"); return 1; }
    if (dg->momentum_space == 1) { set_error(2, "attempting to export while in momentum space"); return 2; }
    const long n = (long)dg->N * dg->N * (dg->N + 2);
    if (dg->precision == MITOS_FP64) {
        MITOS_CUDA(cudaMemcpyAsync(host, dg->box, sizeof(double) * n, cudaMemcpyDeviceToHost, stream()));
    } else {
        double *t = (double *)workspace(sizeof(double) * n, 23);
        if (!t) return 5;
        int e = widen_to_double(n, (const float *)dg->box, t);
        if (e) return e;
        MITOS_CUDA(cudaMemcpyAsync(host, t, sizeof(double) * n, cudaMemcpyDeviceToHost, stream()));
    }
    MITOS_CUDA(cudaStreamSynchronize(stream()));  // host memory: synchronous in either mode
    return 0;
}
extern "C" int dg_copy_from_host(struct distributed_grid *dg, int which, const void *host) {
    void *dst = which == 0 ? (void *)dg->fbox : (void *)dg->box;
    if (!dst) { set_error(1, "grid part not allocated"); return 1; }
    MITOS_CUDA(cudaMemcpyAsync(dst, host, grid_bytes(dg), cudaMemcpyHostToDevice, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));  // host memory: synchronous in either mode
    return 0;
}

// ==== FFT ===================================================================================
extern "C" void fft_wavevector(int x, int y, int z, int N, double delta_k, double *kx, double *ky,
                               double *kz, double *k) {
    *kx = (x > N / 2) ? (x - N) * delta_k : x * delta_k;
    *ky = (y > N / 2) ? (y - N) * delta_k : y * delta_k;
    *kz = (z > N / 2) ? (z - N) * delta_k : z * delta_k;
    *k = sqrt((*kx) * (*kx) + (*ky) * (*ky) + (*kz) * (*kz));
}

extern "C" int fft_c2r_dg(struct distributed_grid *dg) {
    const GridGeom *g = geom(dg->N, dg->precision);
    if (!g) return 3;
    int e = grid_c2r(*g, dg->precision, dg->boxlen, dg->fbox, dg->box);
    if (e) return e;
    dg->momentum_space = 0;
    return sync_all();
}

extern "C" int mitos_set_cluster_fft(int mode) {
    const int was = cluster_fft();
    set_cluster_fft(mode >= 0 && mode <= 3 ? mode : 0);
    return was;
}

extern "C" int mitos_set_stream(void *s, int async) {
    set_stream((cudaStream_t)s);
    set_async(s != nullptr && async != 0);
    return 0;
}

extern "C" int mitos_set_lattice_tma(int on) {
    const int was = lattice_tma() ? 1 : 0;
    set_lattice_tma(on != 0);
    return was;
}

extern "C" int mitos_set_lattice_order(int regions) {
    const int was = lattice_region() ? 1 : 0;
    set_lattice_region(regions != 0);
    return was;
}

extern "C" int fft_r2c_dg(struct distributed_grid *dg) {
    const GridGeom *g = geom(dg->N, dg->precision);
    if (!g) return 3;
    int e = grid_r2c(*g, dg->precision, dg->boxlen, dg->box, dg->N + 2, 1.0, 0.0, dg->fbox);
    if (e) return e;
    dg->momentum_space = 1;
    return sync_all();
}

static int kernel_id_of(void (*f)(struct kernel *)) {
    if (f == kernel_constant) return KID_CONSTANT;
    if (f == kernel_lowpass) return KID_LOWPASS;
    if (f == kernel_hipass) return KID_HIPASS;
    if (f == kernel_tophat) return KID_TOPHAT;
    if (f == kernel_elliptic_tophat) return KID_ELLIPTIC_TOPHAT;
    if (f == kernel_translate) return KID_TRANSLATE;
    if (f == kernel_gaussian) return KID_GAUSSIAN;
    if (f == kernel_gaussian_inv) return KID_GAUSSIAN_INV;
    if (f == kernel_inv_poisson) return KID_INV_POISSON;
    if (f == kernel_dx) return KID_DX;
    if (f == kernel_dy) return KID_DY;
    if (f == kernel_dz) return KID_DZ;
    if (f == kernel_power_no_transfer) return KID_POWER_NO_TRANSFER;
    if (f == kernel_transfer_function) return KID_TRANSFER;
    if (f == kernel_inv_transfer_function) return KID_INV_TRANSFER;
    if (f == kernel_undo_Hermite_window) return KID_UNDO_HERMITE;
    return -1;
}

// src/fft.c:257-302
extern "C" int fft_apply_kernel_dg(struct distributed_grid *w, const struct distributed_grid *r,
                                   void (*compute)(struct kernel *), const void *params) {
    if (r->NX != w->NX || r->N != w->N || r->precision != w->precision) {
        set_error(1, "non-matching grid dimensions between read/write");
        return 1;
    }
    if (r->momentum_space != 1) {
        set_error(2, "input field is not in momentum space");
        return 2;
    }
    KernelParams kp;
    memset(&kp, 0, sizeof kp);
    kp.id = kernel_id_of(compute);
    if (kp.id < 0) {
        set_error(3, "unsupported kernel callback %p (no CPU path)", (void *)compute);
        return 3;
    }
    const double *pd = (const double *)params;
    void *tab = nullptr;
    switch (kp.id) {
    case KID_CONSTANT: case KID_LOWPASS: case KID_HIPASS: case KID_GAUSSIAN: case KID_GAUSSIAN_INV:
        kp.c[0] = pd[0];
        break;
    case KID_TOPHAT: kp.c[0] = pd[0]; kp.c[1] = pd[1]; break;
    case KID_TRANSLATE: for (int i = 0; i < 3; i++) kp.c[i] = pd[i]; break;
    case KID_ELLIPTIC_TOPHAT: for (int i = 0; i < 4; i++) kp.c[i] = pd[i]; break;
    case KID_POWER_NO_TRANSFER: {
        const struct cosmology *c = (const struct cosmology *)params;
        kp.c[0] = c->A_s;
        kp.c[1] = c->n_s;
        kp.c[2] = c->k_pivot;
        break;
    }
    case KID_TRANSFER: case KID_INV_TRANSFER: {
        const struct spline_params *sp = (const struct spline_params *)params;
        const struct perturb_data *ptd = sp->spline->ptdat;
        const int ks = ptd->k_size;
        const double *arr = ptd->delta + (long)sp->index_src * ks * ptd->tau_size;
        tab = workspace(sizeof(double) * 3 * ks, 102);
        if (!tab) return 5;
        std::vector<double> h(3 * ks);
        memcpy(h.data(), ptd->k, sizeof(double) * ks);
        memcpy(h.data() + ks, arr + (long)ks * sp->tau_index, sizeof(double) * ks);
        memcpy(h.data() + 2 * ks, arr + (long)ks * (sp->tau_index + 1), sizeof(double) * ks);
        MITOS_CUDA(cudaMemcpyAsync(tab, h.data(), sizeof(double) * 3 * ks, cudaMemcpyHostToDevice, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
        kp.tk = (const double *)tab;
        kp.tlo = kp.tk + ks;
        kp.thi = kp.tk + 2 * ks;
        kp.k_size = ks;
        kp.c[0] = sp->u_tau;
        break;
    }
    case KID_UNDO_HERMITE: {
        const struct Hermite_kern_params *hp = (const struct Hermite_kern_params *)params;
        kp.order = hp->order;
        kp.c[0] = hp->boxlen;
        kp.c[1] = (double)hp->N;
        break;
    }
    default: break;
    }
    int e = apply_kernel_launch(r->N, r->boxlen, r->precision, kp, r->fbox, w->fbox);
    if (e) return e;
    w->momentum_space = 1;
    return sync_all();
}

// ==== white noise ============================================================================
extern "C" int generate_complex_grf(struct distributed_grid *dg, rng_state *state) {
    const GridGeom *g = geom(dg->N, dg->precision);
    if (!g) return 3;
    int e = noise_generate(*g, dg->precision, dg->boxlen, state->s, nullptr, dg->fbox);
    if (e) return e;
    e = sync_all();
    if (e) return e;
    // the sequential reference leaves the state after its last draw
    rng_jump(state->s, 4ULL * ((unsigned long long)g->cells - 1));
    dg->momentum_space = 1;  // src/grf.c:66
    return 0;
}

extern "C" int enforce_hermiticity(struct distributed_grid *dg) {
    const GridGeom *g = geom(dg->N, dg->precision);
    if (!g) return 3;
    int e = hermitian_planes(*g, dg->precision, dg->fbox);
    if (e) return e;
    return sync_all();
}

// ==== perturbation grid, Poisson, 2LPT, Monge-Ampere ==========================================
static int find_title(const struct perturb_data *pd, const char *title) {
    if (!pd->titles || !title) return -1;
    for (int i = 0; i < pd->n_functions; i++)
        if (pd->titles[i] && strcmp(pd->titles[i], title) == 0) return i;
    return -1;
}

extern "C" int generatePerturbationGrid(const struct cosmology *cosmo, const struct perturb_spline *spline,
                                        struct distributed_grid *grf, struct distributed_grid *grid,
                                        const char *title, const char *fname, const double rescale_factor) {
    (void)fname;
    int tau_index;
    double u_tau;
    find_tau_h(spline->ptdat, cosmo->log_tau_source, &tau_index, &u_tau);
    const int index_src = find_title(spline->ptdat, title);
    if (index_src < 0) {
        set_error(1, "transfer function '%s' not found", title ? title : "(null)");
        return 1;
    }
    struct spline_params sp = {spline, index_src, tau_index, u_tau};
    int e = fft_apply_kernel_dg(grid, grf, kernel_transfer_function, &sp);
    if (e) return e;
    if (rescale_factor != 1.0) {
        e = fft_apply_kernel_dg(grid, grid, kernel_constant, &rescale_factor);
        if (e) return e;
    }
    return fft_c2r_dg(grid);
}

extern "C" int solvePoisson_dg(struct distributed_grid *dg) {
    int e = fft_r2c_dg(dg);
    if (!e) e = fft_apply_kernel_dg(dg, dg, kernel_inv_poisson, nullptr);
    if (!e) e = fft_c2r_dg(dg);
    return e;
}

static int check_triplet(struct distributed_grid *p, struct distributed_grid *d, struct distributed_grid *w) {
    if (p->N != d->N || d->N != w->N || p->precision != d->precision || d->precision != w->precision) {
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

// src/2lpt.c:38-143 with the six Hessian grids and the source fused into three passes
extern "C" int solve2LPT(struct distributed_grid *pot, struct distributed_grid *dens,
                         struct distributed_grid *work, double f1, double f2) {
    int e = check_triplet(pot, dens, work);
    if (e) return e;
    const GridGeom *g = geom(dens->N, dens->precision);
    if (!g) return 3;
    e = fft_apply_kernel_dg(pot, dens, kernel_inv_poisson, nullptr);
    if (!e) e = fft_r2c_dg(dens);
    if (!e) e = grid_hessian(*g, dens->precision, dens->boxlen, pot->fbox, ZOP_HESS_2LPT, nullptr, work->box, nullptr, 0);
    if (e) return e;
    work->momentum_space = 0;
    e = solvePoisson_dg(work);
    if (!e) e = fft_c2r_dg(pot);
    if (!e) e = axpby(pot->precision, (long)2 * pot->local_size, f1, pot->box, f2, work->box, pot->box);
    if (!e) e = fft_r2c_dg(pot);
    return e;
}

static std::vector<double> g_ma_eps, g_ma_rel;

// src/monge_ampere.c:50-183
extern "C" int solveMongeAmpere(struct distributed_grid *pot, struct distributed_grid *dens,
                                struct distributed_grid *work, int cycles) {
    int e = check_triplet(pot, dens, work);
    if (e) return e;
    const GridGeom *g = geom(dens->N, dens->precision);
    if (!g) return 3;
    const int N = dens->N;
    e = fft_apply_kernel_dg(pot, dens, kernel_inv_poisson, nullptr);
    if (!e) e = fft_r2c_dg(dens);
    if (e) return e;
    double *red = (double *)workspace(2 * sizeof(double), 103);
    if (!red) return 5;
    g_ma_eps.clear();
    g_ma_rel.clear();
    for (int it = 0; it < cycles; it++) {
        MITOS_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(double), stream()));
        e = grid_hessian(*g, dens->precision, dens->boxlen, pot->fbox, ZOP_HESS_MA, dens->box, work->box, red, 0);
        if (e) return e;
        work->momentum_space = 0;
        e = solvePoisson_dg(work);
        if (!e) e = fft_c2r_dg(pot);
        if (!e) e = axpby(pot->precision, (long)2 * pot->local_size, 1.0, pot->box, 1.0, work->box, pot->box);
        if (!e) e = fft_r2c_dg(pot);
        if (e) return e;
        double h[2];
        MITOS_CUDA(cudaMemcpy(h, red, sizeof h, cudaMemcpyDeviceToHost));
        g_ma_eps.push_back(sqrt((h[0] / h[1]) / ((double)N * N * N)));  // src/monge_ampere.c:177
        g_ma_rel.push_back(sqrt(h[0] / h[1]));
        if (getenv("MITOS_VERBOSE")) printf("%03d] Finished MA cycle: eps = %e\n", it, g_ma_eps.back());
    }
    return 0;
}

// per-cycle residual history of the last solveMongeAmpere call (reference eps and the
// relative rms residual); returns the number of cycles
extern "C" int mitos_ma_history(double *eps, double *rel, int max) {
    int n = (int)g_ma_eps.size();
    for (int i = 0; i < n && i < max; i++) {
        if (eps) eps[i] = g_ma_eps[i];
        if (rel) rel[i] = g_ma_rel[i];
    }
    return n;
}

// ==== power spectra ==========================================================================
static void finish_bins(int bins, double boxlen, double *k, double *p, const long long *n) {
    const double boxvol = boxlen * boxlen * boxlen;
    for (int i = 0; i < bins; i++) {
        k[i] /= (double)n[i];
        p[i] /= (double)n[i];
        p[i] /= boxvol;
    }
}

// the reference's three cross spectra: box1 / box2 hold the rows x0 .. x0 + nx - 1 of the
// half-complex grid (host or device); bins over those rows' modes (on one rank the reduction of
// calc_cross_powerspec_float_mpi, src/calc_powerspec.c:203-205, is the identity)
static int cross_common(int N, int x0, int nx, double boxlen, int prec, const void *b1, const void *b2, int bins,
                        double *k, double *p, long long *n) {
    if (N < 2 || (N & 1) || bins < 1 || x0 < 0 || nx < 1 || x0 + nx > N || !b1 || !b2 || !(boxlen > 0)) {
        set_error(1, "power spectrum: invalid grid, slab or bins");
        return 1;
    }
    const size_t bytes = (size_t)nx * N * (N / 2 + 1) * csize(prec);
    const void *d1 = b1, *d2 = b2;
    if (!is_device_ptr(b1)) {
        void *t = workspace(bytes, 20);
        if (!t) return 5;
        MITOS_CUDA(cudaMemcpyAsync(t, b1, bytes, cudaMemcpyHostToDevice, stream()));
        d1 = t;
    }
    if (b2 == b1) {
        d2 = d1;
    } else if (!is_device_ptr(b2)) {
        void *t = workspace(bytes, 21);
        if (!t) return 5;
        MITOS_CUDA(cudaMemcpyAsync(t, b2, bytes, cudaMemcpyHostToDevice, stream()));
        d2 = t;
    }
    int e = bin_cross(N, x0, nx, boxlen, prec, d1, d2, bins, 0, k, p, n);
    if (e) return e;
    finish_bins(bins, boxlen, k, p, n);
    return 0;
}

extern "C" void calc_cross_powerspec(int N, double boxlen, const mitos_c128 *box1, const mitos_c128 *box2,
                                     int bins, double *k_in_bins, double *power_in_bins, int *obs_in_bins) {
    std::vector<long long> n(bins);
    if (cross_common(N, 0, N, boxlen, MITOS_FP64, box1, box2, bins, k_in_bins, power_in_bins, n.data())) return;
    for (int i = 0; i < bins; i++) obs_in_bins[i] = (int)n[i];
}

extern "C" void calc_cross_powerspec_float(int N, double boxlen, const mitos_c64 *box1, const mitos_c64 *box2,
                                           int bins, double *k_in_bins, double *power_in_bins, int *obs_in_bins) {
    std::vector<long long> n(bins);
    if (cross_common(N, 0, N, boxlen, MITOS_FP32, box1, box2, bins, k_in_bins, power_in_bins, n.data())) return;
    for (int i = 0; i < bins; i++) obs_in_bins[i] = (int)n[i];
}

extern "C" void calc_cross_powerspec_float_mpi(long int N, long int X0, long int NX, double boxlen,
                                               const mitos_c64 *box1, const mitos_c64 *box2, int bins,
                                               double *k_in_bins, double *power_in_bins, long int *obs_in_bins) {
    std::vector<long long> n(bins);
    if (cross_common((int)N, (int)X0, (int)NX, boxlen, MITOS_FP32, box1, box2, bins, k_in_bins, power_in_bins,
                     n.data()))
        return;
    for (int i = 0; i < bins; i++) obs_in_bins[i] = (long)n[i];
}

// ==== bispectrum (src/calc_powerspec.c:295-508) ===============================================
extern "C" void calc_bispectrum(int N, double boxlen, const mitos_c128 *fbox, int bins, int bins3, double *k1_in_bins,
                                double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode, int type,
                                double theta, double k3) {
    const void *d = nullptr;
    if (!volume_mode && fbox) {
        d = fbox;
        if (!is_device_ptr(fbox)) {
            const size_t bytes = (size_t)N * N * (N / 2 + 1) * csize(MITOS_FP64);
            void *t = workspace(bytes, 20);
            if (!t) return;
            if (cudaMemcpyAsync(t, fbox, bytes, cudaMemcpyHostToDevice, stream()) != cudaSuccess) {
                check_cuda(cudaGetLastError(), "bispectrum input");
                return;
            }
            d = t;
        }
    }
    bispectrum_run(N, boxlen, MITOS_FP64, d, bins, bins3, k1_in_bins, k2_in_bins, k3_in_bins, bispectrum, volume_mode,
                   type, theta, k3);
}

extern "C" int calc_bispectrum_dg(const struct distributed_grid *dg, int bins, int bins3, double *k1_in_bins,
                                  double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode,
                                  int type, double theta, double k3) {
    if (!dg || !dg->fbox) {
        set_error(1, "grid not allocated");
        return 1;
    }
    if (!volume_mode && !dg->momentum_space) {
        set_error(2, "grid not in momentum space");
        return 2;
    }
    return bispectrum_run(dg->N, dg->boxlen, dg->precision, volume_mode ? nullptr : dg->fbox, bins, bins3, k1_in_bins,
                          k2_in_bins, k3_in_bins, bispectrum, volume_mode, type, theta, k3);
}

// ==== CIC ====================================================================================
extern "C" int cic_deposit_dg(struct distributed_grid *rho, const float *pos, long n, double mass,
                              double *total_mass) {
    if (!rho || !rho->box) { set_error(1, "grid not allocated"); return 1; }
    const float *dpos = pos;
    if (!is_device_ptr(pos)) {
        float *t = (float *)workspace(sizeof(float) * 3 * (size_t)n, 22);
        if (!t) return 5;
        MITOS_CUDA(cudaMemcpyAsync(t, pos, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, stream()));
        dpos = t;
    }
    const double cell = rho->boxlen * rho->boxlen * rho->boxlen / ((double)rho->N * rho->N * rho->N);
    int e = cic_positions(n, rho->N, rho->boxlen, rho->precision, dpos, (double)(float)mass / cell, rho->box);
    if (e) return e;
    if (total_mass) *total_mass = (double)n * (double)(float)mass;
    rho->momentum_space = 0;
    return sync_all();
}
