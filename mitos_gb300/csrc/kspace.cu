// kspace.cu -- fft_apply_kernel_dg on the device, the kernel callbacks of include/fft_kernels.h
// as host functions (identity tokens for the dispatcher) and the filter tables of the fused
// pipeline.
#include <math.h>
#include <string.h>

#include <vector>

#include "context.cuh"
#include "kspace.cuh"

namespace mitos {

// ---- host evaluation, the reference arithmetic (include/fft_kernels.h, src/primordial.c) --
static inline double sinc_h(double x) { return x == 0 ? 1. : sin(x) / x; }

double primordial_power_h(double k, double A_s, double n_s, double k_pivot) {
    if (k == 0) return 0;
    return A_s * pow(k / k_pivot, n_s - 1.) * k * (2. * M_PI * M_PI);
}

// perturbSplineFindTau (src/perturb_spline.c:73-106)
void find_tau_h(const struct perturb_data *pd, double log_tau, int *index, double *u) {
    int tau_size = pd->tau_size;
    if (log_tau < pd->log_tau[0]) { *index = 0; *u = 0.f; return; }
    if (log_tau >= pd->log_tau[tau_size - 1]) { *index = tau_size - 2; *u = 1.f; return; }
    for (int i = 1; i < tau_size; i++)
        if (pd->log_tau[i] >= log_tau) { *index = i - 1; break; }
    double left = pd->log_tau[*index], right = pd->log_tau[*index + 1];
    *u = (log_tau - left) / (right - left);
}

// perturbLogTauAtRedshift (src/perturb_spline.c:240-267)
double log_tau_at_z_h(const struct perturb_data *pd, double redshift) {
    int tau_size = pd->tau_size;
    if (redshift > pd->redshift[0]) return pd->log_tau[0];
    if (redshift <= pd->redshift[tau_size - 1]) return pd->log_tau[tau_size - 1];
    int index;
    for (index = tau_size - 1; index > 0; index--)
        if (pd->redshift[index] >= redshift) break;
    double left = pd->redshift[index], right = pd->redshift[index + 1];
    double u = (redshift - left) / (right - left);
    return (1 - u) * pd->log_tau[index] + u * pd->log_tau[index + 1];
}


// ---- device kernel application ----------------------------------------------------------
__device__ __forceinline__ double dsinc(double x) { return x == 0 ? 1. : sin(x) / x; }
__device__ __forceinline__ float fsinc(float x) { return x == 0 ? 1.f : sinf(x) / x; }

template <typename T>
__global__ void k_apply(int N, double dk, KernelParams kp, const cplx<T> *__restrict__ in,
                        cplx<T> *__restrict__ out) {
    const int H = N / 2 + 1;
    const long total = (long)N * N * H;
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total;
         id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int y = (int)(xy % N), x = (int)(xy / N);
        // fft_wavevector (src/fft.c:29-35) without contractions
        const double kx = __dmul_rn((double)kint(x, N), dk);
        const double ky = __dmul_rn((double)kint(y, N), dk);
        const double kz = __dmul_rn((double)kint(z, N), dk);
        const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
        double kr = 0, ki = 0;
        switch (kp.id) {
        case KID_CONSTANT: kr = kp.c[0]; break;
        case KID_LOWPASS: kr = (k < kp.c[0]) ? 1.0 : 0.0; break;
        case KID_HIPASS: kr = (k > kp.c[0]) ? 1.0 : 0.0; break;
        case KID_TOPHAT: kr = (k >= kp.c[0] && k <= kp.c[1]) ? 1.0 : 0.0; break;
        case KID_ELLIPTIC_TOPHAT: {
            double krr = kx * kp.c[0] + ky * kp.c[1] + kz * kp.c[2];
            double kk = kx * kx + ky * ky + kz * kz;
            double rr = kp.c[0] * kp.c[0] + kp.c[1] * kp.c[1] + kp.c[2] * kp.c[2];
            double theta = kk * rr + (kp.c[3] - 1) * krr * krr;
            kr = (theta <= 4 * M_PI * M_PI) ? 1.0 : 0.0;
            break;
        }
        case KID_TRANSLATE: {
            double ph = kp.c[0] * kx + kp.c[1] * ky + kp.c[2] * kz;
            sincos(ph, &ki, &kr);
            break;
        }
        case KID_GAUSSIAN: { double kR = k * kp.c[0]; kr = exp(-kR * kR); break; }
        case KID_GAUSSIAN_INV: { double kR = k * kp.c[0]; kr = exp(kR * kR); break; }
        case KID_INV_POISSON: kr = (k > 0) ? __ddiv_rn(__ddiv_rn(-1.0, k), k) : 1.0; break;
        case KID_DX: ki = kx; break;
        case KID_DY: ki = ky; break;
        case KID_DZ: ki = kz; break;
        case KID_POWER_NO_TRANSFER:
            kr = (k == 0) ? 0.0
                          : sqrt(__dmul_rn(__dmul_rn(__dmul_rn(kp.c[0], pow(__ddiv_rn(k, kp.c[2]), __dsub_rn(kp.c[1], 1.))), k),
                                           2. * M_PI * M_PI));
            break;
        case KID_TRANSFER:
        case KID_INV_TRANSFER:
            if (k == 0) {
                kr = 0.0;
            } else {
                double T = transfer_at<double>(kp.tk, kp.tlo, kp.thi, kp.k_size, k, kp.c[0]);
                kr = (kp.id == KID_TRANSFER) ? T : 1.0 / T;
            }
            break;
        case KID_UNDO_HERMITE:
            if (k == 0) {
                kr = 1.0;
            } else {
                const double s = kp.c[0] / kp.c[1];  // boxlen / N
                double Wx = dsinc(0.5 * kx * kp.c[0] / kp.c[1]);
                double Wy = dsinc(0.5 * ky * kp.c[0] / kp.c[1]);
                double Wz = dsinc(0.5 * kz * kp.c[0] / kp.c[1]);
                (void)s;
                kr = 1.0 / pow(Wx * Wy * Wz, (double)kp.order);
            }
            break;
        default: break;
        }
        const cplx<T> a = in[id];
        const double ar = (double)a.x, ai = (double)a.y;
        // complex product as the reference's double complex multiply, no contractions
        const double re = __dsub_rn(__dmul_rn(ar, kr), __dmul_rn(ai, ki));
        const double im = __dadd_rn(__dmul_rn(ar, ki), __dmul_rn(ai, kr));
        out[id] = mk<T>((T)re, (T)im);
    }
}

// FP32 grids.  A kernel that depends on k alone is evaluated once per integer |n|^2 (FP64, at
// k = sqrt(n^2) dk, the reference formulas above) and applied as an FP32 factor; the TSC window undo
// is separable (one FP64 table of W(k_i)^-order per axis index).  Per mode the FP64 evaluation ran
// on GB300's FP64 pipe, a small fraction of its FP32 rate (1.17 ms at 256^3 for the transfer
// function, against the 0.02 ms the grid's bytes take); the factor differs from the per-mode FP64
// value by an ulp of k or so, far inside the FP32 result's rounding.
static bool isotropic(int id) {
    switch (id) {
    case KID_CONSTANT: case KID_LOWPASS: case KID_HIPASS: case KID_TOPHAT: case KID_GAUSSIAN:
    case KID_GAUSSIAN_INV: case KID_INV_POISSON: case KID_POWER_NO_TRANSFER: case KID_TRANSFER:
    case KID_INV_TRANSFER:
        return true;
    default:
        return false;
    }
}

// tab[n2] = the kernel's real factor at k = sqrt(n2) dk, n2 <= n2max (isotropic kernels: no
// imaginary part); through k_apply's own switch on one complex one
__global__ void k_iso_table(long n2max, double dk, KernelParams kp, float *__restrict__ tab) {
    for (long n2 = (long)blockIdx.x * blockDim.x + threadIdx.x; n2 <= n2max; n2 += (long)gridDim.x * blockDim.x) {
        const double k = sqrt((double)n2) * dk;
        double kr = 0;
        switch (kp.id) {
        case KID_CONSTANT: kr = kp.c[0]; break;
        case KID_LOWPASS: kr = (k < kp.c[0]) ? 1.0 : 0.0; break;
        case KID_HIPASS: kr = (k > kp.c[0]) ? 1.0 : 0.0; break;
        case KID_TOPHAT: kr = (k >= kp.c[0] && k <= kp.c[1]) ? 1.0 : 0.0; break;
        case KID_GAUSSIAN: { double kR = k * kp.c[0]; kr = exp(-kR * kR); break; }
        case KID_GAUSSIAN_INV: { double kR = k * kp.c[0]; kr = exp(kR * kR); break; }
        case KID_INV_POISSON: kr = (k > 0) ? -1.0 / k / k : 1.0; break;
        case KID_POWER_NO_TRANSFER:
            kr = (k == 0) ? 0.0 : sqrt(kp.c[0] * pow(k / kp.c[2], kp.c[1] - 1.) * k * (2. * M_PI * M_PI));
            break;
        case KID_TRANSFER:
        case KID_INV_TRANSFER:
            if (k == 0) {
                kr = 0.0;
            } else {
                const double T = transfer_at<double>(kp.tk, kp.tlo, kp.thi, kp.k_size, k, kp.c[0]);
                kr = (kp.id == KID_TRANSFER) ? T : 1.0 / T;
            }
            break;
        default: break;
        }
        tab[n2] = (float)kr;
    }
}

// w[j] = W(k_j)^-order for the axis index j < N (kint order), the TSC window undo's factor per axis
__global__ void k_window_table(int N, double half_cell, int order, double *__restrict__ w) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        const double x = (double)kint(j, N) * half_cell;
        const double W = x == 0 ? 1. : sin(x) / x;
        w[j] = 1.0 / pow(W, (double)order);
    }
}

__global__ void k_apply32_iso(int N, const float *__restrict__ tab, const float2 *__restrict__ in,
                              float2 *__restrict__ out) {
    const int H = N / 2 + 1;
    const long total = (long)N * N * H;
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int jy = kint((int)(xy % N), N), jx = kint((int)(xy / N), N);
        const float f = tab[jx * jx + jy * jy + z * z];
        const float2 a = in[id];
        out[id] = make_float2(a.x * f, a.y * f);
    }
}

__global__ void k_apply32_window(int N, const double *__restrict__ w, const float2 *__restrict__ in,
                                 float2 *__restrict__ out) {
    const int H = N / 2 + 1;
    const long total = (long)N * N * H;
    for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
        const int z = (int)(id % H);
        const long xy = id / H;
        const int y = (int)(xy % N), x = (int)(xy / N);
        // k = 0 keeps its mode (the reference's kr = 1 there); w[0] = 1 already
        const float f = (float)w[x] * (float)w[y] * (float)w[z];
        const float2 a = in[id];
        out[id] = make_float2(a.x * f, a.y * f);
    }
}

int apply_kernel_launch(int N, double boxlen, int precision, const KernelParams &kp,
                        const void *in, void *out) {
    const double dk = 2 * M_PI / boxlen;
    const long total = (long)N * N * (N / 2 + 1);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (precision == MITOS_FP32 && (isotropic(kp.id) || kp.id == KID_UNDO_HERMITE)) {
        if (kp.id == KID_UNDO_HERMITE) {
            double *w = (double *)workspace(sizeof(double) * (size_t)N, 170);
            if (!w) return 5;
            launch_begin("apply_kernel_table");
            k_window_table<<<(N + 255) / 256, 256, 0, stream()>>>(N, 0.5 * kp.c[0] / kp.c[1] * dk, kp.order, w);
            count_launch();
            MITOS_LAUNCH_CHECK("fft_apply_kernel_dg window table");
            launch_begin("apply_kernel");
            k_apply32_window<<<blocks, 256, 0, stream()>>>(N, w, (const float2 *)in, (float2 *)out);
        } else {
            const long n2max = 3L * (N / 2) * (N / 2);
            float *tab = (float *)workspace(sizeof(float) * (size_t)(n2max + 1), 171);
            if (!tab) return 5;
            launch_begin("apply_kernel_table");
            k_iso_table<<<(unsigned)((n2max + 256) / 256), 256, 0, stream()>>>(n2max, dk, kp, tab);
            count_launch();
            MITOS_LAUNCH_CHECK("fft_apply_kernel_dg table");
            launch_begin("apply_kernel");
            k_apply32_iso<<<blocks, 256, 0, stream()>>>(N, tab, (const float2 *)in, (float2 *)out);
        }
        count_launch();
        MITOS_LAUNCH_CHECK("fft_apply_kernel_dg");
        return 0;
    }
    launch_begin("apply_kernel");
    if (precision == MITOS_FP32)
        k_apply<float><<<blocks, 256, 0, stream()>>>(N, dk, kp, (const float2 *)in, (float2 *)out);
    else
        k_apply<double><<<blocks, 256, 0, stream()>>>(N, dk, kp, (const double2 *)in, (double2 *)out);
    count_launch();
    MITOS_LAUNCH_CHECK("fft_apply_kernel_dg");
    return 0;
}

// ---- fused-pipeline filter: sqrt(P_prim(k)) T(k, tau_src) rescale G(k) per n2 -------------
// (include/fft_kernels.h:116-155 then :96-99), tabulated per squared integer wavevector norm
int filter_table(int N, double boxlen, int precision, double A_s, double n_s, double k_pivot,
                 const double *kt, const double *tlo, const double *thi, int k_size, double u_tau,
                 double rescale, int poisson, void **dev) {
    const long n2max = 3L * (N / 2) * (N / 2);
    const double dk = 2 * M_PI / boxlen;
    std::vector<double> f(n2max + 1, 0.0);
    for (long n2 = 1; n2 <= n2max; n2++) {
        const double k = sqrt((double)n2) * dk;
        double v = sqrt(primordial_power_h(k, A_s, n_s, k_pivot));
        v *= transfer_at<double>(kt, tlo, thi, k_size, k, u_tau);
        v *= rescale;
        if (poisson) v *= -1.0 / k / k;
        f[n2] = v;
    }
    const size_t es = precision == MITOS_FP32 ? 4 : 8;
    void *d = workspace(es * (n2max + 1), 100);
    if (!d) return 5;
    if (precision == MITOS_FP32) {
        std::vector<float> ff(f.begin(), f.end());
        MITOS_CUDA(cudaMemcpyAsync(d, ff.data(), es * (n2max + 1), cudaMemcpyHostToDevice, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
    } else {
        MITOS_CUDA(cudaMemcpyAsync(d, f.data(), es * (n2max + 1), cudaMemcpyHostToDevice, stream()));
        MITOS_CUDA(cudaStreamSynchronize(stream()));
    }
    *dev = d;
    return 0;
}

}  // namespace mitos

// ---- the kernel callbacks (include/fft_kernels.h:28-219), host arithmetic ------------------
using mitos::primordial_power_h;
extern "C" {
void kernel_constant(struct kernel *kn) { kn->kern[0] = *((const double *)kn->params); kn->kern[1] = 0; }
void kernel_lowpass(struct kernel *kn) { kn->kern[0] = (kn->k < *((const double *)kn->params)) ? 1.0 : 0.0; kn->kern[1] = 0; }
void kernel_hipass(struct kernel *kn) { kn->kern[0] = (kn->k > *((const double *)kn->params)) ? 1.0 : 0.0; kn->kern[1] = 0; }
void kernel_tophat(struct kernel *kn) {
    const double *p = (const double *)kn->params;
    kn->kern[0] = (kn->k >= p[0] && kn->k <= p[1]) ? 1.0 : 0.0;
    kn->kern[1] = 0;
}
void kernel_elliptic_tophat(struct kernel *kn) {
    const double *p = (const double *)kn->params;
    double kr = kn->kx * p[0] + kn->ky * p[1] + kn->kz * p[2];
    double kk = kn->kx * kn->kx + kn->ky * kn->ky + kn->kz * kn->kz;
    double rr = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    double theta = kk * rr + (p[3] - 1) * kr * kr;
    kn->kern[0] = (theta <= 4 * M_PI * M_PI) ? 1.0 : 0.0;
    kn->kern[1] = 0;
}
void kernel_translate(struct kernel *kn) {
    const double *p = (const double *)kn->params;
    double ph = p[0] * kn->kx + p[1] * kn->ky + p[2] * kn->kz;
    kn->kern[0] = cos(ph);
    kn->kern[1] = sin(ph);
}
void kernel_gaussian(struct kernel *kn) { double kR = kn->k * *((const double *)kn->params); kn->kern[0] = exp(-kR * kR); kn->kern[1] = 0; }
void kernel_gaussian_inv(struct kernel *kn) { double kR = kn->k * *((const double *)kn->params); kn->kern[0] = exp(kR * kR); kn->kern[1] = 0; }
void kernel_inv_poisson(struct kernel *kn) { kn->kern[0] = (kn->k > 0) ? -1.0 / kn->k / kn->k : 1.0; kn->kern[1] = 0; }
void kernel_dx(struct kernel *kn) { kn->kern[0] = 0; kn->kern[1] = kn->kx; }
void kernel_dy(struct kernel *kn) { kn->kern[0] = 0; kn->kern[1] = kn->ky; }
void kernel_dz(struct kernel *kn) { kn->kern[0] = 0; kn->kern[1] = kn->kz; }
void kernel_power_no_transfer(struct kernel *kn) {
    const struct cosmology *c = (const struct cosmology *)kn->params;
    kn->kern[0] = sqrt(primordial_power_h(kn->k, c->A_s, c->n_s, c->k_pivot));
    kn->kern[1] = 0;
}
static double transfer_host(struct kernel *kn) {
    const struct spline_params *sp = (const struct spline_params *)kn->params;
    const struct perturb_data *pd = sp->spline->ptdat;
    const double *arr = pd->delta + (long)sp->index_src * pd->k_size * pd->tau_size;
    return mitos::transfer_at<double>(pd->k, arr + (long)pd->k_size * sp->tau_index,
                                      arr + (long)pd->k_size * (sp->tau_index + 1), pd->k_size, kn->k,
                                      sp->u_tau);
}
void kernel_transfer_function(struct kernel *kn) {
    kn->kern[0] = (kn->k == 0) ? 0.f : transfer_host(kn);
    kn->kern[1] = 0;
}
void kernel_inv_transfer_function(struct kernel *kn) {
    kn->kern[0] = (kn->k == 0) ? 0.f : 1.0 / transfer_host(kn);
    kn->kern[1] = 0;
}
void kernel_undo_Hermite_window(struct kernel *kn) {
    if (kn->k == 0) { kn->kern[0] = 1.0; kn->kern[1] = 0; return; }
    const struct Hermite_kern_params *p = (const struct Hermite_kern_params *)kn->params;
    double Wx = sin(0.5 * kn->kx * p->boxlen / p->N), Wy, Wz;
    double ax = 0.5 * kn->kx * p->boxlen / p->N, ay = 0.5 * kn->ky * p->boxlen / p->N,
           az = 0.5 * kn->kz * p->boxlen / p->N;
    Wx = ax == 0 ? 1. : sin(ax) / ax;
    Wy = ay == 0 ? 1. : sin(ay) / ay;
    Wz = az == 0 ? 1. : sin(az) / az;
    kn->kern[0] = 1.0 / pow(Wx * Wy * Wz, p->order);
    kn->kern[1] = 0;
}
}
