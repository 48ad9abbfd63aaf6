// kspace.cuh -- device kernel-callback dispatch and filter tables.
#pragma once

#include "common.cuh"

namespace mitos {

enum KernelId {
    KID_CONSTANT = 0, KID_LOWPASS, KID_HIPASS, KID_TOPHAT, KID_ELLIPTIC_TOPHAT, KID_TRANSLATE,
    KID_GAUSSIAN, KID_GAUSSIAN_INV, KID_INV_POISSON, KID_DX, KID_DY, KID_DZ,
    KID_POWER_NO_TRANSFER, KID_TRANSFER, KID_INV_TRANSFER, KID_UNDO_HERMITE
};

struct KernelParams {
    int id;
    int order;         // KID_UNDO_HERMITE
    double c[4];       // scalar parameters (see k_apply)
    const double *tk;  // KID_TRANSFER: device k table and the two tau rows
    const double *tlo, *thi;
    int k_size;
};

int apply_kernel_launch(int N, double boxlen, int precision, const KernelParams &kp,
                        const void *in, void *out);
double primordial_power_h(double k, double A_s, double n_s, double k_pivot);
void find_tau_h(const struct perturb_data *pd, double log_tau, int *index, double *u);
double log_tau_at_z_h(const struct perturb_data *pd, double redshift);
int filter_table(int N, double boxlen, int precision, double A_s, double n_s, double k_pivot,
                 const double *kt, const double *tlo, const double *thi, int k_size, double u_tau,
                 double rescale, int poisson, void **dev);
// transfer function at k: perturbSplineFindK + perturbSplineInterp (src/perturb_spline.c:109-169);
// the index search returns the node whose interpolation the reference's linear search uses
// (an equal value when k sits exactly on a node)
template <typename R>
__host__ __device__ inline R transfer_at(const R *kt, const R *lo, const R *hi, int k_size, R k,
                                         R u_tau) {
    int i;
    R u;
    if (k > kt[k_size - 1]) {
        i = k_size - 2;
        u = 1.0;
    } else {
        int a = 0, b = k_size - 1;  // largest i with kt[i] <= k, in [0, k_size - 2]
        while (b - a > 1) {
            int m = (a + b) >> 1;
            if (kt[m] <= k) a = m; else b = m;
        }
        i = a;
        u = (k - kt[i]) / (kt[i + 1] - kt[i]);
    }
    const R T11 = lo[i], T21 = lo[i + 1], T12 = hi[i], T22 = hi[i + 1];
    return (1 - u_tau) * ((1 - u) * T11 + u * T21) + u_tau * ((1 - u) * T12 + u * T22);
}

}  // namespace mitos
