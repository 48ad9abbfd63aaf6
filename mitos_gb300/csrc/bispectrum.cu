// bispectrum.cu -- calc_bispectrum (src/calc_powerspec.c:295-508) on the GPU.  For each log bin i
// (k1 = k2 in bin i of `bins`; k3 in the bin of `bins3` picked by theta, type 0, or by the value k3,
// type 1): one pass masks the field to both shells (ones in volume mode) and sums their wavenumbers
// and multiplicities, the library's c2r takes both masks to real space (/ V), and a reduction sums
// delta_1^2 delta_3 over the N^3 cells.  The bin of every |n|^2 comes from the same table as
// calc_cross_powerspec's log bins (float u, src/calc_powerspec.c:62).  Empty bins keep zeros; the
// reference's per-bin printf is not reproduced.
//
// The reference skips a bin whose shell 1 or shell 3 holds no mode (:436); the host knows those
// counts from the bin tables, so every bin is enqueued without a wait and the sums come back in one
// copy at the end.  When shell 3 is shell 1 (bins3 = bins and k3 in bin i: the equilateral case),
// the two masks are the same array, so one c2r serves both (the second would be bit-identical).
#include <math.h>
#include <string.h>

#include <vector>

#include "context.cuh"
#include "grids.cuh"

namespace mitos {

// acc: [k1 sum, k3 sum, k1 multiplicity, k3 multiplicity].  One warp a row (x, y) of the half-complex
// grid, its lanes along z (one division a row, none an element).
// The shells are the |n|^2 ranges [lo1, hi1] and [lo3, hi3] of the bins (log bins are monotone in
// |n|^2), so the mask needs no table reads.
template <typename T>
__global__ void k_bispec_mask(int N, double dk, const cplx<T> *__restrict__ f, int lo1, int hi1, int lo3, int hi3,
                              int volume, cplx<T> *__restrict__ o1, cplx<T> *__restrict__ o3, double *acc) {
    const int H = N / 2 + 1;
    const int lane = threadIdx.x & 31;
    const long warps = (long)gridDim.x * (blockDim.x >> 5);
    double s1 = 0, s3 = 0, c1 = 0, c3 = 0;
    for (long row = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < (long)N * N; row += warps) {
        const int x = (int)(row / N), y = (int)(row - (long)x * N);
        const int jx = kint(x, N), jy = kint(y, N);
        const int b2 = jx * jx + jy * jy;
        const long base = row * H;
        for (int z = lane; z < H; z += 32) {
            const long id = base + z;
            const int n2 = b2 + z * z;
            cplx<T> v1 = mk<T>(0, 0), v3 = mk<T>(0, 0);
            if (n2 > 0) {
                const bool in1 = n2 >= lo1 && n2 <= hi1, in3 = n2 >= lo3 && n2 <= hi3;
                if (in1 || in3) {
                    const cplx<T> val = volume ? mk<T>(1, 0) : f[id];
                    const double mult = (z == 0 || z == N / 2) ? 1.0 : 2.0;
                    // fft_wavevector's k (src/fft.c:29-35), without contractions
                    const double kx = __dmul_rn((double)jx, dk), ky = __dmul_rn((double)jy, dk),
                                 kz = __dmul_rn((double)z, dk);
                    const double k = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz)));
                    if (in1) {
                        v1 = val;
                        s1 += mult * k;
                        c1 += mult;
                    }
                    if (in3) {
                        v3 = val;
                        s3 += mult * k;
                        c3 += mult;
                    }
                }
            }
            o1[id] = v1;
            if (o3) o3[id] = v3;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        s1 += __shfl_down_sync(0xffffffffu, s1, off);
        s3 += __shfl_down_sync(0xffffffffu, s3, off);
        c1 += __shfl_down_sync(0xffffffffu, c1, off);
        c3 += __shfl_down_sync(0xffffffffu, c3, off);
    }
    if (lane == 0 && (c1 != 0 || c3 != 0)) {
        atomicAdd(acc, s1);
        atomicAdd(acc + 1, s3);
        atomicAdd(acc + 2, c1);
        atomicAdd(acc + 3, c3);
    }
}

// sum of m1^2 m3 over the N^3 cells of two padded real grids (row pitch N + 2): one warp a row
template <typename T>
__global__ void k_triple_sum(int N, const T *__restrict__ m1, const T *__restrict__ m3, double *out) {
    const int lane = threadIdx.x & 31;
    const long warps = (long)gridDim.x * (blockDim.x >> 5);
    T s = 0;
    for (long row = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < (long)N * N; row += warps) {
        const T *r1 = m1 + row * (N + 2), *r3 = m3 + row * (N + 2);
        for (int z = lane; z < N; z += 32) {
            const T a = r1[z];
            s += a * a * r3[z];
        }
    }
    double d = (double)s;
    for (int off = 16; off > 0; off >>= 1) d += __shfl_down_sync(0xffffffffu, d, off);
    if (lane == 0) atomicAdd(out, d);
}

int bispectrum_run(int N, double boxlen, int prec, const void *fbox, int bins, int bins3, double *k1_in_bins,
                   double *k2_in_bins, double *k3_in_bins, double *bispectrum, int volume_mode, int type,
                   double theta, double k3) {
    if (bins < 1 || bins3 < 1 || (!fbox && !volume_mode)) {
        set_error(1, "calc_bispectrum: bins >= 1, bins3 >= 1 and a field (outside volume mode) needed");
        return 1;
    }
    const GridGeom *gp = geom(N, prec);
    if (!gp) return 3;
    const GridGeom &g = *gp;
    const size_t gb = (size_t)g.cells * csize(prec);
    const double *ks1, *ks3;
    const long long *cn1, *cn3;
    if (bin_geometry(N, bins, 0, boxlen, &ks1, &cn1) || bin_geometry(N, bins3, 0, boxlen, &ks3, &cn3)) return 5;
    void *o1 = workspace(gb, 30), *o3 = workspace(gb, 31), *m1 = workspace(gb, 32), *m3 = workspace(gb, 33);
    // per bin: [k1 sum, k3 sum, k1 multiplicity, k3 multiplicity, sum delta_1^2 delta_3]
    double *acc = (double *)workspace(sizeof(double) * 5 * bins, 34);
    if (!o1 || !o3 || !m1 || !m3 || !acc) return 5;
    const double dk = 2 * M_PI / boxlen;
    const double max_k = sqrt(3) * dk * N / 2;
    const double min_k = dk;
    const double log_max_k = log(max_k);
    const double log_min_k = log(min_k);
    for (int i = 0; i < bins; i++) {
        k1_in_bins[i] = 0;
        k2_in_bins[i] = 0;
        k3_in_bins[i] = 0;
        bispectrum[i] = 0;
    }
    MITOS_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 5 * bins, stream()));
    const long total = (long)N * N * (N / 2 + 1);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    std::vector<char> done(bins, 0);
    for (int i = 0; i < bins; i++) {
        // src/calc_powerspec.c:347-369, host libm as in the reference
        int required_bin3;
        if (type == 0) {
            const double k1 = exp((i + 0.5) * (log_max_k - log_min_k) / (bins3 - 1) + log_min_k);
            const double k2 = exp((i + 0.5) * (log_max_k - log_min_k) / (bins3 - 1) + log_min_k);
            const double required_k3 = sqrt(k1 * k1 + k2 * k2 + 2 * k1 * k2 * cos(theta));
            const float u3 = (log(required_k3) - log_min_k) / (log_max_k - log_min_k);
            required_bin3 = (int)floor((bins3 - 1) * u3);
        } else if (type == 1) {
            const float u3 = (log(k3) - log_min_k) / (log_max_k - log_min_k);
            required_bin3 = (int)floor((bins3 - 1) * u3);
        } else {
            required_bin3 = 0;
        }
        // src/calc_powerspec.c:436: a shell without modes skips the bin
        const long long c1 = cn1[i];
        const long long c3 = (required_bin3 >= 0 && required_bin3 < bins3) ? cn3[required_bin3] : 0;
        if (c1 == 0 || c3 == 0) continue;
        done[i] = 1;
        const bool same = bins == bins3 && required_bin3 == i;
        long lo1, hi1, lo3, hi3;
        int er = bin_n2_range(N, bins, 0, boxlen, i, &lo1, &hi1);
        if (!er) er = bin_n2_range(N, bins3, 0, boxlen, required_bin3, &lo3, &hi3);
        if (er) return er;
        double *ab = acc + 5 * (size_t)i;
        launch_begin("bispec_mask");
        if (prec == MITOS_FP32)
            k_bispec_mask<float><<<blocks, 256, 0, stream()>>>(N, dk, (const float2 *)fbox, (int)lo1, (int)hi1, (int)lo3,
                                                               (int)hi3, volume_mode, (float2 *)o1,
                                                               same ? nullptr : (float2 *)o3, ab);
        else
            k_bispec_mask<double><<<blocks, 256, 0, stream()>>>(N, dk, (const double2 *)fbox, (int)lo1, (int)hi1,
                                                                (int)lo3, (int)hi3, volume_mode, (double2 *)o1,
                                                                same ? nullptr : (double2 *)o3, ab);
        count_launch();
        MITOS_LAUNCH_CHECK("bispectrum mask");
        int e = grid_c2r(g, prec, boxlen, o1, m1);
        if (!e && !same) e = grid_c2r(g, prec, boxlen, o3, m3);
        if (e) return e;
        const void *m3s = same ? m1 : m3;
        launch_begin("bispec_sum");
        if (prec == MITOS_FP32)
            k_triple_sum<float><<<152 * 8, 256, 0, stream()>>>(N, (const float *)m1, (const float *)m3s, ab + 4);
        else
            k_triple_sum<double><<<152 * 8, 256, 0, stream()>>>(N, (const double *)m1, (const double *)m3s, ab + 4);
        count_launch();
        MITOS_LAUNCH_CHECK("bispectrum sum");
    }
    std::vector<double> h(5 * (size_t)bins);
    MITOS_CUDA(cudaMemcpyAsync(h.data(), acc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream()));
    MITOS_CUDA(cudaStreamSynchronize(stream()));
    for (int i = 0; i < bins; i++) {
        if (!done[i]) continue;
        const double *hb = h.data() + 5 * (size_t)i;
        bispectrum[i] = hb[4];
        k1_in_bins[i] = hb[0] / hb[2];
        k2_in_bins[i] = hb[0] / hb[2];
        k3_in_bins[i] = hb[1] / hb[3];
    }
    return 0;
}

}  // namespace mitos
