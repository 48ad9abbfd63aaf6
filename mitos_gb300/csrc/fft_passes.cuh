// fft_passes.cuh -- the pass kernels of the 3D real FFT and their fused k-space epilogues.
//
// Layouts (one rank, reference layout of struct distributed_grid):
//   complex grid  element (x, y, kz) at (x*N + y)*H + kz,    H = N/2 + 1
//   real grid     element (x, y, z)  at (x*N + y)*rp + z,    rp = N + 2 (padded) or N
// c2r = X pass (complex, along x) -> Y pass (complex, along y) -> Z pass (half-complex -> real)
// r2c = Z pass (real -> half-complex) -> Y pass -> X pass.  The Z c2r uses only the real parts
// of the kz = 0 and kz = N/2 elements, as FFTW's c2r does.
#pragma once

#include "fft_core.cuh"

namespace mitos {

// shared description of one grid size / precision
struct GridGeom {
    int N, H;
    long plane;   // N*H complex elements per x-plane
    long cells;   // N*N*H complex elements
    int E;        // elements per thread (8 for 2^k, 12 for 3*2^k)
    FFTPlan plN;  // length-N plan (X and Y passes)
    FFTPlan plH;  // length-N/2 plan (Z passes)
    int P_xy;     // pencils per block in X/Y passes
    int P_z;      // rows per block in Z passes
    const void *twN;  // device table exp(-2 pi i m / N), m < N, in the grid precision
    int custom_radix; // 1: radix schedules set by set_radix (the runtime-plan kernels run them)
};

const GridGeom *geom(int N, int precision);  // cached; NULL if N unsupported

// ---- the fused operations a pass can carry -----------------------------------------------
enum XOp {
    XOP_PLAIN = 0,    // out = FFT(in) * scale
    XOP_HESS,         // out0..2 = FFT(phi), FFT(i kx phi), FFT(-kx^2 phi)            (inverse)
    XOP_DISP,         // out0..1 = FFT(phi), FFT(i kx phi)                           (inverse)
    XOP_COMBINE_2LPT, // out = [f1 * in2 + f2 * G(k) * FFT(in) * scale] * W(k)       (forward)
    XOP_ADD_POISSON,  // out = in2 + G(k) * FFT(in) * scale                          (forward)
    XOP_PK,           // P(k) binning of |FFT(in) * scale * W(k)|^2 (+ optional out)  (forward)
    XOP_COMBINE_DISP  // phi = [f1 * in2 + f2 * G(k) * FFT(in) * scale] * W(k) (forward), then
                      // out0..1 = FFT^-1(phi), FFT^-1(i kx phi) (inverse): the 2LPT potential never
                      // leaves the block
};
enum YOp {
    YOP_PLAIN = 0,    // out = FFT(in) * scale
    YOP_DISP_A,       // 1 in -> 2 out: i ky C (y stencil), C (the displacements' d_y and d_z chains)
    YOP_STN,          // 1 in -> 1 out: C (y stencil) (the d_x chain)
    YOP_HESS_A,       // 1 in -> 3 out: -ky^2 A, i ky A, A (the Hessian's yy, yz, zz chains)
    YOP_HESS_B        // 1 in -> 2 out: i ky A, A (xy, xz)
};
enum ZOp {
    ZOP_C2R = 0,      // real out = c2r(in) * scale
    ZOP_HESS_2LPT,    // 6 in (kz factors 1, 1, i kz, 1, i kz, -kz^2) -> S = sum_{i<j} (p_ii p_jj - p_ij^2)
    ZOP_HESS_MA,      // same 6 in -> residual (1 + rho) - det(I + H), sums of res^2 and rho^2;
                      // out[1] (optional): the second-order source S of the same Hessian
    ZOP_DISP,         // 3 in (kz factors 1, 1, i kz) -> 3 real out
    ZOP_HESS_2LPT_K,  // ZOP_HESS_2LPT followed by the r2c of S along z in the same pass: out[0] is
                      // the complex z-transformed source (N/2+1 per row, unnormalised), as
                      // ZOP_HESS_2LPT + a z r2c with scale 1 would leave it
    ZOP_HESS_MA_K,    // ZOP_HESS_MA with the residual's r2c along z in the same pass (out[0] complex,
                      // as above), without the source output: the residual is accumulated as the
                      // rows arrive, four rows live instead of six
    ZOP_HESS_MA_KS    // ZOP_HESS_MA_K with out[1], the second-order source S (real), as well
};

struct PassArgs {
    const void *in[6];
    void *out[6];
    const void *in2;      // second input (XOP_COMBINE_2LPT / XOP_ADD_POISSON) or rho (ZOP_HESS_MA)
    double scale;         // multiplies the transform result
    double dk;            // 2 pi / boxlen
    double f1, f2;        // combination factors
    int window_order;     // 0: none, else 1 / W(k)^order with W = prod sinc(k_i L / 2N)
    int rp_in, rp_out;    // real row pitch for Z passes
    double rho_a, rho_b;  // Z r2c transform on load: x -> x * rho_a + rho_b
    // P(k) binning (XOP_PK)
    const int *bin_of_n2; // bin per squared integer wavevector norm (-1: skip)
    int nbins;
    double *bin_k, *bin_p; long long *bin_n;  // device accumulators
    double *red;          // device FP64 reductions (ZOP_HESS_MA: [0] += res^2, [1] += rho^2)
    // displacement passes: fold the on-node TSC interpolation stencil (1/8, 3/4, 1/8) into the
    // axes along which the later gather sits on grid nodes (x for d_x, y for d_x and d_y, z for
    // all three); table of 3/4 + cos(2 pi m / N)/4 at m + N/2
    const void *stencil;
    // batched launches (the ensemble): batch realisations, blockIdx.y = realisation, every grid
    // pointer (in, out, in2) bstride bytes apart, the P(k) / residual sums acc_stride doubles apart
    int batch;            // 0 or 1: one realisation
    long long bstride;
    int acc_stride;
    // FP32 copies of scale, dk, f1, f2, rho_a, rho_b, filled at launch (with_f32): the FP32
    // kernels read these, as a double -> float conversion per thread runs on the FP64 pipe
    float fscale, fdk, ff1, ff2, frho_a, frho_b;
    // mapped host word a Z pass sets when one of its row copies never completed (bounded wait;
    // the pass then reads the rows from global memory); filled at launch
    int *fault;
    // a region the 2LPT-source Z pass zeroes on the side with streaming stores (16-byte aligned,
    // zero_bytes a multiple of 16; its blocks take consecutive slices): the deposit's density grid
    void *zero;
    size_t zero_bytes;
};

// the kernel's copy of a with the FP32 scalars filled
inline PassArgs with_f32(const PassArgs &a) {
    PassArgs b = a;
    b.fscale = (float)a.scale;
    b.fdk = (float)a.dk;
    b.ff1 = (float)a.f1;
    b.ff2 = (float)a.f2;
    b.frho_a = (float)a.rho_a;
    b.frho_b = (float)a.rho_b;
    return b;
}
// a scalar of PassArgs in the kernel's precision
template <typename T> __device__ __forceinline__ T parg(double d, float f);
template <> __device__ __forceinline__ float parg<float>(double, float f) { return f; }
template <> __device__ __forceinline__ double parg<double>(double d, float) { return d; }

// pointer p shifted by bo bytes (null stays null)
template <typename P> __host__ __device__ __forceinline__ P *bat(const void *p, size_t bo) {
    return p ? reinterpret_cast<P *>(const_cast<char *>(reinterpret_cast<const char *>(p)) + bo) : nullptr;
}

template <typename T> int launch_x(const GridGeom &g, XOp op, int sign, const PassArgs &a);
template <typename T> int launch_y(const GridGeom &g, YOp op, int sign, const PassArgs &a);
template <typename T> int launch_z_c2r(const GridGeom &g, ZOp op, const PassArgs &a);
template <typename T> int launch_z_r2c(const GridGeom &g, const PassArgs &a);

// the r2c's Z and Y steps in one thread-block-cluster pass (fft_cluster.cu); -1: no cluster shape
// for this grid (FP32 N = 256 and 512 have them) or the pass is off, the caller runs the two passes
int launch_zy_r2c(const GridGeom &g, int precision, const PassArgs &a);
void set_cluster_fft(int mode);  // 0: off (the two-pass route); 1..3: a cluster shape
int cluster_fft();
// launch_zy_r2c, else the Z r2c pass and the Y pass in place on a.out[0] (api.cu)
int grid_r2c_zy(const GridGeom &g, int prec, const PassArgs &a);

}  // namespace mitos
