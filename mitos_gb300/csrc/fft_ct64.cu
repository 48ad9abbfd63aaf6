// fft_ct64.cu -- compile-time specialised FP32 FFT passes for N = 64 (X / Y length 64, Z length 32,
// 64 pencils per X / Y block): the ensemble's smallest boxes.
#include "fft_kernels.cuh"

namespace mitos {
int launch_x_ct64(const GridGeom &g, XOp op, int sign, const PassArgs &a) { return launch_x_t<float, 64, 64>(g, op, sign, a); }
int launch_y_ct64(const GridGeom &g, YOp op, int sign, const PassArgs &a) { return launch_y_t<float, 64, 64>(g, op, sign, a); }
int launch_zc_ct64(const GridGeom &g, ZOp op, const PassArgs &a) { return launch_zc_t<float, 32>(g, op, a); }
int launch_zr_ct64(const GridGeom &g, const PassArgs &a) { return launch_zr_t<float, 32>(g, a); }
}  // namespace mitos
