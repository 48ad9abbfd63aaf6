// fft_ct128.cu -- compile-time specialised FP32 FFT passes for N = 128 (X / Y length 128, Z length
// 64, 32 pencils per X / Y block): the ensemble's largest boxes.
#include "fft_kernels.cuh"

namespace mitos {
int launch_x_ct128(const GridGeom &g, XOp op, int sign, const PassArgs &a) { return launch_x_t<float, 128, 32>(g, op, sign, a); }
int launch_y_ct128(const GridGeom &g, YOp op, int sign, const PassArgs &a) { return launch_y_t<float, 128, 32>(g, op, sign, a); }
int launch_zc_ct128(const GridGeom &g, ZOp op, const PassArgs &a) { return launch_zc_t<float, 64>(g, op, a); }
int launch_zr_ct128(const GridGeom &g, const PassArgs &a) { return launch_zr_t<float, 64>(g, a); }
}  // namespace mitos
