// fft_ct256.cu -- compile-time specialised FP32 FFT passes for N = 256 (X / Y length 256,
// Z length 128; 16 pencils per X / Y block at 8 elements a thread, twice that at 16).
#include "fft_kernels.cuh"

namespace mitos {
int launch_x_ct256(const GridGeom &g, XOp op, int sign, const PassArgs &a) { return launch_x_t<float, 256, 16>(g, op, sign, a); }
int launch_y_ct256(const GridGeom &g, YOp op, int sign, const PassArgs &a) { return launch_y_t<float, 256, 16>(g, op, sign, a); }
int launch_zc_ct256(const GridGeom &g, ZOp op, const PassArgs &a) { return launch_zc_t<float, 128>(g, op, a); }
int launch_zr_ct256(const GridGeom &g, const PassArgs &a) { return launch_zr_t<float, 128>(g, a); }
}  // namespace mitos
