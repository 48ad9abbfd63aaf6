// fft_ct96.cu -- compile-time specialised FP32 FFT passes for N = 96 = 3 2^5 (12 elements a thread:
// X / Y length 96 in radices 4, 4, 2, 3; Z length 48; 64 pencils per X / Y block): the ensemble's
// middle boxes.
#include "fft_kernels.cuh"

namespace mitos {
int launch_x_ct96(const GridGeom &g, XOp op, int sign, const PassArgs &a) { return launch_x_t<float, 96, 64>(g, op, sign, a); }
int launch_y_ct96(const GridGeom &g, YOp op, int sign, const PassArgs &a) { return launch_y_t<float, 96, 64>(g, op, sign, a); }
int launch_zc_ct96(const GridGeom &g, ZOp op, const PassArgs &a) { return launch_zc_t<float, 48>(g, op, a); }
int launch_zr_ct96(const GridGeom &g, const PassArgs &a) { return launch_zr_t<float, 48>(g, a); }
}  // namespace mitos
