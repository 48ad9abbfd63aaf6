// fft_passes.cu -- dispatch of the FFT passes: compile-time specialised kernels for the FP32
// sizes 64, 96, 128, 256, 512 and 1024 (instantiated in fft_ct*.cu), runtime-plan kernels otherwise.
#include "fft_kernels.cuh"

namespace mitos {

// specialised entry points (fft_ct64.cu, fft_ct96.cu, fft_ct128.cu, fft_ct256.cu, fft_ct512.cu,
// fft_ct1024.cu)
#define MITOS_CT_DECL(N)                                                                          \
    int launch_x_ct##N(const GridGeom &g, XOp op, int sign, const PassArgs &a);                  \
    int launch_y_ct##N(const GridGeom &g, YOp op, int sign, const PassArgs &a);                  \
    int launch_zc_ct##N(const GridGeom &g, ZOp op, const PassArgs &a);                           \
    int launch_zr_ct##N(const GridGeom &g, const PassArgs &a);
MITOS_CT_DECL(64)
MITOS_CT_DECL(96)
MITOS_CT_DECL(128)
MITOS_CT_DECL(256)
MITOS_CT_DECL(512)
MITOS_CT_DECL(1024)

// pencils per block of the specialised X / Y kernels (512 threads of 8 elements)
// (a radix schedule set by set_radix runs on the runtime-plan kernels)
static inline bool ct_ok(const GridGeom &g, int N) {
    const int E = N % 3 == 0 ? 12 : 8;
    return g.N == N && g.E == E && g.P_xy == 512 / (N / E) && !g.custom_radix;
}

template <typename T> int launch_x(const GridGeom &g, XOp op, int sign, const PassArgs &a) {
    if constexpr (sizeof(T) == 4) {
        if (ct_ok(g, 512)) return launch_x_ct512(g, op, sign, a);
        if (ct_ok(g, 256)) return launch_x_ct256(g, op, sign, a);
        if (ct_ok(g, 1024)) return launch_x_ct1024(g, op, sign, a);
        if (ct_ok(g, 128)) return launch_x_ct128(g, op, sign, a);
        if (ct_ok(g, 64)) return launch_x_ct64(g, op, sign, a);
        if (ct_ok(g, 96)) return launch_x_ct96(g, op, sign, a);
    }
    return launch_x_t<T, 0, 0>(g, op, sign, a);
}
template <typename T> int launch_y(const GridGeom &g, YOp op, int sign, const PassArgs &a) {
    if constexpr (sizeof(T) == 4) {
        if (ct_ok(g, 512)) return launch_y_ct512(g, op, sign, a);
        if (ct_ok(g, 256)) return launch_y_ct256(g, op, sign, a);
        if (ct_ok(g, 1024)) return launch_y_ct1024(g, op, sign, a);
        if (ct_ok(g, 128)) return launch_y_ct128(g, op, sign, a);
        if (ct_ok(g, 64)) return launch_y_ct64(g, op, sign, a);
        if (ct_ok(g, 96)) return launch_y_ct96(g, op, sign, a);
    }
    return launch_y_t<T, 0, 0>(g, op, sign, a);
}
template <typename T> int launch_z_c2r(const GridGeom &g, ZOp op, const PassArgs &a) {
    if constexpr (sizeof(T) == 4) {
        if (ct_ok(g, 512)) return launch_zc_ct512(g, op, a);
        if (ct_ok(g, 256)) return launch_zc_ct256(g, op, a);
        if (ct_ok(g, 1024)) return launch_zc_ct1024(g, op, a);
        if (ct_ok(g, 128)) return launch_zc_ct128(g, op, a);
        if (ct_ok(g, 64)) return launch_zc_ct64(g, op, a);
        if (ct_ok(g, 96)) return launch_zc_ct96(g, op, a);
    }
    return launch_zc_t<T, 0>(g, op, a);
}
template <typename T> int launch_z_r2c(const GridGeom &g, const PassArgs &a) {
    if constexpr (sizeof(T) == 4) {
        if (ct_ok(g, 512)) return launch_zr_ct512(g, a);
        if (ct_ok(g, 256)) return launch_zr_ct256(g, a);
        if (ct_ok(g, 1024)) return launch_zr_ct1024(g, a);
        if (ct_ok(g, 128)) return launch_zr_ct128(g, a);
        if (ct_ok(g, 64)) return launch_zr_ct64(g, a);
        if (ct_ok(g, 96)) return launch_zr_ct96(g, a);
    }
    return launch_zr_t<T, 0>(g, a);
}

template int launch_x<float>(const GridGeom &, XOp, int, const PassArgs &);
template int launch_x<double>(const GridGeom &, XOp, int, const PassArgs &);
template int launch_y<float>(const GridGeom &, YOp, int, const PassArgs &);
template int launch_y<double>(const GridGeom &, YOp, int, const PassArgs &);
template int launch_z_c2r<float>(const GridGeom &, ZOp, const PassArgs &);
template int launch_z_c2r<double>(const GridGeom &, ZOp, const PassArgs &);
template int launch_z_r2c<float>(const GridGeom &, const PassArgs &);
template int launch_z_r2c<double>(const GridGeom &, const PassArgs &);

}  // namespace mitos
