// context.cuh -- cached device tables and workspace.
#pragma once

#include "fft_passes.cuh"

namespace mitos {

const void *window_table(int N, int order, int precision);
const void *stencil_table(int N, int precision);
const int *bin_table(int N, int bins, int linear, double boxlen);
// the bin of a mode of squared integer wavevector norm n2 (-1: outside the bins): linear shells of
// width k_Nyquist / bins, or the reference's log bins (src/calc_powerspec.c:61-63) with
// k = dk sqrt(n2), lmin = log(dk), lmax = log(sqrt(3) dk N / 2); non-decreasing in n2 where >= 0
int pk_bin_of_n2(long n2, int N, int bins, int linear, double dk, double lmin, double lmax);
// the |n|^2 range [lo, hi] of bin b (bins are monotone in |n|^2, so one range; lo > hi when empty);
// status 3 if the bin's |n|^2 values are not contiguous
int bin_n2_range(int N, int bins, int linear, double boxlen, int b, long *lo, long *hi);
// per-bin multiplicity-weighted mode counts and |k| sums of the half-complex grid (host arrays)
int bin_geometry(int N, int bins, int linear, double boxlen, const double **ksum, const long long **count);
// grid-sized scratch buffer number `slot` of `bytes` bytes (kept until mitos_release_all)
void *workspace(size_t bytes, int slot);
// the Z passes' row-copy fault word: its device address (a mapped pinned host int), and the
// host-side check, status 6 when set (call after the library stream has synchronised)
int *zrow_fault_device();
int zrow_fault_check();
// FFT tiles of one grid size: pencils per block of the X / Y passes and rows per block of the Z
// passes (the autotuner's knobs); returns 1 when the tile does not fit the kernels' limits
int set_tiles(int N, int precision, int p_xy, int p_z);
int get_tiles(int N, int precision, int *p_xy, int *p_z);
// radix schedules of the length-N (X / Y) and length-N/2 (Z) transforms, first stage first (the
// autotuner's third knob); returns 1 for a schedule that does not fit.  A schedule other than the
// default moves the FP32 sizes with compile-time kernels (256, 512, 1024) to the runtime-plan ones.
int set_radix(int N, int precision, const int *rad_n, int ns_n, const int *rad_h, int ns_h);
int get_radix(int N, int precision, int *rad_n, int *ns_n, int *rad_h, int *ns_h);
void release_all();
// the cached xoshiro jump-polynomial tables (noise.cu) and thermal sampler tables (thermal.cu)
void release_jump_tables();
void release_thermal_tables();

// white noise (noise.cu)
struct NoiseFilter {
    const void *table;  // device, filter value per n2 (precision of the grid), or NULL
};
// batched form: states (device, one 32-byte start state per realisation) and batch grids
// bstride bytes apart; states = nullptr for one realisation started at st.  zero / zero_bytes
// (optional, 16-byte aligned, a multiple of 16 bytes): a buffer the kernel clears as well (the
// deposit's density grid: the noise is integer-bound and leaves HBM idle, a separate memset not)
int noise_generate(const GridGeom &g, int precision, double boxlen, uint64_t st[4],
                   const void *filter_by_n2, void *fbox, const void *states = nullptr, int batch = 1,
                   size_t bstride = 0, void *zero = nullptr, size_t zero_bytes = 0);
int hermitian_planes(const GridGeom &g, int precision, void *fbox, int batch = 1, size_t bstride = 0);
void rng_jump(uint64_t st[4], unsigned long long n);

}  // namespace mitos
