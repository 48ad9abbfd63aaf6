/* Stand-in for the FFTW3 API used by the reference's hot-path sources, backed by the
 * oracle's own FFT (FFTW conventions).  Test infrastructure only. */
#ifndef ORC_SHIM_FFTW3_H
#define ORC_SHIM_FFTW3_H
#include <complex.h>
#include <stddef.h>
typedef double _Complex fftw_complex;
typedef float _Complex fftwf_complex;
typedef struct orc_shim_plan *fftw_plan;
typedef struct orc_shim_plan *fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_complex *fftw_alloc_complex(size_t n);
double *fftw_alloc_real(size_t n);
fftwf_complex *fftwf_alloc_complex(size_t n);
float *fftwf_alloc_real(size_t n);
void fftwf_free(void *p);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned f);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned f);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
