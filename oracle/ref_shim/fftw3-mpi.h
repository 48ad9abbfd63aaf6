/* Single-rank stand-in for the FFTW3-MPI API (padded real rows of 2(N/2+1)). */
#ifndef ORC_SHIM_FFTW3_MPI_H
#define ORC_SHIM_FFTW3_MPI_H
#include "fftw3.h"
#include "mpi.h"
typedef long ptrdiff_t_shim;
void fftw_mpi_init(void);
long fftw_mpi_local_size_3d(long n0, long n1, long n2, MPI_Comm c, long *local_n0, long *local_0_start);
fftw_plan fftw_mpi_plan_dft_r2c_3d(long n0, long n1, long n2, double *in, fftw_complex *out,
                                   MPI_Comm c, unsigned f);
fftw_plan fftw_mpi_plan_dft_c2r_3d(long n0, long n1, long n2, fftw_complex *in, double *out,
                                   MPI_Comm c, unsigned f);
#endif
