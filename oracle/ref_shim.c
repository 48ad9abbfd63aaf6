/*
 * ref_shim.c -- single-rank MPI, FFTW-over-oracle-FFT and no-op I/O stand-ins that let the
 * reference's hot-path C files compile and run unmodified inside the oracle build.
 * TEST INFRASTRUCTURE ONLY (linked into oracle/_ref/libmitos_ref.so, never into the product).
 */
#include <stdlib.h>
#include <string.h>
#include "ref_shim/mpi.h"
#include "ref_shim/fftw3-mpi.h"
#include "mitos_oracle.h"

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

static size_t tsize(MPI_Datatype t) {
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_LONG: return sizeof(long);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_DOUBLE_COMPLEX: return 2 * sizeof(double);
    case MPI_FLOAT: return sizeof(float);
    default: return 1;
    }
}
int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c) {
    (void)rc; (void)rt; (void)c;
    memcpy(r, s, sc * tsize(st));
    return 0;
}
int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r, const int *rcs, const int *displs,
                   MPI_Datatype rt, MPI_Comm c) {
    (void)rcs; (void)c;
    memcpy((char *)r + (size_t)displs[0] * tsize(rt), s, sc * tsize(st));
    return 0;
}
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
    (void)op; (void)root; (void)c;
    if (s != MPI_IN_PLACE && s != r) memcpy(r, s, n * tsize(t));
    return 0;
}
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    return MPI_Reduce(s, r, n, t, op, 0, c);
}

/* ---- FFTW over the oracle's FFT ----------------------------------------------------- */
struct orc_shim_plan { int kind; int N; long rpitch; void *in, *out; };
void *fftw_malloc(size_t n) { return calloc(1, n ? n : 1); }
void fftw_free(void *p) { free(p); }
void fftwf_free(void *p) { free(p); }
fftw_complex *fftw_alloc_complex(size_t n) { return fftw_malloc(n * sizeof(fftw_complex)); }
double *fftw_alloc_real(size_t n) { return fftw_malloc(n * sizeof(double)); }
fftwf_complex *fftwf_alloc_complex(size_t n) { return fftw_malloc(n * sizeof(fftwf_complex)); }
float *fftwf_alloc_real(size_t n) { return fftw_malloc(n * sizeof(float)); }

static fftw_plan mkplan(int kind, int N, long rpitch, void *in, void *out) {
    struct orc_shim_plan *p = malloc(sizeof *p);
    p->kind = kind; p->N = N; p->rpitch = rpitch; p->in = in; p->out = out;
    return p;
}
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned f) {
    (void)n1; (void)n2; (void)f;
    return mkplan(0, n0, n0, in, out);
}
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned f) {
    (void)n1; (void)n2; (void)f;
    return mkplan(1, n0, n0, in, out);
}
fftw_plan fftw_mpi_plan_dft_r2c_3d(long n0, long n1, long n2, double *in, fftw_complex *out,
                                   MPI_Comm c, unsigned f) {
    (void)n1; (void)n2; (void)c; (void)f;
    return mkplan(0, (int)n0, 2 * (n0 / 2 + 1), in, out);
}
fftw_plan fftw_mpi_plan_dft_c2r_3d(long n0, long n1, long n2, fftw_complex *in, double *out,
                                   MPI_Comm c, unsigned f) {
    (void)n1; (void)n2; (void)c; (void)f;
    return mkplan(1, (int)n0, 2 * (n0 / 2 + 1), in, out);
}
void fftw_execute(const fftw_plan p) {
    if (p->kind == 0) orc_dft_r2c_3d(p->N, p->in, p->rpitch, p->out);
    else orc_dft_c2r_3d(p->N, p->in, p->out, p->rpitch);
}
void fftw_destroy_plan(fftw_plan p) { free(p); }
void fftw_mpi_init(void) {}
long fftw_mpi_local_size_3d(long n0, long n1, long n2, MPI_Comm c, long *local_n0, long *local_0_start) {
    (void)c;
    *local_n0 = n0;
    *local_0_start = 0;
    return n0 * n1 * n2;
}

/* ---- no-op I/O and the compiled-out SPT driver ------------------------------------- */
struct distributed_grid;
int writeFieldFile_dg(struct distributed_grid *dg, const char *fname) { (void)dg; (void)fname; return 0; }
int sptChunked(int N, double boxlen, int cycles, char *basename, char *a, char *b, char *c, char *d) {
    (void)N; (void)boxlen; (void)cycles; (void)basename; (void)a; (void)b; (void)c; (void)d;
    return 0;
}
