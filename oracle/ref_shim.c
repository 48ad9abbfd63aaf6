/*
 * ref_shim.c -- single-rank MPI, FFTW-over-oracle-FFT and no-op I/O stand-ins that let the
 * reference's hot-path C files compile and run unmodified inside the oracle build.
 * TEST INFRASTRUCTURE ONLY (linked into oracle/_ref/libmitos_ref.so, never into the product).
 */
#include <stdio.h>
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

/* ---- HDF5 attribute recorder (see ref_shim/hdf5.h) --------------------------------------- */
#include "ref_shim/hdf5.h"
#define ORC_H5_MAX 64
struct orc_h5attr {
    char group[32];
    char name[64];
    int type; /* 1 double, 2 int, 3 long */
    int n;
    double d[8];
    long long l[8];
};
static struct orc_h5attr h5_attr[ORC_H5_MAX];
static int h5_nattr = 0;
static char h5_group[16][32];
static int h5_ngroup = 0;
static int h5_extent[16];
static int h5_nspace = 0;

hid_t H5Gcreate(hid_t loc, const char *name, hid_t lcpl, hid_t gcpl, hid_t gapl) {
    (void)loc; (void)lcpl; (void)gcpl; (void)gapl;
    if (h5_ngroup >= 16) return -1;
    snprintf(h5_group[h5_ngroup], sizeof h5_group[0], "%s", name);
    return 100 + h5_ngroup++;
}
herr_t H5Gclose(hid_t grp) { (void)grp; return 0; }
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims) {
    (void)rank; (void)maxdims;
    if (h5_nspace >= 16) return -1;
    h5_extent[h5_nspace] = (int)dims[0];
    return 200 + h5_nspace++;
}
herr_t H5Sset_extent_simple(hid_t space, int rank, const hsize_t *dims, const hsize_t *maxdims) {
    (void)rank; (void)maxdims;
    h5_extent[space - 200] = (int)dims[0];
    return 0;
}
herr_t H5Sclose(hid_t space) { (void)space; return 0; }
hid_t H5Acreate1(hid_t loc, const char *name, hid_t type, hid_t space, hid_t acpl) {
    (void)acpl;
    if (h5_nattr >= ORC_H5_MAX) return -1;
    struct orc_h5attr *a = &h5_attr[h5_nattr];
    memset(a, 0, sizeof *a);
    snprintf(a->group, sizeof a->group, "%s", h5_group[loc - 100]);
    snprintf(a->name, sizeof a->name, "%s", name);
    a->type = (int)type;
    a->n = h5_extent[space - 200];
    return 300 + h5_nattr++;
}
herr_t H5Awrite(hid_t attr, hid_t type, const void *buf) {
    struct orc_h5attr *a = &h5_attr[attr - 300];
    for (int i = 0; i < a->n && i < 8; i++) {
        if (type == H5T_NATIVE_DOUBLE) a->d[i] = ((const double *)buf)[i];
        else if (type == H5T_NATIVE_INT) a->l[i] = ((const int *)buf)[i];
        else a->l[i] = ((const long *)buf)[i];
    }
    return 0;
}
herr_t H5Aclose(hid_t attr) { (void)attr; return 0; }

void orc_h5_reset(void) { h5_nattr = h5_ngroup = h5_nspace = 0; }
int orc_h5_count(void) { return h5_nattr; }
/* attribute i: group and name (NUL-terminated, 32 and 64 bytes), type, count and values */
int orc_h5_get(int i, char *group, char *name, int *type, int *n, double *d, long long *l) {
    if (i < 0 || i >= h5_nattr) return 1;
    memcpy(group, h5_attr[i].group, 32);
    memcpy(name, h5_attr[i].name, 64);
    *type = h5_attr[i].type;
    *n = h5_attr[i].n;
    memcpy(d, h5_attr[i].d, sizeof h5_attr[i].d);
    memcpy(l, h5_attr[i].l, sizeof h5_attr[i].l);
    return 0;
}
