/* Single-rank stand-in for the MPI API used by the reference's hot-path sources.
 * Test infrastructure: lets the oracle build compile those sources unmodified. */
#ifndef ORC_SHIM_MPI_H
#define ORC_SHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_LONG 2
#define MPI_DOUBLE 3
#define MPI_DOUBLE_COMPLEX 4
#define MPI_FLOAT 5
#define MPI_SUM 0
#define MPI_IN_PLACE ((void *)1)
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *s);
int MPI_Barrier(MPI_Comm c);
int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c);
int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r, const int *rcs, const int *displs,
                   MPI_Datatype rt, MPI_Comm c);
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
#endif
