/* Single-rank stand-in for the MPI interface used by the reference sources.
 * TEST INFRASTRUCTURE ONLY (builds the reference's own C files as a CPU
 * oracle).  With one rank every collective is a local copy or a no-op, which
 * is what running the reference under `mpirun -np 1` does. */
#ifndef HQR_SHIM_MPI_H
#define HQR_SHIM_MPI_H
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;          /* builtin types carry their size in bytes */
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_UNSIGNED_LONG 8
#define MPI_SUCCESS 0

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code); return 0; }
static inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *t) { *t = n * old; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn,
                             MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rn; (void)rt; (void)root; (void)c; memcpy(r, s, (size_t)sn * (size_t)st); return 0; }
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn,
                                MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)rt; (void)c; memcpy(r, s, (size_t)sn * (size_t)st); return 0; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }
#endif
