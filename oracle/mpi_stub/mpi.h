/* Single-rank stand-in for the few MPI calls repeat_cpu_omp.cpp makes
 * (Init, Finalize, Comm_rank, Comm_size, Reduce). Written for this project. */
#ifndef MPI_STUB_H
#define MPI_STUB_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_SUM 1
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype t, MPI_Op op, int root,
                             MPI_Comm c) {
    (void)op; (void)root; (void)c;
    memcpy(recv, send, (size_t)count * (size_t)t);
    return 0;
}
#endif
