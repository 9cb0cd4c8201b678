/* Single-rank stand-in for the MPI interface pyLOM's compiled SVD path uses
 * (pyLOM/vmmath/src/svd.c, vector_matrix.c): COMM_WORLD of size 1, so the
 * TSQR butterfly has no levels, point-to-point traffic never happens and an
 * allreduce is a copy.  Test infrastructure: it lets the reference's own C
 * sources build into the CPU baseline without an MPI installation. */
#ifndef PLOM_REF_MPI_STUB_H
#define PLOM_REF_MPI_STUB_H
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
  int unused;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_C_FLOAT_COMPLEX 8
#define MPI_C_DOUBLE_COMPLEX 16
#define MPI_SUM 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)1)

static inline int MPI_Comm_rank(MPI_Comm c, int* r) {
  (void)c;
  *r = 0;
  return 0;
}
static inline int MPI_Comm_size(MPI_Comm c, int* s) {
  (void)c;
  *s = 1;
  return 0;
}
/* one rank: nobody to talk to */
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)dst; (void)tag; (void)c;
  abort();
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c,
                           MPI_Status* s) {
  (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)s;
  abort();
}
/* the datatype constants above are their element sizes in bytes */
static inline int MPI_Allreduce(const void* sb, void* rb, int n, MPI_Datatype t, MPI_Op op,
                                MPI_Comm c) {
  (void)op; (void)c;
  if (sb != MPI_IN_PLACE && sb != rb) memcpy(rb, sb, (size_t)n * (size_t)t);
  return 0;
}
#endif
