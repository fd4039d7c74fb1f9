/* Serial single-rank stand-in for the MPI subset the reference DMD sources use
 * (grep of MPI_* over src_v4.5.7: Init/Initialized/Finalize/Abort/Comm_size/Comm_rank/Barrier/
 * Allreduce/Reduce/Bcast/Send/Recv/Probe/Get_count). Oracle build infrastructure only: with one
 * rank every in-place reduction is the identity and every broadcast is a no-op. */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4

#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_DOUBLE 3
#define MPI_DOUBLE_COMPLEX 4
#define MPI_UNSIGNED_CHAR 5
#define MPI_UNSIGNED_SHORT 6
#define MPI_UNSIGNED 7
#define MPI_UNSIGNED_LONG 8
#define MPI_UNSIGNED_LONG_LONG 9
#define MPI_LONG 10
#define MPI_FLOAT 11

static inline size_t oracle_mpi_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: case MPI_UNSIGNED_CHAR: return 1;
    case MPI_UNSIGNED_SHORT: return 2;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_DOUBLE: case MPI_UNSIGNED_LONG: case MPI_UNSIGNED_LONG_LONG: case MPI_LONG: return 8;
    case MPI_DOUBLE_COMPLEX: return 16;
    default: return 8;
  }
}
static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Initialized(int* flag) { *flag = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * oracle_mpi_type_size(t));
  return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)root; return MPI_Allreduce(s, r, n, t, op, c);
}
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; fprintf(stderr, "serial MPI stub: MPI_Send unsupported\n"); abort(); return 0;
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status* st) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; fprintf(stderr, "serial MPI stub: MPI_Recv unsupported\n"); abort(); return 0;
}
static inline int MPI_Probe(int s, int tag, MPI_Comm c, MPI_Status* st) {
  (void)s; (void)tag; (void)c; (void)st; fprintf(stderr, "serial MPI stub: MPI_Probe unsupported\n"); abort(); return 0;
}
static inline int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* n) { (void)st; (void)t; *n = 0; return 0; }
#endif
