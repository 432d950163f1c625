/* Single-rank stand-in for the MPI calls GraphMP's engine makes
 * (GraphMP/system/Global.h:336-343, GraphMP/system/GraphPS.h:296,309-313).
 * Test infrastructure only: it lets the reference's own engine run in one
 * process so its outputs can pin the oracle. */
#ifndef GX_STUB_MPI_H
#define GX_STUB_MPI_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_LONG 8
#define MPI_FLOAT 14
#define MPI_DOUBLE 18
#define MPI_SUM 0
#define MPI_MAX_PROCESSOR_NAME 64
static inline int gx_stub_size(MPI_Datatype t) {
  switch (t) { case MPI_CHAR: return 1; case MPI_INT: return 4; case MPI_FLOAT: return 4;
               case MPI_LONG: return 8; case MPI_DOUBLE: return 8; default: return 1; }
}
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Get_processor_name(char* name, int* len) {
  strcpy(name, "localhost"); *len = 9; return 0;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
  memcpy(r, s, (size_t)n * gx_stub_size(t)); return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  memcpy(r, s, (size_t)n * gx_stub_size(t)); return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  memcpy(r, s, (size_t)n * gx_stub_size(t)); return 0;
}
#endif
