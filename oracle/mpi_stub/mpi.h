/*
 * Serial stand-in for the handful of MPI calls the SFCMM/LBM reference makes.
 *
 * TEST INFRASTRUCTURE ONLY: this header lets oracle/build_ref.sh compile the
 * reference's own grid generator and LBM solver on a machine without an MPI
 * installation, so that its CPU results can pin the project's oracle and the
 * GPU kernels.  The reference refuses to run on more than one rank
 * (src/gridgenerator/gridGenerator.cpp:118-120), so a one-rank world is exact:
 * every collective degenerates to a copy and every barrier to a no-op.
 */
#ifndef LBM_ORACLE_MPI_STUB_H
#define LBM_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Errhandler;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_ERRORS_RETURN 0
#define MPI_THREAD_FUNNELED 1
#define MPI_SUM 0
#define MPI_DOUBLE 8
#define MPI_MAX_INFO_KEY 255
#define MPI_MAX_INFO_VAL 1024

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Init_thread(int*, char***, int required, int* provided) {
  *provided = required;
  return 0;
}
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) {
  *rank = 0;
  return 0;
}
static inline int MPI_Comm_size(MPI_Comm, int* size) {
  *size = 1;
  return 0;
}
static inline int MPI_Comm_set_errhandler(MPI_Comm, MPI_Errhandler) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) {
  fprintf(stderr, "MPI_Abort(%d) called (serial stub)\n", code);
  fflush(stderr);
  exit(code == 0 ? 1 : code);
}
static inline double MPI_Wtime() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
/* one rank: a reduction is a copy of the send buffer */
static inline int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm) {
  if(send != recv) memcpy(recv, send, (size_t)count * (size_t)type);
  return 0;
}
static inline int MPI_Info_create(MPI_Info* info) {
  *info = 0;
  return 0;
}
static inline int MPI_Info_set(MPI_Info, const char*, const char*) { return 0; }
static inline int MPI_Info_get_nkeys(MPI_Info, int* nkeys) {
  *nkeys = 0;
  return 0;
}
static inline int MPI_Info_get_nthkey(MPI_Info, int, char* key) {
  key[0] = 0;
  return 0;
}
static inline int MPI_Info_get_valuelen(MPI_Info, const char*, int* len, int* flag) {
  *len  = 0;
  *flag = 0;
  return 0;
}
static inline int MPI_Info_get(MPI_Info, const char*, int, char* value, int* flag) {
  value[0] = 0;
  *flag    = 0;
  return 0;
}

#endif
