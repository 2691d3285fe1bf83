/* Single-rank stand-in for the MPI calls ThunderEgg makes, so that its hot
 * path compiles and runs as one process without an MPI installation.
 * Collectives over one rank copy their input; point-to-point calls are never
 * reached with one rank and abort if they are. TEST INFRASTRUCTURE ONLY. */
#ifndef TE_REF_MPI_SHIM_H
#define TE_REF_MPI_SHIM_H
#include <cstdlib>
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int count;
};
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_SUCCESS 0
#define MPI_ANY_SOURCE -1
#define MPI_MAX_ERROR_STRING 64
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Finalized(int* f) { *f = 0; return 0; }
inline int MPI_Initialized(int* f) { *f = 1; return 0; }
inline int MPI_Abort(MPI_Comm, int c) { std::exit(c); }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* o) { *o = c; return 0; }
inline int MPI_Comm_free(MPI_Comm*) { return 0; }
inline int MPI_Error_string(int, char* s, int* l) { s[0] = 0; *l = 0; return 0; }
/* the datatype constants above are their byte sizes */
inline int MPI_Allreduce(const void* a, void* b, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  std::memcpy(b, a, (size_t)n * t); return 0; }
inline int MPI_Scan(const void* a, void* b, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  std::memcpy(b, a, (size_t)n * t); return 0; }
inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { std::abort(); }
inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { std::abort(); }
inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { std::abort(); }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { std::abort(); }
inline int MPI_Probe(int, int, MPI_Comm, MPI_Status*) { std::abort(); }
inline int MPI_Get_count(const MPI_Status*, MPI_Datatype, int*) { std::abort(); }
inline int MPI_Waitany(int, MPI_Request*, int*, MPI_Status*) { std::abort(); }
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
#endif
