/*
 * Single-rank MPI stand-in used ONLY to compile the reference's header-only
 * hot path (tree_topology.h, bodies_system.h helpers, physics headers) into
 * the oracle under oracle/_ref.  This is test infrastructure, not product.
 *
 * With one rank every collective is a copy (or a no-op for MPI_IN_PLACE);
 * point-to-point calls are unreachable on one rank and abort if reached.
 */
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_;
};

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_THREAD_MULTIPLE 3
#define MPI_THREAD_SINGLE 0

/* datatypes encode their byte size */
#define MPI_BYTE 1
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 0x104
#define MPI_DOUBLE 8
#define MPI_INT64_T 0x108
#define MPI_UNSIGNED_LONG_LONG 0x208
#define MPI_LONG_LONG 0x308

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

static inline int mpistub_size_(MPI_Datatype t) {
  if(t > 0x1000)
    return t - 0x1000; /* contiguous types created by MPI_Type_contiguous */
  return t & 0xff;
}

static inline void mpistub_unreachable_(const char * f) {
  std::fprintf(stderr, "mpi stub: %s is unreachable with one rank\n", f);
  std::abort();
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Init_thread(int *, char ***, int, int * p) {
  if(p) *p = MPI_THREAD_MULTIPLE;
  return 0;
}
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) {
  std::fprintf(stderr, "MPI_Abort(%d)\n", code);
  std::abort();
  return 0;
}
static inline int MPI_Comm_rank(MPI_Comm, int * r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int * s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void * s, void * r, int n, MPI_Datatype t,
  MPI_Op, MPI_Comm) {
  if(s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)n * mpistub_size_(t));
  return 0;
}
static inline int MPI_Reduce(const void * s, void * r, int n, MPI_Datatype t,
  MPI_Op, int, MPI_Comm) {
  if(s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)n * mpistub_size_(t));
  return 0;
}
static inline int MPI_Allgather(const void * s, int ns, MPI_Datatype ts, void * r,
  int, MPI_Datatype, MPI_Comm) {
  if(s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)ns * mpistub_size_(ts));
  return 0;
}
static inline int MPI_Gather(const void * s, int ns, MPI_Datatype ts, void * r,
  int, MPI_Datatype, int, MPI_Comm) {
  if(s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)ns * mpistub_size_(ts));
  return 0;
}
static inline int MPI_Allgatherv(const void * s, int ns, MPI_Datatype ts,
  void * r, const int *, const int * displs, MPI_Datatype, MPI_Comm) {
  if(s != MPI_IN_PLACE)
    std::memcpy((char *)r + (size_t)displs[0] * mpistub_size_(ts), s,
      (size_t)ns * mpistub_size_(ts));
  return 0;
}
static inline int MPI_Alltoall(const void * s, int ns, MPI_Datatype ts, void * r,
  int, MPI_Datatype, MPI_Comm) {
  if(s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)ns * mpistub_size_(ts));
  return 0;
}
static inline int MPI_Alltoallv(const void * s, const int * sc, const int * sd,
  MPI_Datatype ts, void * r, const int *, const int * rd, MPI_Datatype,
  MPI_Comm) {
  std::memcpy((char *)r + (size_t)rd[0] * mpistub_size_(ts),
    (const char *)s + (size_t)sd[0] * mpistub_size_(ts),
    (size_t)sc[0] * mpistub_size_(ts));
  return 0;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype * nt) {
  *nt = 0x1000 + n * mpistub_size_(t);
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_Type_free(MPI_Datatype *) { return 0; }
static inline int MPI_Iprobe(int, int, MPI_Comm, int * flag, MPI_Status *) {
  *flag = 0;
  return 0;
}
static inline int MPI_Test(MPI_Request *, int * flag, MPI_Status *) {
  *flag = 1;
  return 0;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Get_count(const MPI_Status *, MPI_Datatype, int * c) {
  *c = 0;
  return 0;
}
static inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *) {
  mpistub_unreachable_("MPI_Probe");
  return 0;
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  mpistub_unreachable_("MPI_Send");
  return 0;
}
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm,
  MPI_Status *) {
  mpistub_unreachable_("MPI_Recv");
  return 0;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm,
  MPI_Request *) {
  mpistub_unreachable_("MPI_Isend");
  return 0;
}
static inline int MPI_Issend(const void *, int, MPI_Datatype, int, int, MPI_Comm,
  MPI_Request *) {
  mpistub_unreachable_("MPI_Issend");
  return 0;
}
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *,
  int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  mpistub_unreachable_("MPI_Sendrecv");
  return 0;
}
