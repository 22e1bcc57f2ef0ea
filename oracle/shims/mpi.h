/* Single-rank MPI stand-in used only to compile the reference solver's
 * serial path as a test oracle.  Every call behaves as on a one-process
 * communicator: rank 0, size 1, collectives copy send to receive, and
 * point-to-point calls are never reached on the serial path. */
#pragma once
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Info;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Init(void*, void*) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
  memcpy(r, s, (size_t)sc * (size_t)st); return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* q) { *q = 0; return 0; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* q) { *q = 0; return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
typedef int MPI_Op;
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
/* one rank: the reduction of one contribution is that contribution */
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  memcpy(r, s, (size_t)n * (size_t)t); return 0; }
