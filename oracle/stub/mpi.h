/* Single-rank stand-in for <mpi.h>, used only to compile the reference
 * unbinding sources (test infrastructure; never linked into the product).
 *
 * Every communicator has one rank.  Collectives copy the send buffer to the
 * receive buffer where the reference relies on that (Allreduce, Allgather,
 * Bcast is a no-op); everything else does nothing and returns MPI_SUCCESS.
 * Datatype handles carry their element size so that copies have the right
 * length.  This is the project's own header, written for a one-process
 * build; it declares only what the unbinding translation units name. */
#ifndef HBTG_ORACLE_STUB_MPI_H
#define HBTG_ORACLE_STUB_MPI_H

#include <stddef.h>
#include <string.h>

typedef int MPI_Comm;
typedef long MPI_Datatype; /* element size in bytes (0 = opaque) */
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef struct
{
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_BOTTOM ((void *)0)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_LONG ((MPI_Datatype)8)
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_LONG_INT ((MPI_Datatype)16)
#define MPI_DATATYPE_NULL ((MPI_Datatype)0)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Finalized(int *flag) { *flag = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_split_type(MPI_Comm c, int, int, MPI_Info, MPI_Comm *out) { *out = c; return MPI_SUCCESS; }
static inline int MPI_Get_processor_name(char *name, int *len)
{
  strcpy(name, "localhost");
  *len = 9;
  return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm, int) { return MPI_SUCCESS; }

static inline size_t hbtg_stub_bytes(int count, MPI_Datatype t) { return (size_t)count * (size_t)(t > 0 ? t : 0); }

static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
  if (s != MPI_IN_PLACE && s != r)
    memcpy(r, s, hbtg_stub_bytes(n, t));
  return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm)
{
  if (s != MPI_IN_PLACE && s != r)
    memcpy(r, s, hbtg_stub_bytes(n, t));
  return MPI_SUCCESS;
}
static inline int MPI_Alltoall(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm)
{
  if (s != MPI_IN_PLACE && s != r)
    memcpy(r, s, hbtg_stub_bytes(n, t));
  return MPI_SUCCESS;
}
static inline int MPI_Alltoallv(const void *, const int *, const int *, MPI_Datatype, void *, const int *, const int *,
                                MPI_Datatype, MPI_Comm)
{
  return MPI_SUCCESS;
}
static inline int MPI_Alltoallw(const void *, const int *, const int *, const MPI_Datatype *, void *, const int *,
                                const int *, const MPI_Datatype *, MPI_Comm)
{
  return MPI_SUCCESS;
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int, MPI_Comm,
                               MPI_Status *)
{
  return MPI_SUCCESS;
}
static inline int MPI_Get_address(const void *p, MPI_Aint *a) { *a = (MPI_Aint)p; return MPI_SUCCESS; }
static inline int MPI_Type_create_struct(int, const int *, const MPI_Aint *, const MPI_Datatype *, MPI_Datatype *t)
{
  *t = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Type_create_resized(MPI_Datatype, MPI_Aint, MPI_Aint ext, MPI_Datatype *t)
{
  *t = (MPI_Datatype)ext;
  return MPI_SUCCESS;
}
static inline int MPI_Type_create_hindexed(int, const int *, const MPI_Aint *, MPI_Datatype, MPI_Datatype *t)
{
  *t = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype o, MPI_Datatype *t) { *t = n * o; return MPI_SUCCESS; }
static inline int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *ext)
{
  *lb = 0;
  *ext = t;
  return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }

#endif
