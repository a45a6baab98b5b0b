/*
 * Single-rank MPI stand-in used ONLY to compile the reference solver's own
 * routine sources (ricklee209/Channel_Flow) into the CPU oracle library
 * under oracle/_ref/.  Test infrastructure, never linked into the product.
 *
 * Semantics for a communicator of size 1:
 *   - MPI_Sendrecv with MPI_PROC_NULL on both sides is a no-op; with rank 0
 *     (self) on both sides it copies the send buffer into the receive buffer,
 *     which is what a real MPI does for a self-message.
 *   - MPI_Reduce / MPI_Allreduce (MPI_SUM) copy the single contribution.
 *   - MPI_Send / MPI_Recv to self are unsupported (only Output.cpp uses them
 *     for ranks != 0, which never happens with one rank).
 * stdio.h is included because Driven_force.cpp and Flux_Y_limiter.cpp call
 * printf without including it themselves.
 */
#ifndef CF_ORACLE_MPI_STANDIN_H
#define CF_ORACLE_MPI_STANDIN_H

#include <stdio.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 1
#define MPI_PROC_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }

static inline int MPI_Sendrecv(void *sbuf, int scount, MPI_Datatype stype, int dest, int,
                               void *rbuf, int rcount, MPI_Datatype rtype, int source, int,
                               MPI_Comm, MPI_Status *)
{
    if (dest == 0 && source == 0 && sbuf != rbuf) {
        int n = scount < rcount ? scount : rcount;
        memmove(rbuf, sbuf, (size_t)n * (size_t)(stype < rtype ? stype : rtype));
    }
    return 0;
}

static inline int MPI_Allreduce(void *s, void *r, int count, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (s != r) memmove(r, s, (size_t)count * (size_t)t);
    return 0;
}

static inline int MPI_Reduce(void *s, void *r, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    if (s != r) memmove(r, s, (size_t)count * (size_t)t);
    return 0;
}

static inline int MPI_Send(void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }

#endif
