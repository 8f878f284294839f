/* Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * hot-path sources into the oracle library (oracle/_ref).  It provides exactly
 * what those translation units name: the MPI_Allreduce that
 * compute_global_bbox calls (src/bounding_box.cpp:46-52), which on one rank
 * copies the send buffer into the receive buffer.  No other MPI behaviour is
 * modelled.  Test infrastructure only. */
#pragma once
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

static inline int MPI_Allreduce(const void* send, void* recv, int count,
                                MPI_Datatype type, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    memcpy(recv, send, (size_t)count * (size_t)type);
    return 0;
}
