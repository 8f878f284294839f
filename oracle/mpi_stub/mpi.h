/* Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * sources into the oracle library (oracle/_ref).  It provides exactly what
 * those translation units name: the MPI_Allreduce that compute_global_bbox
 * calls (src/bounding_box.cpp:46-52), the gathers and all-to-alls of
 * src/exchange.cpp and the MPI_Reduce of computeDistanceSum
 * (src/io.cpp:776).  On one rank each copies the send buffer into the
 * receive buffer (at the first displacement).  A datatype's value is its
 * size in bytes.  No other MPI behaviour is modelled.  Test infrastructure
 * only. */
#pragma once
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
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

static inline int MPI_Allgather(const void* send, int scount, MPI_Datatype stype, void* recv, int rcount,
                                MPI_Datatype rtype, MPI_Comm comm)
{
    (void)rcount; (void)rtype; (void)comm;
    memcpy(recv, send, (size_t)scount * (size_t)stype);
    return 0;
}

static inline int MPI_Allgatherv(const void* send, int scount, MPI_Datatype stype, void* recv, const int* rcounts,
                                 const int* displs, MPI_Datatype rtype, MPI_Comm comm)
{
    (void)rcounts; (void)comm;
    memcpy((char*)recv + (size_t)displs[0] * (size_t)rtype, send, (size_t)scount * (size_t)stype);
    return 0;
}

static inline int MPI_Alltoall(const void* send, int scount, MPI_Datatype stype, void* recv, int rcount,
                               MPI_Datatype rtype, MPI_Comm comm)
{
    (void)rcount; (void)rtype; (void)comm;
    memcpy(recv, send, (size_t)scount * (size_t)stype);
    return 0;
}

static inline int MPI_Alltoallv(const void* send, const int* scounts, const int* sdispls, MPI_Datatype stype,
                                void* recv, const int* rcounts, const int* rdispls, MPI_Datatype rtype, MPI_Comm comm)
{
    (void)rcounts; (void)comm;
    memcpy((char*)recv + (size_t)rdispls[0] * (size_t)rtype, (const char*)send + (size_t)sdispls[0] * (size_t)stype,
           (size_t)scounts[0] * (size_t)stype);
    return 0;
}

static inline int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, int root,
                             MPI_Comm comm)
{
    (void)op; (void)root; (void)comm;
    memcpy(recv, send, (size_t)count * (size_t)type);
    return 0;
}
