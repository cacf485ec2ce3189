/*
 * mpi_shim.c — one-process implementation of the MPI calls listed in
 * mpi_shim/mpi.h.  Test infrastructure: it exists so that the reference's
 * MPI_REAL solvers can be compiled and run here, unmodified, as the checker
 * that pins the CPU oracle.  With one rank the reference never reaches the
 * halo-exchange branch of Lap_Vec_mult (MPI_REAL/system.c:106 tests size > 1),
 * so MPI_Ineighbor_alltoallv only has to reject being called.
 */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static size_t type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm *comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
    return MPI_SUCCESS;
}

int MPI_Dims_create(int nnodes, int ndims, int dims[])
{
    for (int i = 0; i < ndims; i++) if (dims[i] == 0) dims[i] = 1;
    return nnodes == 1 ? MPI_SUCCESS : 1;
}

int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[], const int periods[],
                    int reorder, MPI_Comm *cart)
{
    (void)old; (void)ndims; (void)dims; (void)periods; (void)reorder;
    *cart = 2;
    return MPI_SUCCESS;
}

int MPI_Cart_coords(MPI_Comm cart, int rank, int maxdims, int coords[])
{
    (void)cart; (void)rank;
    for (int i = 0; i < maxdims; i++) coords[i] = 0;
    return MPI_SUCCESS;
}

int MPI_Cart_rank(MPI_Comm cart, const int coords[], int *rank)
{
    (void)cart; (void)coords; *rank = 0;
    return MPI_SUCCESS;
}

int MPI_Dist_graph_create_adjacent(MPI_Comm old, int indegree, const int sources[],
                                   const int sourceweights[], int outdegree,
                                   const int destinations[], const int destweights[],
                                   MPI_Info info, int reorder, MPI_Comm *graph)
{
    (void)old; (void)indegree; (void)sources; (void)sourceweights; (void)outdegree;
    (void)destinations; (void)destweights; (void)info; (void)reorder;
    *graph = 3;
    return MPI_SUCCESS;
}

int MPI_Ineighbor_alltoallv(const void *sendbuf, const int sendcounts[], const int sdispls[],
                            MPI_Datatype sendtype, void *recvbuf, const int recvcounts[],
                            const int rdispls[], MPI_Datatype recvtype, MPI_Comm comm,
                            MPI_Request *request)
{
    (void)sendbuf; (void)sendcounts; (void)sdispls; (void)sendtype; (void)recvbuf;
    (void)recvcounts; (void)rdispls; (void)recvtype; (void)comm; (void)request;
    fprintf(stderr, "mpi_shim: neighbour exchange requested in a one-rank world\n");
    abort();
}

int MPI_Wait(MPI_Request *request, MPI_Status *status)
{
    (void)request; (void)status;
    return MPI_SUCCESS;
}
