/*
 * mpi.h — single-rank MPI stand-in used ONLY to compile the reference
 * solvers (MPI_REAL/*.c of YaphetS-jx/Linear-Solver) into the CPU checker
 * under oracle/_ref/.  Test infrastructure, never part of the product.
 *
 * It provides exactly the MPI names those sources use (MPI_REAL/system.c:94,
 * 134-135, 324, 378-382, 462, 539-540; tools.c:25,42; AAR.c:48,89,212;
 * PGR.c:206; PL2R.c:206; CG.c:38,53-54; main.c:21-23,111,115) with the
 * semantics of a one-process world: every reduction is the identity, the
 * Cartesian topology is a 1x1x1 periodic grid and no neighbour exchange is
 * ever issued (Lap_Vec_mult takes its sequential branch when size == 1).
 */
#ifndef ORACLE_MPI_SHIM_H
#define ORACLE_MPI_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_NULL      ((MPI_Comm)0)
#define MPI_COMM_WORLD     ((MPI_Comm)1)
#define MPI_DOUBLE         ((MPI_Datatype)8)
#define MPI_INT            ((MPI_Datatype)4)
#define MPI_SUM            ((MPI_Op)1)
#define MPI_INFO_NULL      ((MPI_Info)0)
#define MPI_IN_PLACE       ((void *)-1)
#define MPI_UNWEIGHTED     ((int *)2)
#define MPI_STATUS_IGNORE  ((MPI_Status *)0)
#define MPI_SUCCESS        0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type,
                  MPI_Op op, MPI_Comm comm);
int MPI_Dims_create(int nnodes, int ndims, int dims[]);
int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[], const int periods[],
                    int reorder, MPI_Comm *cart);
int MPI_Cart_coords(MPI_Comm cart, int rank, int maxdims, int coords[]);
int MPI_Cart_rank(MPI_Comm cart, const int coords[], int *rank);
int MPI_Dist_graph_create_adjacent(MPI_Comm old, int indegree, const int sources[],
                                   const int sourceweights[], int outdegree,
                                   const int destinations[], const int destweights[],
                                   MPI_Info info, int reorder, MPI_Comm *graph);
int MPI_Ineighbor_alltoallv(const void *sendbuf, const int sendcounts[], const int sdispls[],
                            MPI_Datatype sendtype, void *recvbuf, const int recvcounts[],
                            const int rdispls[], MPI_Datatype recvtype, MPI_Comm comm,
                            MPI_Request *request);
int MPI_Wait(MPI_Request *request, MPI_Status *status);

#ifdef __cplusplus
}
#endif
#endif
