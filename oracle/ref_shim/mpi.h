/* Single-rank MPI for building the reference's unmodified sources (TEST
 * INFRASTRUCTURE ONLY).  Declares the names the reference's host code uses;
 * mpi_single.c gives them single-rank bodies: one process, rank 0, a
 * Cartesian topology whose periodic directions are their own neighbours and
 * whose walls are MPI_PROC_NULL, and self-exchanges as copies.  Used for the
 * reference's kernels (compiled to cubins) and for the reference's own driver
 * and I/O (src/main.cu, output.cu, parallel.cu, ...) linked against the
 * legacy-name library. */
#ifndef REF_SHIM_MPI_H
#define REF_SHIM_MPI_H
#define OPEN_MPI 1
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_SUCCESS 0
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_DOUBLE 1
#define MPI_FLOAT 2
#define MPI_COMM_WORLD 0

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[], int reorder,
                    MPI_Comm *comm_cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *rank_source, int *rank_dest);
int MPI_Cart_rank(MPI_Comm comm, const int coords[], int *rank);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm, MPI_Status *status);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag, void *recvbuf,
                 int recvcount, MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm, MPI_Status *status);
#ifdef __cplusplus
}
#endif
#endif
