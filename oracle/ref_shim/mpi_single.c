/* Single-rank bodies of the MPI calls declared in mpi.h (TEST INFRASTRUCTURE
 * ONLY): what one MPI process would see on a one-rank communicator. */
#include <stdio.h>
#include <string.h>
#include <time.h>

#include "mpi.h"

static int g_ndims = 0;
static int g_periods[8];

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }

int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[], int reorder,
                    MPI_Comm *comm_cart)
{
    int d;
    (void)reorder;
    if (ndims < 0 || ndims > 8) return 1;
    for (d = 0; d < ndims; d++) {
        if (dims[d] != 1) return 1; /* one rank: every dimension has one process */
        g_periods[d] = periods[d];
    }
    g_ndims = ndims;
    *comm_cart = comm_old;
    return MPI_SUCCESS;
}

int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[])
{
    int d;
    (void)comm; (void)rank;
    for (d = 0; d < maxdims; d++) coords[d] = 0;
    return MPI_SUCCESS;
}

/* a periodic direction wraps onto this rank; a non-periodic one has no neighbour */
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *rank_source, int *rank_dest)
{
    (void)comm;
    if (direction < 0 || direction >= g_ndims) return 1;
    if (disp == 0 || g_periods[direction]) {
        *rank_source = 0;
        *rank_dest = 0;
    } else {
        *rank_source = MPI_PROC_NULL;
        *rank_dest = MPI_PROC_NULL;
    }
    return MPI_SUCCESS;
}

int MPI_Cart_rank(MPI_Comm comm, const int coords[], int *rank)
{
    (void)comm; (void)coords;
    *rank = 0;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static size_t type_size(MPI_Datatype t) { return t == MPI_FLOAT ? 4 : 8; }

/* point-to-point messages never occur on one rank (the reference skips its own
 * rank in every gather); reaching one is an error */
int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm)
{
    (void)buf; (void)count; (void)datatype; (void)tag; (void)comm;
    if (dest == MPI_PROC_NULL) return MPI_SUCCESS;
    fprintf(stderr, "single-rank MPI: MPI_Send to rank %d\n", dest);
    return 1;
}

int MPI_Recv(void *buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm, MPI_Status *status)
{
    (void)buf; (void)count; (void)datatype; (void)tag; (void)comm; (void)status;
    if (source == MPI_PROC_NULL) return MPI_SUCCESS;
    fprintf(stderr, "single-rank MPI: MPI_Recv from rank %d\n", source);
    return 1;
}

/* the halo exchange with itself: the send buffer lands in the receive buffer */
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag, void *recvbuf,
                 int recvcount, MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm, MPI_Status *status)
{
    (void)sendtag; (void)recvtag; (void)comm; (void)status;
    if (dest == MPI_PROC_NULL || source == MPI_PROC_NULL) return MPI_SUCCESS;
    if (sendcount != recvcount || sendtype != recvtype) return 1;
    memmove(recvbuf, sendbuf, (size_t)sendcount * type_size(sendtype));
    return MPI_SUCCESS;
}
