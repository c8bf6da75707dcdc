/* Minimal single-rank MPI declarations so that the reference's unmodified
 * src/dugks.cu compiles to a device-code cubin (TEST INFRASTRUCTURE ONLY: the
 * cubin is the oracle of the reference's own GPU kernels).  Only the names
 * the reference's headers and host code mention are declared; nothing here is
 * linked or executed. */
#ifndef REF_SHIM_MPI_H
#define REF_SHIM_MPI_H
#define OPEN_MPI 1
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_DOUBLE 1
#define MPI_FLOAT 2
#define MPI_COMM_WORLD 0
#endif
