/* Single-rank stand-in for Open MPI's extension header (test infrastructure). */
#define MPIX_CUDA_AWARE_SUPPORT 1
