// Host-side launchers of the step and auxiliary kernels, one explicit
// instantiation per storage form (kern_fp64.cu, kern_fp32.cu, kern_fp16.cu,
// kern_bf16.cu) so that the four forms compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include "dugks_kernels.cuh"
#include "aux_kernels.cuh"

namespace dg {

// Flux-kernel tile per form: BX x BY cells, NT threads.
template <class T, class S>
struct TileCfg {
    static constexpr int BX = 32, BY = 4, NT = 128;
};
template <>
struct TileCfg<double, double> {
    static constexpr int BX = 32, BY = 4, NT = 128;
};

template <class T, class S>
struct Kern {
    static cudaError_t fbar(const S *f, S *fb, const StepParams<T, S> &P, cudaStream_t st);
    // f_in may equal f_out (in-place update, as the reference)
    static cudaError_t flux(const S *fb, const S *f_in, S *f_out, const StepParams<T, S> &P, cudaStream_t st);
    static cudaError_t macro(const S *f, const StepParams<T, S> &P, double hdt, const double F[3], double *rho,
                             double *ux, double *uy, double *uz, cudaStream_t st);
    static cudaError_t aos_to_soa(const double *src, S *dst, const StepParams<T, S> &P, cudaStream_t st);
    static cudaError_t soa_to_aos(const S *src, double *dst, const StepParams<T, S> &P, cudaStream_t st);
    static cudaError_t stats_partials(const S *f, const StepParams<T, S> &P, double hdt, const double F[3],
                                      double *partial, int nblocks, cudaStream_t st);
    static cudaError_t moments_partials(const S *f, const StepParams<T, S> &P, double *partial, int nblocks,
                                        cudaStream_t st);
    static size_t flux_smem_bytes();
    static int flux_kchunk(const StepParams<T, S> &P);
};

cudaError_t launch_stats_reduce(const double *partial, int nblocks, int nx, double *total, cudaStream_t st);

}  // namespace dg
