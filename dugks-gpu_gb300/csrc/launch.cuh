// Host-side launchers of the step and auxiliary kernels, one explicit
// instantiation per storage form (kern_fp64.cu, kern_fp32.cu, kern_fp16.cu,
// kern_bf16.cu) so that the four forms compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include "dugks_kernels.cuh"
#include "aux_kernels.cuh"
#include "adjoint_kernels.cuh"

namespace dg {

// Flux-kernel CTA per form: W warps = W-1 rows of 32 cells plus the halo warp.
// TMA selects flux_tma_kernel (f-bar-plus through a TMA-fed shared-memory ring)
// instead of flux_kernel (f-bar-plus through L1).
template <class T, class S>
struct TileCfg {
    static constexpr int W = 8;       // 7 rows of 32 cells
    static constexpr int MINB = 2;    // two CTAs per SM (<= 128 registers)
    static constexpr bool TMA = true; // 4 x 13.7 KB planes per CTA for 16-bit storage
};
template <>
struct TileCfg<float, float> {
    static constexpr int W = 7;       // 6 rows: 4 x 21.9 KB planes, two CTAs per SM
    static constexpr int MINB = 2;
    static constexpr bool TMA = true;
};
template <>
struct TileCfg<double, double> {
    static constexpr int W = 8;       // 7 rows, two CTAs per SM: 128 registers with spills, but 16
    static constexpr int MINB = 2;    // warps per SM keep the FP64 pipe busier (+5 % over one CTA at 255)
    static constexpr bool TMA = false;
};

// tile of the fused adjoint face kernel (TMA forms): W rows of 32 cells, box W+2 rows
template <class T, class S>
struct AdjCfg {
    static constexpr int W = 7;       // 4 x 24.6 KB planes (FP32), two CTAs per SM
    static constexpr int MINB = 2;
};

template <class T, class S>
struct Kern {
    // stage (a) and the x ghost columns of f-bar-plus
    static cudaError_t fbar(const S *f, S *fb, const StepParams<T, S> &P, cudaStream_t st);
    // stages (b)-(e); recon 0 trilinear, 1 central-difference gradient.
    // f_in may equal f_out (in-place update, as the reference).  tmap: the
    // f-bar-plus tensor map of make_tmap (used when TileCfg::TMA).
    static cudaError_t flux(const S *fb, const S *f_in, S *f_out, const StepParams<T, S> &P, int recon,
                            const CUtensorMap *tmap, cudaStream_t st);
    static bool uses_tma() { return TileCfg<T, S>::TMA; }
    // 4-D tensor map (x, y, z, population) over the ghosted f-bar-plus array,
    // box of TmaTile::BXT columns x box_rows rows x 1 plane x 19 populations
    // (forward flux kernel: TileCfg::W + 1 rows; adjoint faces: AdjCfg::W + 2)
    static int make_tmap(const S *fb, int nx, int ny, int nz, int pitch_b, long long ps_b, int box_rows,
                         CUtensorMap *out);
    static cudaError_t macro(const S *f, const StepParams<T, S> &P, double hdt, const double F[3], double *rho,
                             double *ux, double *uy, double *uz, cudaStream_t st);
    static cudaError_t aos_to_soa(const double *src, S *dst, const StepParams<T, S> &P, cudaStream_t st);
    static cudaError_t soa_to_aos(const S *src, double *dst, const StepParams<T, S> &P, cudaStream_t st);
    static cudaError_t stats_partials(const S *f, const StepParams<T, S> &P, double hdt, const double F[3],
                                      double *partial, int nblocks, cudaStream_t st);
    static cudaError_t moments_partials(const S *f, const StepParams<T, S> &P, double *partial, int nblocks,
                                        cudaStream_t st);
    // Adjoint of one step (adjoint_kernels.cuh): recomputes f-bar-plus of f_n into fb,
    // per-face adjoints into lamv (T-typed scratch, adj_nface(0)+2*adj_nface(1) faces x 19),
    // then lam_out = (dS/df)^T lam_next.  FP64 and FP32 forms only.
    // dphi (optional, FP64, dump order [k][j][i]): += dJ/dphi of this step when a force field is set;
    // tmap_adj: f-bar-plus tensor map with AdjCfg::W + 2 rows (TMA forms)
    static cudaError_t adjoint(const S *f_n, S *fb, const S *lam_next, S *lam_out, T *lamv,
                               const StepParams<T, S> &P, double *dphi, const CUtensorMap *tmap_adj,
                               cudaStream_t st);
    static int flux_kchunk(const StepParams<T, S> &P);
};

cudaError_t launch_stats_reduce(const double *partial, int nblocks, int nx, double *total, cudaStream_t st);

// one thread waits `limit` polls on an mbarrier that nothing arrives at, then
// raises *err (kern_fp64.cu); *polled_cycles = SM clock cycles spent waiting
cudaError_t launch_wait_timeout_selftest(int *err, int limit, long long *polled_cycles, cudaStream_t st);

}  // namespace dg
