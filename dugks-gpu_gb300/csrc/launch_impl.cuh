// Template bodies of the launchers declared in launch.cuh.
#pragma once
#include <algorithm>
#include "launch.cuh"

namespace dg {

template <class T, class S>
cudaError_t Kern<T, S>::fbar(const S *f, S *fb, const StepParams<T, S> &P, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    fbar_kernel<T, S><<<grid, bx, 0, st>>>(f, fb, P);
    return cudaGetLastError();
}

template <class T, class S>
size_t Kern<T, S>::flux_smem_bytes()
{
    using C = TileCfg<T, S>;
    return FluxTile<T, C::BX, C::BY>::bytes;
}

template <class T, class S>
int Kern<T, S>::flux_kchunk(const StepParams<T, S> &P)
{
    using C = TileCfg<T, S>;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, flux_kernel<T, S, C::BX, C::BY, C::NT>, C::NT,
                                                  flux_smem_bytes());
    occ = std::max(occ, 1);
    const long long cols = (long long)((P.nx + C::BX - 1) / C::BX) * ((P.ny + C::BY - 1) / C::BY);
    const long long want = 4LL * sms * occ;
    long long nchunks = (want + cols - 1) / cols;
    nchunks = std::max(1LL, std::min<long long>(nchunks, P.nz));
    // at least 4 planes per chunk keeps the halo-plane overhead below 50 %
    nchunks = std::min<long long>(nchunks, std::max(1, P.nz / 4));
    return int((P.nz + nchunks - 1) / nchunks);
}

template <class T, class S>
cudaError_t Kern<T, S>::flux(const S *fb, const S *f_in, S *f_out, const StepParams<T, S> &P, cudaStream_t st)
{
    using C = TileCfg<T, S>;
    auto kern = flux_kernel<T, S, C::BX, C::BY, C::NT>;
    const size_t smem = flux_smem_bytes();
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int kchunk = flux_kchunk(P);
    dim3 grid((P.nx + C::BX - 1) / C::BX, (P.ny + C::BY - 1) / C::BY, (P.nz + kchunk - 1) / kchunk);
    kern<<<grid, C::NT, smem, st>>>(fb, f_in, f_out, P, kchunk);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::macro(const S *f, const StepParams<T, S> &P, double hdt, const double F[3], double *rho,
                              double *ux, double *uy, double *uz, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    macro_kernel<T, S><<<grid, bx, 0, st>>>(f, P, hdt, F[0], F[1], F[2], rho, ux, uy, uz);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::aos_to_soa(const double *src, S *dst, const StepParams<T, S> &P, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    aos_to_soa_kernel<T, S><<<grid, bx, 0, st>>>(src, dst, P);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::soa_to_aos(const S *src, double *dst, const StepParams<T, S> &P, cudaStream_t st)
{
    const int bx = P.nx >= 128 ? 128 : ((P.nx + 31) / 32) * 32;
    dim3 grid((P.nx + bx - 1) / bx, P.ny, P.nz);
    soa_to_aos_kernel<T, S><<<grid, bx, 0, st>>>(src, dst, P);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::stats_partials(const S *f, const StepParams<T, S> &P, double hdt, const double F[3],
                                       double *partial, int nblocks, cudaStream_t st)
{
    const int bx = P.nx >= 256 ? 256 : ((P.nx + 31) / 32) * 32;
    dim3 grid(nblocks, (P.nx + bx - 1) / bx);
    stats_partials_kernel<T, S><<<grid, bx, 0, st>>>(f, P, hdt, F[0], F[1], F[2], partial);
    return cudaGetLastError();
}

template <class T, class S>
cudaError_t Kern<T, S>::moments_partials(const S *f, const StepParams<T, S> &P, double *partial, int nblocks,
                                         cudaStream_t st)
{
    moments_partials_kernel<T, S><<<nblocks, 256, 0, st>>>(f, P, partial);
    return cudaGetLastError();
}

}  // namespace dg
