// Auxiliary kernels: state transposes between the host dump order and the
// device SoA storage, deterministic statistics partial sums, conserved
// moments.  Templated on arithmetic type T and storage type S like the step.
#pragma once
#include "dugks_kernels.cuh"

namespace dg {

// dump order f[((k*ny+j)*nx+i)*19+p] (double)  ->  SoA storage
template <class T, class S>
__global__ void __launch_bounds__(256) aos_to_soa_kernel(const double *__restrict__ src, S *__restrict__ dst,
                                                         const StepParams<T, S> P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= P.nx) return;
    const size_t cell = ((size_t)k * P.ny + j) * P.nx + i;
    const long long c = ((long long)k * P.ny + j) * P.pitch + i;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) P.codec.store(dst, p * P.ps + c, p, T(src[cell * NPOP + p]));
}

// SoA storage -> dump order (double)
template <class T, class S>
__global__ void __launch_bounds__(256) soa_to_aos_kernel(const S *__restrict__ src, double *__restrict__ dst,
                                                         const StepParams<T, S> P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, k = blockIdx.z;
    if (i >= P.nx) return;
    const size_t cell = ((size_t)k * P.ny + j) * P.nx + i;
    const long long c = ((long long)k * P.ny + j) * P.pitch + i;
#pragma unroll
    for (int p = 0; p < NPOP; ++p) dst[cell * NPOP + p] = double(P.codec.load_nc(src, p * P.ps + c, p));
}

// Number of FP64 partial sums per x index written by stats_partials_kernel:
//  0 rho, 1 u, 2 v, 3 w, 4 uw, 5 uv, 6 vw, 7 uu, 8 vv, 9 ww,
//  10..13 min rho,u,v,w, 14..17 max rho,u,v,w, 18 non-finite count
constexpr int NSTAT = 19;

// Block (b, by) sums rows (j,k) = b, b+gridDim.x, ... ; thread owns x index
// i = by*blockDim.x + threadIdx.x.  Output partial[b][i][NSTAT].  The fixed assignment and
// the ordered second pass make the result independent of scheduling.
template <class T, class S>
__global__ void __launch_bounds__(1024) stats_partials_kernel(const S *__restrict__ f, const StepParams<T, S> P,
                                                              double hdt, double fxa, double fya, double fza,
                                                              double *__restrict__ partial)
{
    const int i = blockIdx.y * blockDim.x + threadIdx.x;
    if (i >= P.nx) return;
    double acc[NSTAT];
#pragma unroll
    for (int s = 0; s < 10; ++s) acc[s] = 0.0;
#pragma unroll
    for (int s = 10; s < 14; ++s) acc[s] = 1e300;
#pragma unroll
    for (int s = 14; s < 18; ++s) acc[s] = -1e300;
    acc[18] = 0.0;
    const int rows = P.ny * P.nz;
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const long long c = (long long)row * P.pitch + i;
        double v[NPOP];
#pragma unroll
        for (int p = 0; p < NPOP; ++p) v[p] = double(P.codec.load_nc(f, p * P.ps + c, p));
        double r, jx, jy, jz;
        moments(v, r, jx, jy, jz);
        const double u = jx / r + fxa * hdt, vv = jy / r + fya * hdt, w = jz / r + fza * hdt;
        if (!isfinite(r) || !isfinite(u) || !isfinite(vv) || !isfinite(w)) acc[18] += 1.0;
        acc[0] += r; acc[1] += u; acc[2] += vv; acc[3] += w;
        acc[4] += u * w; acc[5] += u * vv; acc[6] += vv * w;
        acc[7] += u * u; acc[8] += vv * vv; acc[9] += w * w;
        acc[10] = fmin(acc[10], r); acc[11] = fmin(acc[11], u); acc[12] = fmin(acc[12], vv); acc[13] = fmin(acc[13], w);
        acc[14] = fmax(acc[14], r); acc[15] = fmax(acc[15], u); acc[16] = fmax(acc[16], vv); acc[17] = fmax(acc[17], w);
    }
    double *out = partial + ((size_t)blockIdx.x * P.nx + i) * NSTAT;
#pragma unroll
    for (int s = 0; s < NSTAT; ++s) out[s] = acc[s];
}

// Ordered reduction over blocks of the statistics partials of x index i:
// acc[s] = sum / min / max over b of partial[b][i][s] (b ascending).  Shared by
// stats_reduce_kernel and the allocation-free statistics, so that both give
// the same numbers.
__device__ __forceinline__ void stats_combine_blocks(const double *__restrict__ partial, int nblocks, int nx, int i,
                                                     double acc[NSTAT])
{
    for (int s = 0; s < NSTAT; ++s) acc[s] = partial[size_t(i) * NSTAT + s];
    for (int b = 1; b < nblocks; ++b) {
        const double *q = partial + (size_t(b) * nx + i) * NSTAT;
        for (int s = 0; s < 10; ++s) acc[s] += q[s];
        for (int s = 10; s < 14; ++s) acc[s] = fmin(acc[s], q[s]);
        for (int s = 14; s < 18; ++s) acc[s] = fmax(acc[s], q[s]);
        acc[18] += q[18];
    }
}

// Ordered reduction over blocks: total[i][s] = sum/min/max over b of partial[b][i][s].
__global__ void stats_reduce_kernel(const double *__restrict__ partial, int nblocks, int nx, double *__restrict__ total);
// acc[i][s] += total[i][s] for the 10 sums
__global__ void stats_accumulate_kernel(const double *__restrict__ total, int nx, double *__restrict__ acc);

// Conserved moments: block partial sums of (rho, jx, jy, jz) over cells; a
// fixed assignment of cells to threads and a fixed-order tree make the sums
// reproducible.
// Warp-shuffle sum of a double over the 32 lanes (fixed order: deterministic).
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Mass and momentum partial sums, one per block (deterministic order).  Every
// thread takes cells t, t + gridDim.x*blockDim.x, ... of the interior in x-fastest
// order (coalesced).  FP64 form: one FP64 sum per population over the thread's
// cells, combined into (rho, j) at the end: 19 additions per cell instead of
// the per-cell moments (46) plus four accumulations, on GB300's reduced-rate
// FP64 pipe.  Other forms: moments per cell in the arithmetic type, summed over
// cells in FP64.  Warps reduce with shuffles, warp 0 combines the warps.
template <class T, class S>
__global__ void __launch_bounds__(256) moments_partials_kernel(const S *__restrict__ f, const StepParams<T, S> P,
                                                               double *__restrict__ partial)
{
    __shared__ double red[8][4];
    double a[4] = {0, 0, 0, 0};
    const long long ncell = (long long)P.nx * P.ny * P.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (sizeof(T) == 8) {
        double sp[NPOP];
#pragma unroll
        for (int p = 0; p < NPOP; ++p) sp[p] = 0.0;
        for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ncell; t += stride) {
            const long long row = t / P.nx;
            const long long c = row * P.pitch + (t - row * P.nx);
#pragma unroll
            for (int p = 0; p < NPOP; ++p) sp[p] += double(P.codec.load_nc(f, p * P.ps + c, p));
        }
#pragma unroll
        for (int p = 0; p < NPOP; ++p) {
            a[0] += sp[p];
            if (cx(p)) a[1] += cx(p) > 0 ? sp[p] : -sp[p];
            if (cy(p)) a[2] += cy(p) > 0 ? sp[p] : -sp[p];
            if (cz(p)) a[3] += cz(p) > 0 ? sp[p] : -sp[p];
        }
    } else {
        for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ncell; t += stride) {
            const long long row = t / P.nx;
            const long long c = row * P.pitch + (t - row * P.nx);
            T v[NPOP];
#pragma unroll
            for (int p = 0; p < NPOP; ++p) v[p] = P.codec.load_nc(f, p * P.ps + c, p);
            T r, jx, jy, jz;
            moments(v, r, jx, jy, jz);
            a[0] += double(r); a[1] += double(jx); a[2] += double(jy); a[3] += double(jz);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const double s = warp_sum(a[m]);
        if (lane == 0) red[warp][m] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const double s = warp_sum(lane < 8 ? red[lane][m] : 0.0);
            if (lane == 0) partial[blockIdx.x * 4 + m] = s;
        }
    }
}

}  // namespace dg
