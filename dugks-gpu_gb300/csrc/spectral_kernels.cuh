// Spectral statistics of a periodic box: the decaying-turbulence statistics of
// the reference's Fortran code (src/fortran/dhit/src/stat.f90:5-205), on the
// device with cuFFT.  Velocity u = j / rho per cell (src/fortran/dhit/src/
// main.cuf:86-103, no force shift), its 3-D DFT, the shell spectrum and
// dissipation spectrum, and the skewness / flatness of the longitudinal
// velocity derivatives.  All arithmetic in FP64 (the reference keeps the
// velocity, spectra and sums in single precision around double FFTs).
//
// Layouts: complex fields in dense x-fastest order t = (k ny + j) nx + i.
#pragma once
#include <cuda_runtime.h>

#include "dugks_kernels.cuh"

namespace dg {

// Signed integer frequency of FFT index i0 (0-based) on n points: i0 for
// i0 < n/2, else i0 - n (the kx array of src/fortran/dhit/src/stat.f90:85-106).
__host__ __device__ inline int spec_freq(int i0, int n) { return i0 < n / 2 ? i0 : i0 - n; }

// Block-partial sums of a[0..NA-1] over the block's threads: warp shuffles,
// then warp 0 over the warps (fixed order, deterministic).
template <int NA>
__device__ __forceinline__ void spec_block_partials(double a[NA], double *partial)
{
    __shared__ double red[32][NA];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int m = 0; m < NA; ++m) {
        double v = a[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][m] = v;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int m = 0; m < NA; ++m) {
            double v = lane < nw ? red[lane][m] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) partial[blockIdx.x * NA + m] = v;
        }
    }
}

// u = j / rho of every cell into the real parts of U, V, W (imaginary parts
// zero); block partials of sum |u|^2 (the kinetic energy before the mean is
// removed, stat.f90:60).
template <class T, class S>
__global__ void __launch_bounds__(256) spec_velocity_kernel(const S *__restrict__ f, const StepParams<T, S> P,
                                                            double2 *__restrict__ U, double2 *__restrict__ V,
                                                            double2 *__restrict__ W, double *__restrict__ partial)
{
    const long long n = (long long)P.nx * P.ny * P.nz;
    double a[1] = {0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long row = t / P.nx;
        const long long c = row * P.pitch + (t - row * P.nx);
        double v[NPOP];
#pragma unroll
        for (int p = 0; p < NPOP; ++p) v[p] = double(P.codec.load_nc(f, p * P.ps + c, p));
        double r, jx, jy, jz;
        moments(v, r, jx, jy, jz);
        const double u = jx / r, vv = jy / r, w = jz / r;
        U[t] = make_double2(u, 0.0);
        V[t] = make_double2(vv, 0.0);
        W[t] = make_double2(w, 0.0);
        a[0] += u * u + vv * vv + w * w;
    }
    spec_block_partials<1>(a, partial);
}

// After the forward transforms: scale by 1/N, remove the mean (mode 0), the
// energy and dissipation densities per mode (stat.f90:127-132), then the
// longitudinal derivatives' spectra i kx u^, i ky v^, i kz w^ (stat.f90:176-178)
// in place for the inverse transforms.
__global__ void __launch_bounds__(256) spec_modes_kernel(double2 *__restrict__ U, double2 *__restrict__ V,
                                                         double2 *__restrict__ W, double *__restrict__ ET,
                                                         double *__restrict__ ETS, int nx, int ny, int nz,
                                                         double inv_n, double kscale, double two_nu)
{
    const long long n = (long long)nx * ny * nz;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long row = t / nx;
        const int i = int(t - row * nx), j = int(row % ny), k = int(row / ny);
        const double kx = kscale * spec_freq(i, nx), ky = kscale * spec_freq(j, ny), kz = kscale * spec_freq(k, nz);
        double2 u = U[t], v = V[t], w = W[t];
        if (t == 0) u = v = w = make_double2(0.0, 0.0);
        u.x *= inv_n; u.y *= inv_n;
        v.x *= inv_n; v.y *= inv_n;
        w.x *= inv_n; w.y *= inv_n;
        const double et = 0.5 * (u.x * u.x + u.y * u.y + v.x * v.x + v.y * v.y + w.x * w.x + w.y * w.y);
        ET[t] = et;
        ETS[t] = two_nu * et * (kx * kx + ky * ky + kz * kz);
        U[t] = make_double2(-kx * u.y, kx * u.x);
        V[t] = make_double2(-ky * v.y, ky * v.x);
        W[t] = make_double2(-kz * w.y, kz * w.x);
    }
}

// Block partials of sum d^2, d^3, d^4 over the real parts of the three
// derivative fields (stat.f90:186-190).
__global__ void __launch_bounds__(256) spec_deriv_moments_kernel(const double2 *__restrict__ U,
                                                                 const double2 *__restrict__ V,
                                                                 const double2 *__restrict__ W, long long n,
                                                                 double *__restrict__ partial)
{
    double a[3] = {0.0, 0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double d[3] = {U[t].x, V[t].x, W[t].x};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double d2 = d[q] * d[q];
            a[0] += d2;
            a[1] += d2 * d[q];
            a[2] += d2 * d2;
        }
    }
    spec_block_partials<3>(a, partial);
}

// Shell sums (stat.f90:142-151): block b adds the modes of shell b, listed in
// order[off[b] .. off[b+1]) (ascending mode index), in a fixed order.
__global__ void __launch_bounds__(256) spec_shell_kernel(const double *__restrict__ ET, const double *__restrict__ ETS,
                                                         const int *__restrict__ order, const int *__restrict__ off,
                                                         double *__restrict__ shells)
{
    const int b = blockIdx.x;
    double a[2] = {0.0, 0.0};
    for (int q = off[b] + threadIdx.x; q < off[b + 1]; q += blockDim.x) {
        const int t = order[q];
        a[0] += ET[t];
        a[1] += ETS[t];
    }
    spec_block_partials<2>(a, shells);
}

}  // namespace dg
