// Allocation-free statistics entry point.
//
// dg_stats_values (engine.cu) reduces the diag.dat / profiles-2.dat statistics
// through a scratch buffer that the handle allocates with cudaMalloc on first
// use.  Some callers cannot allocate device memory at the point where they
// want statistics: host programs that hand all device memory to their own
// pool or arena up front and forbid later allocations, and callers whose
// memory budget the state arrays have already spent.  For them this file
// provides dg_stats_values_noalloc: the same reduction over an FP64 state that
// the caller holds in device memory, with its scratch in a fixed
// file-scope __device__ array instead of an allocation.
//
// The scratch array is sized for nx <= DG_NOALLOC_MAX_NX x-indices; it is part
// of the library's device image, so every GPU that loads the library holds it
// (about 5 MB) until the process exits.  All calls share it: calls whose
// kernels overlap on the GPU (different streams without ordering, or several
// host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/dugks_gb300.h"
#include "aux_kernels.cuh"

namespace {

constexpr int kMaxNx = DG_NOALLOC_MAX_NX;
constexpr int kBlocks = 64;                       // row blocks of the first pass
constexpr size_t kPartial = size_t(kBlocks) * kMaxNx * dg::NSTAT;
constexpr size_t kTotal = size_t(kMaxNx) * dg::NSTAT;

// partial[kBlocks][nx][NSTAT] followed by total[nx][NSTAT]; every call writes
// every entry it later reads, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_stats_scratch[kPartial + kTotal];

constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;
// fixed-size message buffer: the error path allocates nothing either
thread_local char g_noalloc_error[256];

int fail(int code, const char *msg)
{
    std::snprintf(g_noalloc_error, sizeof(g_noalloc_error), "%s", msg);
    return code;
}

// Device address of the scratch array on the current device, resolved once per
// device with that device current.
int scratch_for_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(DG_ERR_ARG, "device ordinal beyond the supported range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_stats_scratch);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_ptr[dev];
    return DG_OK;
}

// One thread per x index: totals over the row blocks, then the profile row
// of src/output.cu:279-323 (plane averages, covariances, variances).
__global__ void noalloc_reduce_kernel(const double *__restrict__ partial, int nblocks, int nx, int nyz,
                                      double *__restrict__ total, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    double acc[dg::NSTAT];
    dg::stats_combine_blocks(partial, nblocks, nx, i, acc);  // the reduction of dg_stats_values
    for (int s = 0; s < dg::NSTAT; ++s) total[size_t(i) * dg::NSTAT + s] = acc[s];
    const double n = double(nyz);
    const double ua = acc[1] / n, va = acc[2] / n, wa = acc[3] / n;
    double *o = out + 12 + 9 * size_t(i);
    o[0] = ua; o[1] = va; o[2] = wa;
    o[3] = acc[4] / n - ua * wa;
    o[4] = acc[5] / n - ua * va;
    o[5] = acc[6] / n - va * wa;
    o[6] = acc[7] / n - ua * ua;
    o[7] = acc[8] / n - va * va;
    o[8] = acc[9] / n - wa * wa;
}

// Single thread: the diag.dat line (mean, min, max of rho, u, v, w;
// src/output.cu:235-266) and the non-finite count.
__global__ void noalloc_diag_kernel(const double *__restrict__ total, int nx, double ncell, double *__restrict__ out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double sum[4] = {0, 0, 0, 0}, mn[4], mx[4], bad = 0;
    for (int a = 0; a < 4; ++a) { mn[a] = 99999; mx[a] = -99999; }
    for (int i = 0; i < nx; ++i) {
        const double *t = total + size_t(i) * dg::NSTAT;
        for (int a = 0; a < 4; ++a) {
            sum[a] += t[a];
            if (t[10 + a] < mn[a]) mn[a] = t[10 + a];
            if (t[14 + a] > mx[a]) mx[a] = t[14 + a];
        }
        bad += t[18];
    }
    for (int a = 0; a < 4; ++a) {
        out[a] = sum[a] / ncell;
        out[4 + a] = mn[a];
        out[8 + a] = mx[a];
    }
    out[12 + 9 * size_t(nx)] = bad;
}

}  // namespace

extern "C" {

const char *dg_noalloc_last_error(void) { return g_noalloc_error; }

int dg_stats_values_noalloc(const double *f, int nx, int ny, int nz, int pitch, long long pop_stride, double hdt,
                            double fx, double fy, double fz, double *out, void *stream)
{
    if (!f || !out) return fail(DG_ERR_ARG, "NULL state or output pointer");
    if (nx < 1 || ny < 1 || nz < 1) return fail(DG_ERR_SHAPE, "grid sizes must be positive");
    if (nx > kMaxNx) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "nx = %d exceeds the allocation-free maximum of %d (use dg_stats_values)", nx,
                      kMaxNx);
        return fail(DG_ERR_SHAPE, msg);
    }
    if (pitch < nx || pop_stride < (long long)pitch * ny * nz)
        return fail(DG_ERR_SHAPE, "pitch / pop_stride smaller than the grid");
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dg::StepParams<double, double> P;
    std::memset(&P, 0, sizeof(P));
    P.nx = nx; P.ny = ny; P.nz = nz; P.pitch = pitch; P.ps = pop_stride;
    const int nblocks = ny * nz < kBlocks ? ny * nz : kBlocks;
    double *partial = scratch, *total = scratch + kPartial;
    const int bx = nx >= 256 ? 256 : ((nx + 31) / 32) * 32;
    dim3 grid(nblocks, (nx + bx - 1) / bx);
    dg::stats_partials_kernel<double, double><<<grid, bx, 0, st>>>(f, P, hdt, fx, fy, fz, partial);
    noalloc_reduce_kernel<<<(nx + 127) / 128, 128, 0, st>>>(partial, nblocks, nx, ny * nz, total, out);
    noalloc_diag_kernel<<<1, 1, 0, st>>>(total, nx, double(nx) * ny * nz, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, cudaGetErrorString(e));
    return DG_OK;
}

}  // extern "C"
