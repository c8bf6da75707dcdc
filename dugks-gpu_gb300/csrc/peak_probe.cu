// FP64 arithmetic-pipe peak of the current GPU, for the compute roofline of
// the FP64 step (its kernels are bound by FP64 instruction issue, not HBM).
//
// Every thread runs 8 independent chains of dependent FMAs; the grid fills
// all SMs several times over.  The rate is FP64 FMA instructions per second
// (one FMA = 2 flops), timed with CUDA events on the given stream.  The
// library holds no state; each call allocates and frees one small buffer.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fma_chain_kernel(double *out, int iters, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = double(threadIdx.x + c) * 1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" {

// FP64 FMA instructions per second (thread-level) over `reps` launches after
// one warm-up launch; returns 0 on success, a CUDA error code otherwise.
int dg_probe_fp64_fma_rate(void *stream, int reps, double *fma_per_s)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return int(e);
    const int threads = 256, blocks = sms * 8, iters = 4096;
    double *out = nullptr;
    e = cudaMalloc(&out, sizeof(double) * size_t(blocks) * threads);
    if (e != cudaSuccess) return int(e);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chain_kernel<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) fma_chain_kernel<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        *fma_per_s = double(blocks) * threads * double(iters) * kChains * reps / (double(ms) * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return int(e);
}

}  // extern "C"
