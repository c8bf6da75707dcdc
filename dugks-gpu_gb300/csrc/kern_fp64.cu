// Explicit instantiation of the step and auxiliary kernels for the fp64 form
// (arithmetic double, storage double).
#include "launch_impl.cuh"

namespace dg {
template struct Kern<double, double>;

// The time-out path of the bounded waits, on its own: one thread waits on an
// mbarrier that nothing ever arrives at (no copy is issued, so nothing is in
// flight), gives up after `limit` polls, raises the error flag that dg_sync
// reports and returns.  Used by dg_selftest_wait_timeout.
namespace {
__global__ void wait_timeout_selftest_kernel(int *err, int limit, long long *polled_cycles)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t0 = clock64();
        if (!mbar_wait(smem_u32(&bar), 0u, limit)) atomicOr(err, 1);
        *polled_cycles = clock64() - t0;
    }
}
}  // namespace

cudaError_t launch_wait_timeout_selftest(int *err, int limit, long long *polled_cycles, cudaStream_t st)
{
    wait_timeout_selftest_kernel<<<1, 32, 0, st>>>(err, limit, polled_cycles);
    return cudaGetLastError();
}
}  // namespace dg
