// Explicit instantiation of the step and auxiliary kernels for the bf16 form
// (arithmetic float, storage __nv_bfloat16).
#include "launch_impl.cuh"

namespace dg {
template struct Kern<float, __nv_bfloat16>;
}
