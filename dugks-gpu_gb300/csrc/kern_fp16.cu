// Explicit instantiation of the step and auxiliary kernels for the fp16 form
// (arithmetic float, storage __half).
#include "launch_impl.cuh"

namespace dg {
template struct Kern<float, __half>;
}
