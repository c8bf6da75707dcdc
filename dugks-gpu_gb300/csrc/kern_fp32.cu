// Explicit instantiation of the step and auxiliary kernels for the fp32 form
// (arithmetic float, storage float).
#include "launch_impl.cuh"

namespace dg {
template struct Kern<float, float>;
}
