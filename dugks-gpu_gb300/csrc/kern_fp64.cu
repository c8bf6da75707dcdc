// Explicit instantiation of the step and auxiliary kernels for the fp64 form
// (arithmetic double, storage double).
#include "launch_impl.cuh"

namespace dg {
template struct Kern<double, double>;
}
