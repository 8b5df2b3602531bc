// Instantiates the batched propagation kernels for double compute.
#include "prop.cuh"

namespace fwi {
template void launch_forward_step<double>(const Batch<double> &, int, int, int, int, int, bool, cudaStream_t);
template void launch_adjoint_step<double>(const Batch<double> &, int, int, int, int, int, bool, int, cudaStream_t);
}  // namespace fwi
