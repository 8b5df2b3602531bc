// Instantiates the batched propagation kernels for float compute.
#include "prop.cuh"

namespace fwi {
template void launch_forward_step<float>(const Batch<float> &, int, int, int, int, int, bool, cudaStream_t);
template void launch_adjoint_step<float>(const Batch<float> &, int, int, int, int, int, bool, int, cudaStream_t);
}  // namespace fwi
