// Instantiates the batched propagation kernels for double compute.
#include "prop.cuh"

namespace fwi {
template void launch_forward_step<double>(const Batch<double> &, int, int, int, int, int, bool, const StepStreams &);
template void launch_adjoint_step<double>(const Batch<double> &, int, int, int, int, int, bool, int,
                                           const StepStreams &);
}  // namespace fwi
