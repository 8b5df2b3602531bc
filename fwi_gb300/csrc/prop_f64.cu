// Instantiates the batched propagation kernels for double compute.
#include "prop_boundary.cuh"
#include "prop.cuh"

namespace fwi {
template void launch_forward_step<double>(const Batch<double> &, int, int, int, int, int, bool, const StepStreams &);
template void launch_adjoint_step<double>(const Batch<double> &, int, int, int, int, int, bool, int,
                                           const StepStreams &);
template void launch_save_ring<double>(const Batch<double> &, int, int, int, int, double *, long, cudaStream_t);
template void launch_rebuild_begin<double>(const Batch<double> &, int, int, int, int, const double *, long,
                                           cudaStream_t);
template void launch_rebuild_step<double>(const Batch<double> &, int, int, int, int, const double *, long, int,
                                          cudaStream_t);
}  // namespace fwi
