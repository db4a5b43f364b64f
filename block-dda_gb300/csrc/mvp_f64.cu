// Block-MVP launcher and runtime-plan kernels instantiated for double (one
// translation unit per arithmetic type, so the build compiles them in parallel).
#include "mvp_launch.cuh"

namespace bdda {
template cudaError_t launch_block_mvp<double>(const MvpGeom&, const MvpPrec<double>&, const double2*, int, double2*, int, int,
                                          const double2*, const double2*, double2*, double2*, cudaStream_t, KernelTimer*, const int*);
template cudaError_t configure_mvp_kernels<double>();
}  // namespace bdda
