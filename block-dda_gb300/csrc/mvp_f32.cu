// Block-MVP launcher and runtime-plan kernels instantiated for float (one
// translation unit per arithmetic type, so the build compiles them in parallel).
#include "mvp_launch.cuh"

namespace bdda {
template cudaError_t launch_block_mvp<float>(const MvpGeom&, const MvpPrec<float>&, const float2*, int, float2*, int, int,
                                          const float2*, const float2*, float2*, float2*, cudaStream_t, KernelTimer*, const int*);
template cudaError_t configure_mvp_kernels<float>();
}  // namespace bdda
