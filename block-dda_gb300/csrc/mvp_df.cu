// Block-MVP launcher and runtime-plan kernels instantiated for dfl (one
// translation unit per arithmetic type, so the build compiles them in parallel).
#include "mvp_launch.cuh"

namespace bdda {
template cudaError_t launch_block_mvp<dfl>(const MvpGeom&, const MvpPrec<dfl>&, const dfc*, int, dfc*, int, int,
                                          const dfc*, const dfc*, dfc*, dfc*, cudaStream_t, KernelTimer*, const int*);
template cudaError_t configure_mvp_kernels<dfl>();
}  // namespace bdda
