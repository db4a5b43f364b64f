// Block-MVP launcher and runtime-plan kernels instantiated for the
// double-float MVP arithmetic dfz (one translation unit per arithmetic type,
// so the build compiles them in parallel).
#include "mvp_launch.cuh"

namespace bdda {
template cudaError_t launch_block_mvp<dfz>(const MvpGeom&, const MvpPrec<dfz>&, const dfzc*, int, dfzc*, int, int,
                                          const dfzc*, const dfzc*, dfzc*, dfzc*, cudaStream_t, KernelTimer*,
                                          const int*);
template cudaError_t configure_mvp_kernels<dfz>();
}  // namespace bdda
