// Compile-time-plan z pass, part 3 of zstatic::kParts (split for a parallel build).
#include "zpass_static.cuh"

namespace bdda {
bool pass_c_static_part3(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
                          const int* done, cudaError_t* err) {
  return zstatic::dispatch<3>(g, t2, L, twz, ghat, st, done, err);
}
}  // namespace bdda
