// Compile-time-plan kernels of complex FP32, part 3 of sparts::kParts.
#include "static_parts.cuh"

namespace bdda {
bool static_z_part3(const MvpGeom& g, float2* t2, int L, const float2* twz, const float4* twzp, const float2* ghat,
                    cudaStream_t st, const int* done, cudaError_t* err) {
  return sparts::dispatch_z<3>(g, t2, L, twz, twzp, ghat, st, done, err);
}
bool static_tile_part3(int pass, const TileArgs& a, cudaError_t* err) { return sparts::dispatch_tile<3>(pass, a, err); }
bool static_z_df_part3(const MvpGeom& g, dfzc* t2, int L, const dfzc* twz, const dfzc* ghat, cudaStream_t st,
                       const int* done, cudaError_t* err) {
  return sparts::dispatch_z_df<3>(g, t2, L, twz, ghat, st, done, err);
}
}  // namespace bdda
