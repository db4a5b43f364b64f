// Compile-time-plan z pass, part 0 of zstatic::kParts (split for a parallel build).
#include "zpass_static.cuh"

namespace bdda {
bool pass_c_static_part0(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
                          const int* done, cudaError_t* err) {
  return zstatic::dispatch<0>(g, t2, L, twz, ghat, st, done, err);
}

bool pass_c_static_part1(const MvpGeom&, float2*, int, const float2*, const float2*, cudaStream_t, const int*, cudaError_t*);
bool pass_c_static_part2(const MvpGeom&, float2*, int, const float2*, const float2*, cudaStream_t, const int*, cudaError_t*);
bool pass_c_static_part3(const MvpGeom&, float2*, int, const float2*, const float2*, cudaStream_t, const int*, cudaError_t*);

bool launch_pass_c_static(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
                          const int* done, cudaError_t* err) {
  static_assert(zstatic::kParts == 4, "one function per part");
  return pass_c_static_part0(g, t2, L, twz, ghat, st, done, err) ||
         pass_c_static_part1(g, t2, L, twz, ghat, st, done, err) ||
         pass_c_static_part2(g, t2, L, twz, ghat, st, done, err) ||
         pass_c_static_part3(g, t2, L, twz, ghat, st, done, err);
}
}  // namespace bdda
