// Compile-time-plan kernels of complex FP32, part 0 of sparts::kParts.
#include "static_parts.cuh"

namespace bdda {
bool static_z_part0(const MvpGeom& g, float2* t2, int L, const float2* twz, const float4* twzp, const float2* ghat,
                    cudaStream_t st, const int* done, cudaError_t* err) {
  return sparts::dispatch_z<0>(g, t2, L, twz, twzp, ghat, st, done, err);
}
bool static_tile_part0(int pass, const TileArgs& a, cudaError_t* err) { return sparts::dispatch_tile<0>(pass, a, err); }
bool static_z_df_part0(const MvpGeom& g, dfzc* t2, int L, const dfzc* twz, const dfzc* ghat, cudaStream_t st,
                       const int* done, cudaError_t* err) {
  return sparts::dispatch_z_df<0>(g, t2, L, twz, ghat, st, done, err);
}

bool static_z_part1(const MvpGeom&, float2*, int, const float2*, const float4*, const float2*, cudaStream_t, const int*,
                    cudaError_t*);
bool static_z_part2(const MvpGeom&, float2*, int, const float2*, const float4*, const float2*, cudaStream_t, const int*,
                    cudaError_t*);
bool static_z_part3(const MvpGeom&, float2*, int, const float2*, const float4*, const float2*, cudaStream_t, const int*,
                    cudaError_t*);
bool static_tile_part1(int, const TileArgs&, cudaError_t*);
bool static_tile_part2(int, const TileArgs&, cudaError_t*);
bool static_tile_part3(int, const TileArgs&, cudaError_t*);

bool launch_pass_c_static(const MvpGeom& g, float2* t2, int L, const float2* twz, const float4* twzp, const float2* ghat,
                          cudaStream_t st, const int* done, cudaError_t* err) {
  static_assert(sparts::kParts == 4, "one function per part");
  return static_z_part0(g, t2, L, twz, twzp, ghat, st, done, err) ||
         static_z_part1(g, t2, L, twz, twzp, ghat, st, done, err) ||
         static_z_part2(g, t2, L, twz, twzp, ghat, st, done, err) ||
         static_z_part3(g, t2, L, twz, twzp, ghat, st, done, err);
}

bool static_z_df_part1(const MvpGeom&, dfzc*, int, const dfzc*, const dfzc*, cudaStream_t, const int*, cudaError_t*);
bool static_z_df_part2(const MvpGeom&, dfzc*, int, const dfzc*, const dfzc*, cudaStream_t, const int*, cudaError_t*);
bool static_z_df_part3(const MvpGeom&, dfzc*, int, const dfzc*, const dfzc*, cudaStream_t, const int*, cudaError_t*);

bool launch_pass_c_static_df(const MvpGeom& g, dfzc* t2, int L, const dfzc* twz, const dfzc* ghat, cudaStream_t st,
                             const int* done, cudaError_t* err) {
  return static_z_df_part0(g, t2, L, twz, ghat, st, done, err) || static_z_df_part1(g, t2, L, twz, ghat, st, done, err) ||
         static_z_df_part2(g, t2, L, twz, ghat, st, done, err) || static_z_df_part3(g, t2, L, twz, ghat, st, done, err);
}

bool pipe_z_available(int Pz, int f, int nzp, int L) {
  if (f != 3) return false;
  const int nw = L < kZWarps ? L : kZWarps;
  switch (Pz) {
#define BDDA_ZPLAN(I, N, S, LW, ...)                                                      \
  case N:                                                                                 \
    return zpipe::smem_bytes<sfft::Plan<N, S, LW, __VA_ARGS__>>(nw, nzp) <= (size_t)kZSmemMax;
#include "zplans.inc"
#undef BDDA_ZPLAN
    default:
      return false;
  }
}

bool packed_z_available(int Pz, int f) {
  if (f != 3) return false;
  switch (Pz) {
#define BDDA_ZPLAN(I, N, S, LW, ...) \
  case N:                            \
    return zpacked::supported<sfft::Plan<N, S, LW, __VA_ARGS__>>() && zpacked::fits<sfft::Plan<N, S, LW, __VA_ARGS__>>();
#include "zplans.inc"
#undef BDDA_ZPLAN
    default:
      return false;
  }
}

bool launch_tile_static(int pass, const TileArgs& a, cudaError_t* err) {
  return static_tile_part0(pass, a, err) || static_tile_part1(pass, a, err) || static_tile_part2(pass, a, err) ||
         static_tile_part3(pass, a, err);
}
}  // namespace bdda
