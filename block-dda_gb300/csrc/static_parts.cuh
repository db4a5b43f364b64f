// Dispatch of the compile-time-plan kernels of complex FP32 by line length.
// The plans are spread over kParts translation units (by their position in
// the plan tables) so that the build compiles them in parallel.
#pragma once

#include "tile_static.cuh"
#include "zpass_packed.cuh"
#include "zpass_pipe.cuh"
#include "zpass_static.cuh"

namespace bdda {
namespace sparts {

constexpr int kParts = 4;

template <int PART>
bool dispatch_z(const MvpGeom& g, float2* t2, int L, const float2* twz, const float4* twzp, const float2* ghat,
                cudaStream_t st, const int* done, cudaError_t* err) {
  switch (g.Pz) {
#define BDDA_ZPLAN(I, N, S, LW, ...)                                                     \
  case N:                                                                                \
    if constexpr ((I) % kParts == PART) {                                                \
      using Pl = sfft::Plan<N, S, LW, __VA_ARGS__>;                                      \
      if constexpr (zpacked::supported<Pl>())                                            \
        if (zpacked::chosen<Pl>(g, twzp)) {                                              \
          *err = zpacked::launch<Pl>(g, t2, L, twzp, ghat, st, done);                    \
          return true;                                                                   \
        }                                                                                \
      if ((g.tune.zkern < 0 || g.tune.zkern == 2) &&                                     \
          zpipe::launch<Pl>(g, t2, L, twz, ghat, st, done, err))                         \
        return true;                                                                     \
      *err = zstatic::launch<Pl>(g, t2, L, twz, ghat, st, done);                         \
      return true;                                                                       \
    }                                                                                    \
    return false;
#include "zplans.inc"
#undef BDDA_ZPLAN
    default:
      break;
  }
  return false;
}

// The double-float z pass of f = 3 operators with the 16-byte z table's
// compile-time plans (the double-float Green spectrum is in their digit order).
template <int PART>
bool dispatch_z_df(const MvpGeom& g, dfzc* t2, int L, const dfzc* twz, const dfzc* ghat, cudaStream_t st,
                   const int* done, cudaError_t* err) {
  if (g.f != 3) return false;
  switch (g.Pz) {
#define BDDA_ZWPLAN(I, N, S, LW, ...)                                                                 \
  case N:                                                                                             \
    if constexpr ((I) % kParts == PART) {                                                             \
      *err = zstatic::launch_f<sfft::Plan<N, S, LW, __VA_ARGS__>, false, dfzc>(g, t2, L, twz, ghat, st, done); \
      return true;                                                                                    \
    }                                                                                                 \
    return false;
#include "zwplans.inc"
#undef BDDA_ZWPLAN
    default:
      break;
  }
  return false;
}

template <int PART>
bool dispatch_tile(int pass, const TileArgs& a, cudaError_t* err) {
  if (pass == kTileA || pass == kTileE) {
    switch (a.g->Px) {
#define BDDA_TPLAN(I, N, S, LW, ...)                                                     \
  case N:                                                                                \
    if constexpr ((I) % kParts == PART) {                                                \
      *err = tstatic::launch_x<sfft::Plan<N, S, LW, __VA_ARGS__>>(pass, a);              \
      return true;                                                                       \
    }                                                                                    \
    return false;
#include "tplans.inc"
#undef BDDA_TPLAN
      default:
        break;
    }
    return false;
  }
  switch (a.g->Py) {
#define BDDA_YPLAN(I, N, S, LW, ...)                                                     \
  case N:                                                                                \
    if constexpr ((I) % kParts == PART) {                                                \
      *err = tstatic::launch_y<sfft::Plan<N, S, LW, __VA_ARGS__>>(pass, a);              \
      return true;                                                                       \
    }                                                                                    \
    return false;
#include "yplans.inc"
#undef BDDA_YPLAN
    default:
      break;
  }
  return false;
}

}  // namespace sparts
}  // namespace bdda
