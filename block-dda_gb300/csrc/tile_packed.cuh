// y passes (B, D) for complex FP32 in packed-pair arithmetic.
//
// Same tasks, tiles and double-buffered cp.async staging as k_pass_y2: a task
// is one (field, x, 16-column z tile), i.e. 8 line pairs (columns 2p and
// 2p + 1 in the two lanes of the f32x2 instructions, pfft.cuh); a CTA of
// 8 / NP warps gives each warp NP pairs.  The tile lives in shared memory in the
// pair layout {re_a, re_b, im_a, im_b}: every element is staged as two 4-byte
// copies (real and imaginary part into their lanes), and read back lane by
// lane when the rows are stored.
#pragma once

#include <cuda_runtime.h>

#include "mvp.hpp"
#include "pfft.cuh"
#include "tile_passes.cuh"

namespace bdda {
namespace tile {

// Line pairs per warp for plan P (a warp's NP pairs give N / R * NP
// butterflies per stage): 1 where every stage then still fills most of a
// warp, else 0, the two-line scalar kernel.  Two pairs per warp (CTAs of four
// warps) measured no faster than the scalar kernel on the two-stage radix
// 10 / 12 / 16 plans that one pair underfills.
template <class P> constexpr int packed_y_pairs() {
  int m = P::N;
  for (int s = 0; s < P::nst; ++s) m = P::N / P::rad[s] < m ? P::N / P::rad[s] : m;
  return m >= 20 ? 1 : 0;
}

template <bool INV, class P, int NP>
__global__ void __launch_bounds__(8 / NP * 32)
k_pass_y2p(const float2* __restrict__ src, float2* __restrict__ dst, const unsigned char* __restrict__ tmask, int ny,
           int nz, int nzp, int nzt, int ntask, const float4* __restrict__ twy, const int* done) {
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Py = P::N, lw = P::LW;
  constexpr int kPairs = kTZ2 / 2;
  constexpr int kThreads = kPairs / NP * 32;
  constexpr int kStep = kThreads / kTZ2;  // rows per staging step
  ulonglong2* pairs = reinterpret_cast<ulonglong2*>(smem_raw);  // [2][kPairs][lw]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nin = INV ? Py : ny;
  const int nout = INV ? ny : Py;
  const int nzt2 = (nz + kTZ2 - 1) / kTZ2;
  const int tw = tid & (kTZ2 - 1), ty = tid / kTZ2;  // tile column and first row of this thread
  const int half = tw & 1;                           // lane of the column in its pair
  auto issue = [&](int task, int buf) {
    const int zt2 = task % nzt2;
    const int r = task / nzt2;  // f * Px + q
    const int z = zt2 * kTZ2 + tw;
    const bool zval = z < nz;
    const float2* g = src + (size_t)r * nin * nzp + z + (size_t)ty * nzp;
    const unsigned char* tm = tmask + (zval ? z / kTZ : 0) + (size_t)ty * nzt;
    float* lb = reinterpret_cast<float*>(pairs + (buf * kPairs + (tw >> 1)) * lw) + half;
    for (int yy = ty; yy < nin; yy += kStep, g += (size_t)kStep * nzp, tm += (size_t)kStep * nzt) {
      const bool valid = zval && (INV || *tm);
      const float* gs = reinterpret_cast<const float*>(valid ? g : src);
      float* d = lb + 4 * P::addr(yy);
      cp_async<4>(d, gs, valid);          // real part -> lane `half` of re
      cp_async<4>(d + 2, gs + 1, valid);  // imaginary part -> lane `half` of im
    }
    cp_commit();
  };
  int task = blockIdx.x;
  if (task < ntask) issue(task, 0);
  for (int it = 0; task < ntask; ++it, task += gridDim.x) {
    const int buf = it & 1;
    const int next = task + gridDim.x;
    if (next < ntask) {
      issue(next, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    ulonglong2* wl = pairs + (buf * kPairs + warp * NP) * lw;
    if (!INV) pk::forward<P, NP>(wl, twy, lane, ny);
    else pk::inverse<P, NP>(wl, twy, lane, ny);
    __syncthreads();
    const int zt2 = task % nzt2;
    const int r = task / nzt2;
    const int z = zt2 * kTZ2 + tw;
    if (z < nz) {
      float2* ob = dst + (size_t)r * nout * nzp + z + (size_t)ty * nzp;
      const unsigned char* tm = tmask + z / kTZ + (size_t)ty * nzt;
      const float* lb = reinterpret_cast<const float*>(pairs + (buf * kPairs + (tw >> 1)) * lw) + half;
      for (int yy = ty; yy < nout; yy += kStep, ob += (size_t)kStep * nzp, tm += (size_t)kStep * nzt)
        if (!INV || *tm) {
          const float* s = lb + 4 * P::addr(yy);
          *ob = make_float2(s[0], s[2]);
        }
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of the next-but-one task
  }
}

}  // namespace tile
}  // namespace bdda
