// Fused z pass (pass C) for complex FP32 with a compile-time z plan.
//
// Same work as the runtime-plan k_pass_c: one warp per (x, y, rhs) task runs
// the pruned forward z transform of the 3 (f = 3) or 6 (f = 6) component
// lines, the Green product (zproduct.cuh) and the inverse transform (output
// truncated to nz).  The
// plan (zplans.inc) is a type, so every butterfly element and every line
// element is addressed as a base plus compile-time offsets (static_fft.cuh).
// Its radix sequence is the one the host planner gives the z axis, so the
// transform order matches the Green spectrum's.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "mvp.hpp"
#include "static_fft.cuh"
#include "zproduct.cuh"

namespace bdda {
namespace zstatic {

template <class P, bool SIX, typename C = float2>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c_static(C* __restrict__ t2, int L, int Px, int Py, int nz, int nzp, const C* __restrict__ twz,
                const C* __restrict__ ghat, const int* done) {
  constexpr int fc = SIX ? 6 : 3;
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Pz = P::N, LW = P::LW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long task = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  if (task >= (long long)Px * Py * L) return;
  const int l = (int)(task % L);
  const long long line = task / L;  // q * Py + qy
  C* s0 = reinterpret_cast<C*>(smem_raw) + (size_t)warp * fc * LW;
  const size_t fstride = (size_t)Px * Py * nzp;  // between fields
  C* g0 = t2 + (size_t)(fc * l) * fstride + (size_t)line * nzp;
  constexpr bool six = SIX;
  constexpr int halves = six ? 2 : 1;  // line triples: E, then M
  const C* gl = ghat + (size_t)line * (six ? 9 : 6) * Pz;
  if constexpr (!SIX && sizeof(C) == sizeof(float2) && fused_z(P::N, P::nst, P::Rl)) {
    // complex FP32 (its spectrum is last-radix-major)
    // last forward stage, product and first inverse stage fused (middle3)
    sfft::stage0_from_global<P, 3, C>(s0, twz, lane, nz, g0, fstride);
    sfft::forward_to<P, 3, 1, P::nst - 1, C>(s0, twz, lane, nz);
    sfft::middle3<P, C>(s0, gl, lane);
    sfft::inverse<P, 3, P::nst - 2, 1, C>(s0, twz, lane, nz);
    sfft::stage0_to_global<P, 3, C>(s0, twz, lane, nz, g0, fstride);
    return;
  }
  // the first forward stage reads the lines straight from T2 (no staging loop)
  for (int h = 0; h < halves; ++h)
    sfft::forward_from_global<P, 3>(s0 + 3 * h * LW, twz, lane, nz, g0 + 3 * h * fstride, fstride);
  for (int p = lane; p < Pz; p += 32) z_product(s0, LW, P::addr(p), gl, Pz, p, six);
  __syncwarp();
  // the last inverse stage writes the lines straight back to T2 (rows past nz dropped)
  for (int h = 0; h < halves; ++h)
    sfft::inverse_to_global<P, 3>(s0 + 3 * h * LW, twz, lane, nz, g0 + 3 * h * fstride, fstride);
}

template <class P, bool SIX, typename C = float2>
cudaError_t launch_f(const MvpGeom& g, C* t2, int L, const C* twz, const C* ghat, cudaStream_t st, const int* done) {
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_pass_c_static<P, SIX, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, kZSmemMax);
  });
  if (cfg != cudaSuccess) return cfg;
  const int per_warp = (SIX ? 6 : 3) * P::LW * (int)sizeof(C);
  const int wpc = z_warps_per_cta(per_warp);
  const long long ntask = (long long)g.Px * g.Py * L;
  const unsigned grid = (unsigned)((ntask + wpc - 1) / wpc);
  k_pass_c_static<P, SIX, C><<<grid, wpc * 32, wpc * per_warp, st>>>(t2, L, g.Px, g.Py, g.nz, g.nzp, twz, ghat, done);
  return cudaGetLastError();
}

template <class P>
cudaError_t launch(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
                   const int* done) {
  return g.f == 6 ? launch_f<P, true>(g, t2, L, twz, ghat, st, done) : launch_f<P, false>(g, t2, L, twz, ghat, st, done);
}

}  // namespace zstatic
}  // namespace bdda
