// Fused z pass (pass C) for complex FP32 with a compile-time z plan.
//
// Same work as the runtime-plan k_pass_c: one warp per (x, y, rhs) task runs
// the pruned forward z transform of the three component lines, the symmetric
// 3x3 Green product and the inverse transform (output truncated to nz).  The
// plan (zplans.inc) is a type, so every butterfly element and every line
// element is addressed as a base plus compile-time offsets (static_fft.cuh).
// Its radix sequence is the one the host planner gives the z axis, so the
// transform order matches the Green spectrum's.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "mvp.hpp"
#include "static_fft.cuh"

namespace bdda {
namespace zstatic {

template <class P>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c_static(float2* __restrict__ t2, int L, int Px, int Py, int nz, const float2* __restrict__ twz,
                const float2* __restrict__ ghat, const int* done) {
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Pz = P::N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long task = (long long)blockIdx.x * kZWarps + warp;
  if (task >= (long long)Px * Py * L) return;
  const int l = (int)(task % L);
  const long long line = task / L;  // q * Py + qy
  float2* s0 = reinterpret_cast<float2*>(smem_raw) + (size_t)warp * 3 * P::LW;
  const size_t fstride = (size_t)Px * Py * nz;  // between fields
  float2* g0 = t2 + (size_t)(3 * l) * fstride + (size_t)line * nz;
  for (int z = lane; z < nz; z += 32) {
    const int a = P::addr(z);
    s0[a] = g0[z];
    s0[P::LW + a] = g0[fstride + z];
    s0[2 * P::LW + a] = g0[2 * fstride + z];
  }
  __syncwarp();
  sfft::forward<P, 3>(s0, twz, lane, nz);
  const float2* gl = ghat + (size_t)line * 6 * Pz;
  for (int p = lane; p < Pz; p += 32) {
    const int a = P::addr(p);
    const float2 a0 = s0[a], a1 = s0[P::LW + a], a2 = s0[2 * P::LW + a];
    const float2 gxx = ldg_c(gl + p), gxy = ldg_c(gl + Pz + p), gxz = ldg_c(gl + 2 * Pz + p);
    const float2 gyy = ldg_c(gl + 3 * Pz + p), gyz = ldg_c(gl + 4 * Pz + p), gzz = ldg_c(gl + 5 * Pz + p);
    s0[a] = cadd(cadd(cmul(gxx, a0), cmul(gxy, a1)), cmul(gxz, a2));
    s0[P::LW + a] = cadd(cadd(cmul(gxy, a0), cmul(gyy, a1)), cmul(gyz, a2));
    s0[2 * P::LW + a] = cadd(cadd(cmul(gxz, a0), cmul(gyz, a1)), cmul(gzz, a2));
  }
  __syncwarp();
  sfft::inverse<P, 3>(s0, twz, lane, nz);
  for (int z = lane; z < nz; z += 32) {
    const int a = P::addr(z);
    g0[z] = s0[a];
    g0[fstride + z] = s0[P::LW + a];
    g0[2 * fstride + z] = s0[2 * P::LW + a];
  }
}

template <class P>
cudaError_t launch(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
                   const int* done) {
  constexpr int smem = kZWarps * 3 * P::LW * (int)sizeof(float2);
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_pass_c_static<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  });
  if (cfg != cudaSuccess) return cfg;
  const long long ntask = (long long)g.Px * g.Py * L;
  const unsigned grid = (unsigned)((ntask + kZWarps - 1) / kZWarps);
  k_pass_c_static<P><<<grid, kZWarps * 32, smem, st>>>(t2, L, g.Px, g.Py, g.nz, twz, ghat, done);
  return cudaGetLastError();
}

}  // namespace zstatic
}  // namespace bdda
