// Fused z pass (pass C) for complex FP32 with a compile-time z plan.
//
// Same work as the runtime-plan k_pass_c: one warp per (x, y, rhs) task runs
// the pruned forward z transform of the three component lines, the symmetric
// 3x3 Green product and the inverse transform.  The plan (radix sequence,
// padded layout, line pitch) comes from zplans.inc, so the addresses of every
// butterfly element are a per-task base plus compile-time offsets and the
// divisions of the index arithmetic are by constants.  The radix sequence is
// the one the host planner gives the z axis, so the transform order matches
// the Green spectrum's.
//
// Layout: element idx = q * R_last + r of a line lives at q * S + r; every
// stage s < last steps through its butterfly in multiples of R_last, so its
// elements are (M_s / R_last) * S apart; the last stage's are adjacent.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "fft_core.cuh"
#include "mvp.hpp"

namespace bdda {
namespace zstatic {

template <int N_, int S_, int LW_, int... R>
struct ZPlan {
  static constexpr int N = N_, S = S_, LW = LW_, nst = sizeof...(R);
  static constexpr int rad[nst] = {R...};
  static constexpr int Rl = rad[nst - 1];
  // product of the radices after stage s (the butterfly span M_s)
  static constexpr int M(int s) {
    int m = 1;
    for (int t = s + 1; t < nst; ++t) m *= rad[t];
    return m;
  }
  __device__ static __forceinline__ int addr(int idx) { return (idx / Rl) * S + idx % Rl; }
};

// One stage over the three lines of a warp.  Forward (DIF): DFT then twiddle;
// inverse (DIT, the adjoint): conjugate twiddle then inverse DFT.  The forward
// first stage reads only inputs idx < nv (the rest are zero padding); the
// inverse last stage writes only outputs idx < nv (the rest are discarded).
template <class P, int s, bool INV>
__device__ __forceinline__ void stage(float2* __restrict__ sm, const float2* __restrict__ tw, int lane, int nv) {
  constexpr int R = P::rad[s];
  constexpr int M = P::M(s);
  constexpr int Ls = M * R;
  constexpr int B = P::N / R;    // butterflies per line
  constexpr int T = 3 * B;       // butterflies of the warp
  constexpr int ts = P::N / Ls;  // twiddle table stride
  constexpr int off = (s == P::nst - 1) ? 1 : (M / P::Rl) * P::S;
  constexpr bool prune_in = !INV && s == 0;
  constexpr bool prune_out = INV && s == 0;
  for (int t = lane; t < T; t += 32) {
    const int j = t / B, u = t - j * B;
    const int b = u / M, n1 = u - b * M;
    const int idx0 = b * Ls + n1;
    float2* p = sm + j * P::LW + P::addr(idx0);
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_in) v[i] = (idx0 + i * M < nv) ? p[i * off] : make_float2(0.f, 0.f);
      else v[i] = p[i * off];
    }
    if (!INV) {
      dft<R, false>(v);
      if (M > 1 && n1 != 0) {
        const int step = n1 * ts;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmul(v[k], ldg_c(tw + k * step));
      }
    } else {
      if (M > 1 && n1 != 0) {
        const int step = n1 * ts;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmulc(v[k], ldg_c(tw + k * step));
      }
      dft<R, true>(v);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_out) {
        if (idx0 + i * M < nv) p[i * off] = v[i];
      } else {
        p[i * off] = v[i];
      }
    }
  }
  __syncwarp();
}

template <class P, int s = 0>
__device__ __forceinline__ void forward(float2* sm, const float2* tw, int lane, int nv) {
  if constexpr (s < P::nst) {
    stage<P, s, false>(sm, tw, lane, nv);
    forward<P, s + 1>(sm, tw, lane, nv);
  }
}

template <class P, int s = P::nst - 1>
__device__ __forceinline__ void inverse(float2* sm, const float2* tw, int lane, int nv) {
  if constexpr (s >= 0) {
    stage<P, s, true>(sm, tw, lane, nv);
    inverse<P, s - 1>(sm, tw, lane, nv);
  }
}

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
  forward<P>(s0, twz, lane, nz);
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
  inverse<P>(s0, twz, lane, nz);
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

// Launches the plan of g.Pz if it belongs to this part (plans are spread over
// kParts translation units by their position in zplans.inc).
constexpr int kParts = 4;

template <int PART>
bool dispatch(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
              const int* done, cudaError_t* err) {
  switch (g.Pz) {
#define BDDA_ZPLAN(I, N, S, LW, ...)                                                     \
  case N:                                                                                \
    if constexpr ((I) % kParts == PART) {                                                \
      *err = launch<ZPlan<N, S, LW, __VA_ARGS__>>(g, t2, L, twz, ghat, st, done);        \
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

}  // namespace zstatic
}  // namespace bdda
