// Fused z pass (pass C) for complex FP32, f = 3, in packed-pair arithmetic.
//
// One warp per (x, y, rhs pair) task: the z lines of the three components of
// right-hand sides 2 lp and 2 lp + 1 are transformed as three line pairs
// (pfft.cuh), multiplied by the Green spectrum of the (x, y) line, and
// transformed back, the pair's two lines in the two lanes of every f32x2
// instruction.  The work per line, the plan and the digit order are those of
// the scalar kernel (zpass_static.cuh); an odd last right-hand side runs in
// both lanes and is stored once.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "mvp.hpp"
#include "pfft.cuh"
#include "static_fft.cuh"

namespace bdda {
namespace zpacked {

// E' = A E at one frequency for a line-pair triple (A = -G, symmetric,
// components xx xy xz yy yz zz; mvp_fft/application_function.cpp:36-40)
__device__ __forceinline__ void z_product_pair(ulonglong2* __restrict__ s, int lw, int a, const float2* __restrict__ gl,
                                               int Pz, int p) {
  using pk::u64;
  const pk::cp e0 = pk::lds(s + a), e1 = pk::lds(s + lw + a), e2 = pk::lds(s + 2 * lw + a);
  u64 gr[6], gi[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float2 g = ldg_c(gl + c * Pz + p);
    gr[c] = pk::dup(g.x);
    gi[c] = pk::dup(g.y);
  }
  constexpr int m[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    // re' = sum re_d gr - sum im_d gi ; im' = sum im_d gr + re_d gi
    u64 ar = pk::mul(e0.re, gr[m[o][0]]);
    ar = pk::fma(e1.re, gr[m[o][1]], ar);
    ar = pk::fma(e2.re, gr[m[o][2]], ar);
    u64 ai = pk::mul(e0.im, gi[m[o][0]]);
    ai = pk::fma(e1.im, gi[m[o][1]], ai);
    ai = pk::fma(e2.im, gi[m[o][2]], ai);
    u64 bi = pk::mul(e0.im, gr[m[o][0]]);
    bi = pk::fma(e1.im, gr[m[o][1]], bi);
    bi = pk::fma(e2.im, gr[m[o][2]], bi);
    bi = pk::fma(e0.re, gi[m[o][0]], bi);
    bi = pk::fma(e1.re, gi[m[o][1]], bi);
    bi = pk::fma(e2.re, gi[m[o][2]], bi);
    pk::sts(s + o * lw + a, pk::cp{pk::sub(ar, ai), bi});
  }
}

template <class P>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c_packed(float2* __restrict__ t2, int L, int Px, int Py, int nz, int nzp, const float4* __restrict__ twz,
                const float2* __restrict__ ghat, const int* done) {
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Pz = P::N, LW = P::LW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Lp = (L + 1) >> 1;
  const long long task = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  if (task >= (long long)Px * Py * Lp) return;
  const int lp = (int)(task % Lp);
  const long long line = task / Lp;  // q * Py + qy
  const int la = 2 * lp;
  const bool has_b = la + 1 < L;
  ulonglong2* s0 = reinterpret_cast<ulonglong2*>(smem_raw) + (size_t)warp * 3 * LW;
  const size_t fstride = (size_t)Px * Py * nzp;  // between fields
  float2* g0 = t2 + (size_t)(3 * la) * fstride + (size_t)line * nzp;
  const ptrdiff_t boff = has_b ? (ptrdiff_t)(3 * fstride) : 0;  // right-hand side la + 1
  pk::stage0_from_global<P, 3>(s0, twz, lane, nz, g0, fstride, boff);
  const float2* gl = ghat + (size_t)line * 6 * Pz;
  if constexpr (fused_z(P::N, P::nst, P::Rl)) {  // the spectrum is last-radix-major
    // last forward stage, product and first inverse stage fused (pk::middle3)
    pk::forward_to<P, 3, 1, P::nst - 1>(s0, twz, lane, nz);
    pk::middle3<P>(s0, gl, lane);
    pk::inverse<P, 3, P::nst - 2, 1>(s0, twz, lane, nz);
  } else {
    pk::forward<P, 3, 1>(s0, twz, lane, nz);
    for (int p = lane; p < Pz; p += 32) z_product_pair(s0, LW, P::addr(p), gl, Pz, p);
    __syncwarp();
    pk::inverse<P, 3, P::nst - 1, 1>(s0, twz, lane, nz);
  }
  pk::stage0_to_global<P, 3>(s0, twz, lane, nz, g0, fstride, boff, has_b);
}

// The packed kernel keeps twice the bytes of lines per warp (16-byte pair
// elements); it pays where three 8-warp CTAs still fit on an SM (line pitch
// <= 197: Pz up to ~190).  Longer lines keep the scalar kernel, whose
// occupancy is then twice as high (Pz=250: 9.9 ms scalar vs 10.3 ms packed
// per N=65536, L=32 block MVP; Pz=120: 0.35 vs 0.31 ms at N=8192, L=16).
template <class P> constexpr bool worth() { return 3 * kZWarps * 3 * P::LW * 16 <= kZSmemMax; }
// The packed kernel can run where two 8-warp CTAs fit; between that and
// worth() the autotuner decides (MvpTune::zkern).
template <class P> constexpr bool fits() { return 2 * kZWarps * 3 * P::LW * 16 <= kZSmemMax; }
// Plans the packed kernel is built for: register radices <= 16 (a pair
// element takes four registers), and a fused step only up to radix 5 (three
// lines of 2 R registers of pairs); a plan with a last radix 6..kFusedMaxRadix
// has the last-radix-major spectrum of the scalar kernel's fused step, which
// the packed kernel's separate product would read in the wrong order.
template <class P> constexpr bool supported() {
  for (int s = 0; s < P::nst; ++s)
    if (P::rad[s] > 16) return false;
  return !fused_z(P::N, P::nst, P::Rl) || P::Rl <= kFusedMaxRadixShort;
}
template <class P> bool chosen(const MvpGeom& g, const float4* twzp) {
  if constexpr (!supported<P>()) return false;
  if (!twzp || g.f != 3 || !fits<P>()) return false;
  return g.tune.zkern < 0 ? worth<P>() && !(fused_z(P::N, P::nst, P::Rl) && P::N >= kFusedWideMinN)
                          : g.tune.zkern == 1;
}

template <class P>
cudaError_t launch(const MvpGeom& g, float2* t2, int L, const float4* twz, const float2* ghat, cudaStream_t st,
                   const int* done) {
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_pass_c_packed<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, kZSmemMax);
  });
  if (cfg != cudaSuccess) return cfg;
  const int per_warp = 3 * P::LW * (int)sizeof(ulonglong2);
  const int wpc = z_warps_per_cta(per_warp);
  const long long ntask = (long long)g.Px * g.Py * ((L + 1) / 2);
  const unsigned grid = (unsigned)((ntask + wpc - 1) / wpc);
  k_pass_c_packed<P><<<grid, wpc * 32, wpc * per_warp, st>>>(t2, L, g.Px, g.Py, g.nz, g.nzp, twz, ghat, done);
  return cudaGetLastError();
}

}  // namespace zpacked
}  // namespace bdda
