// Pipelined fused z pass (pass C) for complex FP32, f = 3.
//
// The same arithmetic as zstatic::k_pass_c_static (first forward stage, the
// other forward stages, the Green product -- fused with the last forward and
// first inverse stage where the plan allows, sfft::middle3 -- the inverse
// stages, the last inverse stage; static_fft.cuh, zproduct.cuh), run by
// persistent CTAs that keep every load of the compute phases in shared
// memory:
//
//  * each CTA takes the (x, y) lines blockIdx.x, blockIdx.x + gridDim.x, ...
//    and, for each line, all L right-hand sides in rounds of one task per
//    warp (right-hand side l goes to warp l mod nw);
//  * the line's Green spectrum (6 Pz values, 16-byte rows) is fetched by one
//    bulk copy into one of two spectrum buffers; the copy of line k + 2 is
//    issued by the last warp to finish its Green step of line k;
//  * each warp fetches the three component rows of its next task by bulk
//    copies into its staging rows as soon as its first stage has read the
//    current ones, so the DRAM latency of the rows overlaps the rest of the
//    current task;
//  * the staged twiddles are copied to shared memory once per CTA.
//
// The kernel's outputs are the in-place T2 rows (the last inverse stage
// writes global memory directly).  Every wait on a copy is bounded
// (async_copy.cuh); a wait that gives up sets *status = 1, the warp stops
// computing, waits (bounded) for the copies it issued and returns, and the
// host reports the error.  stall != 0 (test hook, bdda_op_test_z_stall):
// warp 0 of CTA 0 first waits on a barrier that nothing arrives on, so that
// path runs without a fault.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "async_copy.cuh"
#include "mvp.hpp"
#include "static_fft.cuh"
#include "zproduct.cuh"

namespace bdda {
namespace zpipe {

// Plans whose last stage, product and first inverse stage are one step (the
// complex FP32 spectrum is then last-radix-major, green_perm_radix).
template <class P> constexpr bool fused() { return fused_z(P::N, P::nst, P::Rl); }

// Staging row pitch (complex values): even (16-byte rows for the bulk copies)
// and congruent to the first stage's span M0 (or M0 + 1) modulo 16, so the
// lanes t = j M0 + n1 of a half-warp reading element n1 + i M0 of row j hit
// distinct banks.
template <class P> __host__ __device__ inline int stage_pitch(int nzp) {
  constexpr int M0 = P::N / P::rad[0];
  constexpr int Me = (M0 % 2) ? M0 + 1 : M0;
  return nzp + (((Me - nzp) % 16) + 16) % 16;
}

constexpr int kHeader = 128;  // barriers (kZWarps + 2) x 8 B, counters, the test barrier

template <class P> __host__ __device__ inline int tw_elems() { return (P::TWO(P::nst) + 1) & ~1; }

// Dynamic shared memory of a CTA of nw warps.
template <class P> __host__ __device__ inline size_t smem_bytes(int nw, int nzp) {
  return kHeader + sizeof(float2) * ((size_t)tw_elems<P>() + 2 * 6 * P::N + (size_t)nw * 3 * stage_pitch<P>(nzp) +
                                     (size_t)nw * 3 * P::LW);
}

template <class P>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c_pipe(float2* __restrict__ t2, int L, int nlines, int nz, int nzp, const float2* __restrict__ twz,
              const float2* __restrict__ ghat, const int* done, int* status, int stall) {
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  constexpr int Pz = P::N, LW = P::LW;
  const int nw = blockDim.x >> 5;  // warps = min(kZWarps, L), set by the host
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sp = stage_pitch<P>(nzp);
  uint64_t* xbar = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* gbar = xbar + kZWarps;
  int* gdone = reinterpret_cast<int*>(gbar + 2);  // [2] warps done with the spectrum buffer
  int* glast = gdone + 2;                         // [2] line whose spectrum was last issued into the buffer
  volatile int* abort_flag = glast + 2;
  uint64_t* tbar = reinterpret_cast<uint64_t*>(smem_raw + 104);  // never arrived on (test hook)
  float2* tws = reinterpret_cast<float2*>(smem_raw + kHeader);
  float2* gs = tws + tw_elems<P>();
  float2* stg = gs + 2 * 6 * Pz;
  float2* work = stg + (size_t)nw * 3 * sp;
  const int nk = (nlines - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;  // >= 1 (grid <= nlines)
  const size_t fstride = (size_t)nlines * nzp;
  const uint32_t xbytes = (uint32_t)((nz * (int)sizeof(float2) + 15) & ~15);  // <= nzp * 8
  const uint32_t gbytes = (uint32_t)(6 * Pz * sizeof(float2));
  auto line_of = [&](int k) { return (size_t)blockIdx.x + (size_t)k * gridDim.x; };
  auto rows = [&](int k, int l) { return t2 + (size_t)(3 * l) * fstride + line_of(k) * nzp; };
  auto issue_x = [&](int k, int l) {  // one lane
    float2* dst = stg + (size_t)warp * 3 * sp;
    const float2* src = rows(k, l);
    acp::expect_tx(&xbar[warp], 3 * xbytes);
    for (int c = 0; c < 3; ++c) acp::bulk_g2s(dst + c * sp, src + c * fstride, xbytes, &xbar[warp]);
  };
  auto issue_g = [&](int k) {  // one lane
    const int b = k & 1;
    glast[b] = k;
    acp::expect_tx(&gbar[b], gbytes);
    acp::bulk_g2s(gs + b * 6 * Pz, ghat + line_of(k) * 6 * Pz, gbytes, &gbar[b]);
  };
  if (threadIdx.x == 0) {
    for (int w = 0; w < kZWarps; ++w) acp::bar_init(&xbar[w], 1);
    acp::bar_init(&gbar[0], 1);
    acp::bar_init(&gbar[1], 1);
    acp::bar_init(tbar, 1);
    gdone[0] = gdone[1] = 0;
    glast[0] = glast[1] = -1;
    *abort_flag = 0;
    acp::fence_bar_init();
    issue_g(0);
    if (nk > 1) issue_g(1);
  }
  for (int i = threadIdx.x; i < P::TWO(P::nst); i += blockDim.x) tws[i] = twz[i];
  __syncthreads();

  float2* wl = work + (size_t)warp * 3 * LW;
  const float2* sl = stg + (size_t)warp * 3 * sp;
  int k = 0, l = warp;  // warp < nw <= L: every warp has a task in every line
  uint32_t xpar = 0;
  bool xpend = true;
  if (lane == 0) issue_x(0, warp);
  bool ok = true;
  if (stall && blockIdx.x == 0 && warp == 0) ok = __all_sync(0xffffffffu, acp::wait(tbar, 0));  // gives up
  while (ok && k < nk) {
    ok = __all_sync(0xffffffffu, !*abort_flag && acp::wait(&xbar[warp], xpar));
    if (!ok) break;
    xpend = false;
    xpar ^= 1u;
    sfft::stage0_from_global<P, 3, float2, true>(wl, tws, lane, nz, sl, (size_t)sp);
    int k2 = k, l2 = l + nw;
    if (l2 >= L) {
      ++k2;
      l2 = warp;
    }
    if (k2 < nk) {  // the staging rows are free again: fetch the next task's rows
      if (lane == 0) {
        acp::fence_proxy_async();
        issue_x(k2, l2);
      }
      xpend = true;
    }
    sfft::forward_to<P, 3, 1, fused<P>() ? P::nst - 1 : P::nst, float2, true>(wl, tws, lane, nz);
    ok = __all_sync(0xffffffffu, !*abort_flag && acp::wait(&gbar[k & 1], (uint32_t)((k >> 1) & 1)));
    if (!ok) break;
    const float2* gl = gs + (k & 1) * 6 * Pz;
    if constexpr (fused<P>()) {
      sfft::middle3<P, float2, true>(wl, gl, lane);
    } else {
      for (int p = lane; p < Pz; p += 32) z_product<float2, true>(wl, LW, P::addr(p), gl, Pz, p, false);
      __syncwarp();
    }
    if (l + nw >= L && lane == 0) {  // this warp's last Green step of line k
      __threadfence_block();         // its reads of the spectrum buffer before the count
      if (atomicAdd(&gdone[k & 1], 1) == nw - 1) {
        __threadfence_block();       // every warp's reads before the refill
        gdone[k & 1] = 0;
        if (k + 2 < nk && !*abort_flag) {
          acp::fence_proxy_async();
          issue_g(k + 2);
        }
      }
    }
    sfft::inverse<P, 3, fused<P>() ? P::nst - 2 : P::nst - 1, 1, float2, true>(wl, tws, lane, nz);
    sfft::stage0_to_global<P, 3, float2, true>(wl, tws, lane, nz, rows(k, l), fstride);
    k = k2;
    l = l2;
  }
  if (!ok) {
    *abort_flag = 1;
    if (lane == 0) {
      atomicExch(status, 1);
      // the copies this warp may have in flight: its staging rows, and the spectra
      if (xpend) acp::wait(&xbar[warp], xpar);
      for (int b = 0; b < 2; ++b) {
        const int kb = ((volatile int*)glast)[b];
        if (kb >= 0) acp::wait(&gbar[b], (uint32_t)((kb >> 1) & 1));
      }
    }
    __syncwarp();
  }
}

// Launches the pipelined kernel; false (nothing launched) where it does not
// apply: f = 6, no status word, a CTA's shared memory above the limit, or --
// under the default rule (MvpTune::zkern < 0) -- less than two CTAs per SM
// (the autotuner may still pick it with one).
template <class P>
bool launch(const MvpGeom& g, float2* t2, int L, const float2* twz, const float2* ghat, cudaStream_t st,
            const int* done, cudaError_t* err) {
  if (g.f != 3 || !g.kstat || g.gperm != (fused<P>() ? P::Rl : 0)) return false;
  const int nw = L < kZWarps ? L : kZWarps;
  const size_t bytes = smem_bytes<P>(nw, g.nzp);
  if (bytes > (size_t)(g.tune.zkern == 2 ? kZSmemMax : kZSmemMax / 2)) return false;
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  static int nsm = 0;
  std::call_once(once, [] {
    cfg = cudaFuncSetAttribute(k_pass_c_pipe<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, kZSmemMax);
    int dev = 0;
    if (cfg == cudaSuccess) cfg = cudaGetDevice(&dev);
    if (cfg == cudaSuccess) cfg = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  });
  if (cfg != cudaSuccess) {
    *err = cfg;
    return true;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass_c_pipe<P>, nw * 32, bytes);
  if (e != cudaSuccess || per_sm < 1) {
    *err = e != cudaSuccess ? e : cudaErrorInvalidConfiguration;
    return true;
  }
  const long long nlines = (long long)g.Px * g.Py;
  const long long grid = std::min<long long>(nlines, (long long)per_sm * nsm);
  k_pass_c_pipe<P><<<(unsigned)grid, nw * 32, bytes, st>>>(t2, L, (int)nlines, g.nz, g.nzp, twz, ghat, done, g.kstat,
                                                             g.zstall);
  *err = cudaGetLastError();
  return true;
}

}  // namespace zpipe
}  // namespace bdda
