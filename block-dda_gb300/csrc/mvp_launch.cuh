// Fused block-MVP passes: y = [diag o x +] A_off x  [o jpre], all RHS at once.
//
// Replaces the reference's per-RHS chain scatter -> BT_pad -> FFTW fwd ->
// Au_til product -> FFTW inv -> BT_reconstruct -> gather -> DIAG add -> jpre
// (mvp_fft/MBT_fft_mvp.cpp:19-32, bl_krylov_mvp_fft/bl_cocg_rq_jacobi_mvp_fft.cpp:43-60)
// by the mathematically identical 2x-padded 3-D FFT convolution with the
// 6-component symmetric Green tensor (f = 3; f = 6 adds the magnetic dipoles
// and the 3-component antisymmetric coupling).  Fields are the f*L
// (component, RHS) pairs; field = f*l + c.
//
// HBM layouts (element = complex T):
//   x, y   : column-major (rows f*m + c, column l, leading dimension ld) --
//            the reference's Eigen layout of S / AS.
//   occ    : int32 [nx][ny][nz], dipole index of a lattice site or -1.
//   tiles  : int32 list of (y, z-tile) pairs (y*nzt + zt, 8-wide z tiles)
//            holding >= 1 dipole; tmask [ny][nzt] marks them.
//   T1     : [3L][Px][ny][nzp] after the x pass (only rows of listed tiles valid)
//   T2     : [3L][Px][Py][nzp] after the y pass; the z pass works in place
//            (nzp = nz rounded up to a multiple of 4: rows of complex FP32
//            start on 32-byte sectors; the padding is never read)
//   Ghat   : [Px][Py][6][Pz]  Ghat / (Px Py Pz), digit-reversed frequencies,
//            components (xx, xy, xz, yy, yz, zz).
//
// Passes (forward x, y; fused z; inverse y, x), each one kernel:
//   A  x-forward, gathers the occupied sites of a (y, z-tile), loops over
//      the fields; input pruned to nx                       x  -> T1
//   B  y-forward, rows of empty tiles never read, pruned to ny     T1 -> T2
//   C  z-forward (pruned to nz), 3x3 symmetric Ghat product, z-inverse,
//      output truncated to nz; one warp per (x, y, rhs) holds the three
//      components, no block barrier                          T2 -> T2
//   D  y-inverse, rows y < ny of listed tiles written        T2 -> T1
//   E  x-inverse, scatter to occupied sites, + diag o x, o jpre    T1 -> y
// The strided passes stage 8 z-columns per CTA; B, D and E prefetch the next
// tile with cp.async (zero-filled outside the box) while the current one is
// transformed.
#pragma once

#include <algorithm>
#include <type_traits>

#include "fft_core.cuh"

#include "mvp.hpp"
#include "tile_passes.cuh"
#include "zproduct.cuh"

namespace bdda {

namespace {

__device__ __forceinline__ bool skip(const int* done) { return done && *(volatile const int*)done; }

// ---------------------------------------------------------------- pass C
// One warp per task (x = q, y = qy, rhs l): the fc = 3 (E) or 6 (E, M)
// component lines along z, transformed three at a time; blockDim.x / 32
// warps per CTA.
template <typename T>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c(typename cplx<T>::type* __restrict__ t2, int L, int fc, int Px, int Py, int nz, int nzp, AxisPlan pz,
         const typename cplx<T>::type* __restrict__ twz, const typename cplx<T>::type* __restrict__ ghat, int gperm,
         const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Pz = pz.N;
  const int lw = plan_lw<C>(pz), sh = plan_sk<C>(pz);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long task = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  const long long ntask = (long long)Px * Py * L;
  if (task >= ntask) return;
  const int l = (int)(task % L);
  const long long line = task / L;  // q * Py + qy
  C* s0 = reinterpret_cast<C*>(smem_raw) + (size_t)warp * fc * lw;
  const size_t fstride = (size_t)Px * Py * nzp;  // between fields
  C* g0 = t2 + (size_t)(fc * l) * fstride + (size_t)line * nzp;
  const bool six = fc == 6;
  for (int z = lane; z < nz; z += 32) {
    const int a = skw(z, sh);
    for (int c = 0; c < fc; ++c) s0[c * lw + a] = g0[c * fstride + z];
  }
  __syncwarp();
  const int halves = six ? 2 : 1;  // line triples: E, then M
  for (int h = 0; h < halves; ++h) warp_fft_lines<false, 3>(s0 + 3 * h * lw, lw, twz, pz, lane, 32, nz);
  const C* gl = ghat + (size_t)line * (six ? 9 : 6) * Pz;
  for (int p = lane; p < Pz; p += 32) z_product(s0, lw, skw(p, sh), gl, Pz, green_pos(p, Pz, gperm), six);
  __syncwarp();
  for (int h = 0; h < halves; ++h) warp_fft_lines<true, 3>(s0 + 3 * h * lw, lw, twz, pz, lane);
  for (int z = lane; z < nz; z += 32) {
    const int a = skw(z, sh);
    for (int c = 0; c < fc; ++c) g0[c * fstride + z] = s0[c * lw + a];
  }
}


int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

}  // namespace

// ---------------------------------------------------------------- launcher
template <typename T>
cudaError_t launch_block_mvp(const MvpGeom& g, const MvpPrec<T>& p, const typename cplx<T>::type* x, int ldx,
                             typename cplx<T>::type* y, int ldy, int L,
                             const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre,
                             typename cplx<T>::type* t1, typename cplx<T>::type* t2,
                             cudaStream_t st, KernelTimer* timer, const int* done) {
  using C = typename cplx<T>::type;
  const int nfield = g.f * L;
  const int pbase = sizeof(T) == sizeof(double) ? (kPassA64 - kPassA) : 0;
  if (g.ntiles == 0) return cudaSuccess;  // no dipoles
  const int ntask_y = nfield * g.Px * g.nzt;
  // runtime-plan y passes: kYWaves waves of the CTAs resident per SM
  auto grid_y = [&](auto kernel, int smem) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kTileThreads, smem) != cudaSuccess || nb < 1) nb = 1;
    return std::min(ntask_y, g.tune.ywaves * nb * num_sms());
  };
  const tile::RtLine<C> lx{g.px}, ly{g.py};
  // runtime-plan strided passes: tile buffers and shared memory -- one buffer
  // where two would not fit (long lines of 16-byte elements).  Single
  // buffering where two fit was measured no faster for the double-float y
  // passes (N=65536, Py=270: 14.6 / 14.3 vs 14.3 / 14.0 ms).
  const int xbuf = tile::tile_buffers<T>(plan_lw<C>(g.px), g.nx), ybuf = tile::tile_buffers<T>(plan_lw<C>(g.py), 0);
  const int xsm = tile::smem_tile<T>(plan_lw<C>(g.px), g.nx, xbuf), ysm = tile::smem_tile<T>(plan_lw<C>(g.py), 0, ybuf);
  int xfpg = 0;  // x passes: fields per CTA
  const dim3 xgrid(g.ntiles, x_field_groups(nfield, g.ntiles, num_sms(), &xfpg, g.tune.xcta));
  const bool runA = g.passes & 1u, runB = g.passes & 2u, runC = g.passes & 4u, runD = g.passes & 8u,
             runE = g.passes & 16u;
  // Strided pass `pass` with the compile-time plan of its axis (complex FP32);
  // false when it was not launched that way.
  cudaError_t serr = cudaSuccess;
  auto static_tile = [&](int pass) -> bool {
    if constexpr (std::is_same<T, float>::value) {
      const TileArgs a{&g, x, ldx, y, ldy, nfield, diag, jpre, t1, t2, p.twxs, p.twys, num_sms(), st, done};
      cudaError_t e = cudaSuccess;
      const bool ok = launch_tile_static(pass, a, &e);
      if (ok && e != cudaSuccess) serr = e;
      return ok;
    } else {
      (void)pass;
      return false;
    }
  };
  // A
  if (runA && timer) timer->begin(kPassA + pbase, st);
  if (runA && !static_tile(kTileA))
    tile::k_pass_a<T><<<xgrid, kTileThreads, xsm, st>>>(
        x, ldx, nfield, xfpg, g.f, g.occ, g.tiles, g.nx, g.ny, g.nz, g.nzp, g.nzt, lx, p.twx, t1, xbuf, done);
  if (runA && timer) timer->end(kPassA + pbase, st);
  if (serr != cudaSuccess) return serr;
  // B
  if (runB && timer) timer->begin(kPassB + pbase, st);
  if (runB && !static_tile(kTileB))
    tile::k_pass_y<T, false><<<grid_y(tile::k_pass_y<T, false, tile::RtLine<C>>, ysm), kTileThreads, ysm, st>>>(
        t1, t2, g.tmask, g.ny, g.nz, g.nzp, g.nzt, ntask_y, ly, p.twy, ybuf, done);
  if (runB && timer) timer->end(kPassB + pbase, st);
  if (serr != cudaSuccess) return serr;
  // C
  if (runC) {
    const long long ntask = (long long)g.Px * g.Py * L;
    if (timer) timer->begin(kPassC + pbase, st);
    bool launched = false;
    if constexpr (std::is_same<T, float>::value) {
      cudaError_t e = cudaSuccess;
      launched = launch_pass_c_static(g, t2, L, p.twzs, p.twzps, p.ghat, st, done, &e);
      if (launched && e != cudaSuccess) return e;
    } else if constexpr (std::is_same<T, dfz>::value) {
      cudaError_t e = cudaSuccess;
      launched = launch_pass_c_static_df(g, t2, L, p.twzs, p.ghat, st, done, &e);
      if (launched && e != cudaSuccess) return e;
    }
    if (!launched) {
      const int per_warp = g.f * plan_lw<C>(g.pz) * (int)sizeof(C);
      const int wpc = z_warps_per_cta(per_warp);
      const unsigned grid = (unsigned)((ntask + wpc - 1) / wpc);
      k_pass_c<T><<<grid, wpc * 32, wpc * per_warp, st>>>(t2, L, g.f, g.Px, g.Py, g.nz, g.nzp, g.pz, p.twz, p.ghat,
                                                           g.gperm, done);
    }
    if (timer) timer->end(kPassC + pbase, st);
  }
  // D
  if (runD && timer) timer->begin(kPassD + pbase, st);
  if (runD && !static_tile(kTileD))
    tile::k_pass_y<T, true><<<grid_y(tile::k_pass_y<T, true, tile::RtLine<C>>, ysm), kTileThreads, ysm, st>>>(
        t2, t1, g.tmask, g.ny, g.nz, g.nzp, g.nzt, ntask_y, ly, p.twy, ybuf, done);
  if (runD && timer) timer->end(kPassD + pbase, st);
  if (serr != cudaSuccess) return serr;
  // E
  if (runE && timer) timer->begin(kPassE + pbase, st);
  if (runE && !static_tile(kTileE))
    tile::k_pass_e<T><<<xgrid, kTileThreads, xsm, st>>>(
        t1, nfield, xfpg, g.f, g.occ, g.tiles, g.nx, g.ny, g.nz, g.nzp, g.nzt, lx, p.twx, x, ldx, diag, jpre, y, ldy, xbuf,
        done);
  if (runE && timer) timer->end(kPassE + pbase, st);
  if (serr != cudaSuccess) return serr;
  return cudaGetLastError();
}

template <typename T>
cudaError_t configure_mvp_kernels() {
  using C = typename cplx<T>::type;
  using Rt = tile::RtLine<C>;
  const int ts = std::min(tile::smem_tile<T>(kMaxLineWords, kMaxLine / 2), kZSmemMax);
  const int zs = kZSmemMax;
  const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(tile::k_pass_a<T, Rt>, attr, ts)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(tile::k_pass_e<T, Rt>, attr, ts)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(tile::k_pass_y<T, false, Rt>, attr, ts)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(tile::k_pass_y<T, true, Rt>, attr, ts)) != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_pass_c<T>, attr, zs);
}

}  // namespace bdda
