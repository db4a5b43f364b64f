// Strided passes (A, B, D, E) for complex FP32 with compile-time axis plans:
// the column-pair kernels of tile_passes.cuh instantiated for the plan of
// their axis length (x: tplans.inc, y: yplans.inc).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include <mutex>

#include "mvp.hpp"
#include "tile_passes.cuh"

namespace bdda {
namespace tstatic {

template <class K>
cudaError_t set_smem(K kernel, int bytes, std::once_flag& once, cudaError_t& cfg) {
  std::call_once(once, [&] { cfg = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes); });
  return cfg;
}

// x passes (A, E) with the plan of Px (tplans.inc)
template <class P>
cudaError_t launch_x(int pass, const TileArgs& a) {
  const MvpGeom& g = *a.g;
  const int max_nx = kMaxStaticLine / 2;
  // [2 buffers][8 columns][2 fields] lines + the occupancy of the tile
  auto smem_x2 = [](int nx) { return 4 * kTZ * P::LW * (int)sizeof(float2) + nx * kTZ * 4; };
  const int smem_ae = smem_x2(max_nx);
  int fpg = 0;
  const dim3 grid(g.ntiles, x_field_groups(a.nfield, g.ntiles, a.sms, &fpg, g.tune.xcta));
  static std::once_flag oa, oe;
  static cudaError_t ca = cudaSuccess, ce = cudaSuccess;
  cudaError_t e = cudaSuccess;
  if (pass == kTileA) {
    if ((e = set_smem(tile::k_pass_a2i<P>, smem_ae, oa, ca)) != cudaSuccess) return e;
    tile::k_pass_a2i<P><<<grid, kTileThreads, smem_x2(g.nx), a.st>>>(
        a.x, a.ldx, a.nfield, fpg, g.f, g.occ, g.tiles, g.nx, g.ny, g.nz, g.nzp, g.nzt, a.twx, a.t1, a.done);
  } else {
    if ((e = set_smem(tile::k_pass_e2i<P>, smem_ae, oe, ce)) != cudaSuccess) return e;
    tile::k_pass_e2i<P><<<grid, kTileThreads, smem_x2(g.nx), a.st>>>(
        a.t1, a.nfield, fpg, g.f, g.occ, g.tiles, g.nx, g.ny, g.nz, g.nzp, g.nzt, a.twx, a.x, a.ldx, a.diag, a.jpre, a.y,
        a.ldy, a.done);
  }
  return cudaGetLastError();
}

// y passes (B, D) with the plan of Py (yplans.inc: the radix sequence of
// tplans.inc, a layout for interleaved pairs and rows of eight pairs),
// double- or single-buffered (MvpTune::ybuf)
template <class P, int NBUF>
cudaError_t launch_y_buf(int pass, const TileArgs& a) {
  const MvpGeom& g = *a.g;
  const int smem_bd = NBUF * tile::kTZ2 * P::LW * (int)sizeof(float2);  // 16 columns per task and buffer
  const int ntask2 = a.nfield * g.Px * ((g.nz + tile::kTZ2 - 1) / tile::kTZ2);
  static std::once_flag ob, od;
  static cudaError_t cb = cudaSuccess, cd = cudaSuccess;
  static int resident[2] = {0, 0};  // CTAs of each kernel that fit on one SM
  cudaError_t e = cudaSuccess;
  // The grid is a whole number of waves of the CTAs resident at once (see
  // MvpTune::ywaves): a fixed 8 per SM left a partial last wave (1.1-1.6 waves).
  auto grid_of = [&](auto kernel, int inv) {
    if (resident[inv] == 0) {
      int nb = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kTileThreads, smem_bd) != cudaSuccess || nb < 1) nb = 1;
      resident[inv] = nb;
    }
    const int waves = (inv && g.tune.ywavesd > 0) ? g.tune.ywavesd : g.tune.ywaves;
    return std::min(ntask2, waves * resident[inv] * a.sms);
  };
  if (pass == kTileB) {
    if ((e = set_smem(tile::k_pass_y2i<false, P, NBUF>, smem_bd, ob, cb)) != cudaSuccess) return e;
    tile::k_pass_y2i<false, P, NBUF><<<grid_of(tile::k_pass_y2i<false, P, NBUF>, 0), kTileThreads, smem_bd, a.st>>>(
        a.t1, a.t2, g.tmask, g.ny, g.nz, g.nzp, g.nzt, ntask2, a.twy, a.done);
  } else {
    if ((e = set_smem(tile::k_pass_y2i<true, P, NBUF>, smem_bd, od, cd)) != cudaSuccess) return e;
    tile::k_pass_y2i<true, P, NBUF><<<grid_of(tile::k_pass_y2i<true, P, NBUF>, 1), kTileThreads, smem_bd, a.st>>>(
        a.t2, a.t1, g.tmask, g.ny, g.nz, g.nzp, g.nzt, ntask2, a.twy, a.done);
  }
  return cudaGetLastError();
}

template <class P>
cudaError_t launch_y(int pass, const TileArgs& a) {
  const int nbuf = (pass == kTileD && a.g->tune.ybufd > 0) ? a.g->tune.ybufd : a.g->tune.ybuf;
  return nbuf == 1 ? launch_y_buf<P, 1>(pass, a) : launch_y_buf<P, 2>(pass, a);
}

}  // namespace tstatic
}  // namespace bdda
