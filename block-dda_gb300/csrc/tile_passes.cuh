// Strided passes of the block MVP (A: x-forward gather, B: y-forward,
// D: y-inverse, E: x-inverse scatter).
//
// k_pass_a / k_pass_y / k_pass_e: runtime axis plans (fft_core.cuh, skewed
// layout of the plan; every precision).  A CTA stages 8 z-columns (one line
// per warp) of one tile in shared memory; forward transforms read only the
// first nv inputs.
// k_pass_a2i / k_pass_y2i / k_pass_e2i: compile-time plans (static_fft.cuh,
// padded layout; complex FP32).  Each warp transforms two adjacent z-columns
// at once, interleaved element by element in shared memory, so the padded
// T1 / T2 rows are staged and stored one 16-byte column pair per copy;
// inverse transforms write only the first nv outputs.
#pragma once

#include <cuda_runtime.h>

#include "fft_core.cuh"
#include "mvp.hpp"
#include "static_fft.cuh"

namespace bdda {
namespace tile {

template <typename C>
struct RtLine {
  AxisPlan p;
  __device__ __forceinline__ int n() const { return p.N; }
  __device__ __forceinline__ int lw() const { return plan_lw<C>(p); }
  __device__ __forceinline__ int addr(int i) const { return skw(i, plan_sk<C>(p)); }
  template <bool INV>
  __device__ __forceinline__ void fft(C* line, const C* tw, int lane, int nv) const {
    if (!INV) warp_fft_lines<false, 1>(line, 0, tw, p, lane, 32, nv);
    else warp_fft_lines<true, 1>(line, 0, tw, p, lane);
  }
};


// ---- cp.async helpers (LDGSTS: global -> shared without registers) --------
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int sz = valid ? BYTES : 0;  // src-size 0: nothing read, destination zero-filled
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async sizes");
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(BYTES), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ bool skip(const int* done) { return done && *(volatile const int*)done; }

// Rows of a tile one thread visits: rows r, r + kRowStep, ... in column tid % kTZ.
constexpr int kRowStep = kTileThreads / kTZ;

// ---------------------------------------------------------------- pass A
// One CTA per listed (y, z-tile): warp w owns z = z0 + w; loops over fields.
template <typename T, class Line>
__global__ void __launch_bounds__(kTileThreads)
k_pass_a(const typename cplx<T>::type* __restrict__ x, int ldx, int nfield, int fpg, int fc, const int* __restrict__ occ,
         const int* __restrict__ tiles, int nx, int ny, int nz, int nzp, int nzt, Line lay,
         const typename cplx<T>::type* __restrict__ twx, typename cplx<T>::type* __restrict__ t1, int nbuf,
         const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Px = lay.n();
  const int lw = lay.lw();
  C* lines = reinterpret_cast<C*>(smem_raw);                       // [nbuf][kTZ][lw]
  int* socc = reinterpret_cast<int*>(lines + nbuf * kTZ * lw);     // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int y = tile / nzt, z0 = (tile - y * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tw8 = tid & (kTZ - 1), tq = tid / kTZ;  // tile column and first row of this thread
  const bool zval = z0 + tw8 < nz;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + y) * nz + z] : -1;
  }
  __syncthreads();
  const size_t rowstride = (size_t)ny * nzp;  // T1 stride between x rows
  const int f0 = blockIdx.y * fpg, fend = min(nfield, f0 + fpg);  // this CTA's fields (f0 even)
  int l = f0 / fc, c = f0 - (f0 / fc) * fc;
  for (int f = f0; f < fend; ++f) {
    const int buf = nbuf == 2 ? (f & 1) : 0;
    C* line = lines + (buf * kTZ + warp) * lw;
    const C* xc = x + (size_t)l * ldx + c;
    for (int xi = lane; xi < nx; xi += 32) {
      const int m = socc[xi * kTZ + warp];
      line[lay.addr(xi)] = m >= 0 ? xc[fc * (size_t)m] : czero<C>();
    }
    __syncwarp();
    lay.template fft<false>(line, twx, lane, nx);
    __syncthreads();
    // drain: thread tid writes column w = tid % 8 of rows q = tid / 8 + 32 k
    if (zval) {
      const C* lb = lines + (buf * kTZ + tw8) * lw;
      C* out = t1 + (size_t)f * Px * rowstride + (size_t)y * nzp + z0 + tw8 + (size_t)tq * rowstride;
      for (int q = tq; q < Px; q += kRowStep, out += kRowStep * rowstride) *out = lb[lay.addr(q)];
    }
    if (nbuf == 1) __syncthreads();  // the next field's gather overwrites the drained buffer
    if (++c == fc) { c = 0; ++l; }
  }
}

// ---------------------------------------------------------------- pass B / D
// Persistent CTAs over tasks (field, x, z-tile); lines along y.
// B: T1[f][q][y<ny][z] -> T2[f][q][Py][z]   (rows of empty tiles zero-filled)
// D: T2[f][q][Py][z]   -> T1[f][q][y<ny][z] (rows of listed tiles only)
template <typename T, bool INV, class Line>
__global__ void __launch_bounds__(kTileThreads)
k_pass_y(const typename cplx<T>::type* __restrict__ src, typename cplx<T>::type* __restrict__ dst,
         const unsigned char* __restrict__ tmask, int ny, int nz, int nzp, int nzt, int ntask, Line lay,
         const typename cplx<T>::type* __restrict__ twy, int nbuf, const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Py = lay.n();
  const int lw = lay.lw();
  C* lines = reinterpret_cast<C*>(smem_raw);  // [nbuf][kTZ][lw]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nin = INV ? Py : ny;    // rows read
  const int nout = INV ? ny : Py;   // rows written
  const size_t in_rows = (size_t)nin, out_rows = (size_t)nout;

  const int tw8 = tid & (kTZ - 1), ty = tid / kTZ;  // tile column and first row of this thread
  // fill: thread tid loads column w = tid % 8 of rows yy = tid / 8 + 32 k (zero-filled outside the data)
  auto issue = [&](int task, int buf) {
    const int zt = task % nzt;
    const int r = task / nzt;  // f * Px + q
    const int z0 = zt * kTZ;
    const bool zval = z0 + tw8 < nz;
    const C* g = src + (size_t)r * in_rows * nzp + z0 + tw8 + (size_t)ty * nzp;
    const unsigned char* tm = tmask + zt + (size_t)ty * nzt;
    C* lb = lines + (buf * kTZ + tw8) * lw;
    for (int yy = ty; yy < nin; yy += kRowStep, g += (size_t)kRowStep * nzp, tm += (size_t)kRowStep * nzt) {
      const bool valid = zval && (INV || *tm);
      cp_async<sizeof(C)>(lb + lay.addr(yy), valid ? g : src, valid);
    }
    cp_commit();
  };

  int task = blockIdx.x;
  if (nbuf == 2 && task < ntask) issue(task, 0);
  for (int it = 0; task < ntask; ++it, task += gridDim.x) {
    const int buf = nbuf == 2 ? (it & 1) : 0;
    const int next = task + gridDim.x;
    if (nbuf == 1) {
      issue(task, 0);
      cp_wait<0>();
    } else if (next < ntask) {
      issue(next, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    C* line = lines + (buf * kTZ + warp) * lw;
    lay.template fft<INV>(line, twy, lane, ny);
    __syncthreads();
    const int zt = task % nzt;
    const int r = task / nzt;
    const int z0 = zt * kTZ;
    if (z0 + tw8 < nz) {
      C* ob = dst + (size_t)r * out_rows * nzp + z0 + tw8 + (size_t)ty * nzp;
      const unsigned char* tm = tmask + zt + (size_t)ty * nzt;
      const C* lb = lines + (buf * kTZ + tw8) * lw;
      for (int yy = ty; yy < nout; yy += kRowStep, ob += (size_t)kRowStep * nzp, tm += (size_t)kRowStep * nzt)
        if (!INV || *tm) *ob = lb[lay.addr(yy)];
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of the next-but-one task
  }
}

// ---------------------------------------------------------------- static-plan tiles
// The complex FP32 passes with compile-time plans process 16 z-columns (y
// passes) or 8 (x passes) per task as column pairs.
constexpr int kTZ2 = 2 * kTZ;

// ---------------------------------------------------------------- pass E
// One CTA per listed (y, z-tile); loops over fields with the next field's
// tile prefetched by cp.async; scatters the occupied sites.
// ---------------------------------------------------------------- pass B / D, column pairs
// Persistent CTAs over tasks (field, x, 16-column z tile); lines along y.
// Warp w transforms columns 2w and 2w + 1 as one line pair interleaved
// element by element in shared memory (sfft::stage_il), so the tile is
// staged and stored one column pair -- 16 contiguous bytes, since rows are
// padded to a multiple of 4 elements -- per copy (a copy per column left the
// warps stalled on the shared-memory queue).  A pair whose second column is
// row padding transforms it and never stores it.  NBUF = 2: the next task's
// tile is prefetched by cp.async into the second buffer while the current one
// is transformed; NBUF = 1: one buffer, so twice the CTAs fit on an SM
// (the autotuner picks; N=65536, Py=270: 3.28 -> 2.57 ms forward with one
// buffer, Py=160: 0.254 -> 0.267 ms).
constexpr int kPairsY = kTZ2 / 2;
constexpr int kRowStepP = kTileThreads / kPairsY;

template <bool INV, class P, int NBUF = 2>
__global__ void __launch_bounds__(kTileThreads)
k_pass_y2i(const float2* __restrict__ src, float2* __restrict__ dst, const unsigned char* __restrict__ tmask, int ny,
           int nz, int nzp, int nzt, int ntask, const float2* __restrict__ twy, const int* done) {
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Py = P::N, lw = P::LW;
  float2* tile = reinterpret_cast<float2*>(smem_raw);  // [NBUF][kPairsY][lw][2]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nin = INV ? Py : ny;
  const int nout = INV ? ny : Py;
  const int nzt2 = (nz + kTZ2 - 1) / kTZ2;
  const int tp = tid & (kPairsY - 1), ty = tid / kPairsY;  // column pair and first row of this thread
  auto issue = [&](int task, int buf) {
    const int zt2 = task % nzt2;
    const int r = task / nzt2;  // f * Px + q
    const int z = zt2 * kTZ2 + 2 * tp;
    const bool zval = z < nz;
    const float2* g = src + (size_t)r * nin * nzp + z + (size_t)ty * nzp;
    const unsigned char* tm = tmask + (zval ? z / kTZ : 0) + (size_t)ty * nzt;
    float2* lb = tile + (size_t)(buf * kPairsY + tp) * lw * 2;
    for (int yy = ty; yy < nin; yy += kRowStepP, g += (size_t)kRowStepP * nzp, tm += (size_t)kRowStepP * nzt) {
      const bool valid = zval && (INV || *tm);
      cp_async<16>(lb + 2 * P::addr(yy), valid ? g : src, valid);
    }
    cp_commit();
  };
  int task = blockIdx.x;
  if (NBUF == 2 && task < ntask) issue(task, 0);
  for (int it = 0; task < ntask; ++it, task += gridDim.x) {
    const int buf = NBUF == 2 ? (it & 1) : 0;
    const int next = task + gridDim.x;
    if (NBUF == 1) {
      issue(task, 0);
      cp_wait<0>();
    } else if (next < ntask) {
      issue(next, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    float2* wl = tile + (size_t)(buf * kPairsY + warp) * lw * 2;
    if (!INV) sfft::forward_il<P>(wl, twy, lane, ny);
    else sfft::inverse_il<P>(wl, twy, lane, ny);
    __syncthreads();
    const int zt2 = task % nzt2;
    const int r = task / nzt2;
    const int z = zt2 * kTZ2 + 2 * tp;
    if (z < nz) {
      float4* ob = reinterpret_cast<float4*>(dst + (size_t)r * nout * nzp + z + (size_t)ty * nzp);
      const unsigned char* tm = tmask + z / kTZ + (size_t)ty * nzt;
      const float4* lb = reinterpret_cast<const float4*>(tile + (size_t)(buf * kPairsY + tp) * lw * 2);
      for (int yy = ty; yy < nout; yy += kRowStepP, ob += (size_t)kRowStepP * nzp / 2, tm += (size_t)kRowStepP * nzt)
        if (!INV || *tm) *ob = lb[P::addr(yy)];
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of the next-but-one task (next task, NBUF = 1)
  }
}

template <typename T, class Line>
__global__ void __launch_bounds__(kTileThreads)
k_pass_e(const typename cplx<T>::type* __restrict__ t1, int nfield, int fpg, int fc, const int* __restrict__ occ,
         const int* __restrict__ tiles, int nx, int ny, int nz, int nzp, int nzt, Line lay,
         const typename cplx<T>::type* __restrict__ twx, const typename cplx<T>::type* __restrict__ x, int ldx,
         const typename cplx<T>::type* __restrict__ diag, const typename cplx<T>::type* __restrict__ jpre,
         typename cplx<T>::type* __restrict__ y, int ldy, int nbuf, const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Px = lay.n();
  const int lw = lay.lw();
  C* lines = reinterpret_cast<C*>(smem_raw);                       // [nbuf][kTZ][lw]
  int* socc = reinterpret_cast<int*>(lines + nbuf * kTZ * lw);     // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int yy = tile / nzt, z0 = (tile - yy * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t rowstride = (size_t)ny * nzp;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + yy) * nz + z] : -1;
  }
  const int tw8 = tid & (kTZ - 1), tq = tid / kTZ;  // tile column and first row of this thread
  const bool zval = z0 + tw8 < nz;
  // fill: thread tid loads column w = tid % 8 of rows q = tid / 8 + 32 k (zero-filled past nz)
  auto issue = [&](int f, int buf) {
    const C* g = t1 + (size_t)f * Px * rowstride + (size_t)yy * nzp + z0 + tw8 + (size_t)tq * rowstride;
    C* lb = lines + (buf * kTZ + tw8) * lw;
    for (int q = tq; q < Px; q += kRowStep, g += (size_t)kRowStep * rowstride)
      cp_async<sizeof(C)>(lb + lay.addr(q), zval ? g : t1, zval);
    cp_commit();
  };
  const int f0 = blockIdx.y * fpg, fend = min(nfield, f0 + fpg);  // this CTA's fields (f0 even)
  if (nbuf == 2) issue(f0, 0);
  int l = f0 / fc, c = f0 - (f0 / fc) * fc;
  for (int f = f0; f < fend; ++f) {
    const int buf = nbuf == 2 ? (f & 1) : 0;
    if (nbuf == 1) {
      issue(f, 0);
      cp_wait<0>();
    } else if (f + 1 < fend) {
      issue(f + 1, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    C* line = lines + (buf * kTZ + warp) * lw;
    lay.template fft<true>(line, twx, lane, nx);
    for (int xi = lane; xi < nx; xi += 32) {
      const int m = socc[xi * kTZ + warp];
      if (m < 0) continue;
      const size_t r = fc * (size_t)m + c;
      C v = line[lay.addr(xi)];
      if (diag != nullptr) v = cadd(v, cmul(diag[r], x[(size_t)l * ldx + r]));
      if (jpre != nullptr) v = cmul(v, jpre[r]);
      y[(size_t)l * ldy + r] = v;
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of field f + 2
    if (++c == fc) { c = 0; ++l; }
  }
}

// ---------------------------------------------------------------- pass A / E, column pairs
// One CTA per listed (y, 8-column z tile), looping over the fields two at a
// time: warp (pair p, half h) transforms columns 2p and 2p + 1 of field f + h
// as one interleaved line pair (sfft::stage_il), and T1 rows are drained (A)
// and filled (E) one column pair -- 16 aligned bytes in the padded rows -- per
// copy.  Lines: [2 buffers][2 fields][4 pairs][LW][2].
constexpr int kPairsX = kTZ / 2;
constexpr int kRowStepX = kTileThreads / kPairsX;

template <class P>
__device__ __forceinline__ float2* x2i_block(float2* lines, int buf, int h, int p) {
  return lines + (size_t)((buf * 2 + h) * kPairsX + p) * P::LW * 2;
}

template <class P>
__global__ void __launch_bounds__(kTileThreads)
k_pass_a2i(const float2* __restrict__ x, int ldx, int nfield, int fpg, int fc, const int* __restrict__ occ,
           const int* __restrict__ tiles, int nx, int ny, int nz, int nzp, int nzt, const float2* __restrict__ twx,
           float2* __restrict__ t1, const int* done) {
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Px = P::N;
  float2* lines = reinterpret_cast<float2*>(smem_raw);
  int* socc = reinterpret_cast<int*>(lines + 4 * kTZ * P::LW);  // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int y = tile / nzt, z0 = (tile - y * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wp = warp & (kPairsX - 1), wh = warp / kPairsX;  // this warp's column pair and field half
  const int tp = tid & (kPairsX - 1), tq = tid / kPairsX;     // drain: column pair and first row
  const bool pval = z0 + 2 * tp < nz;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + y) * nz + z] : -1;
  }
  __syncthreads();
  const size_t rowstride = (size_t)ny * nzp;
  const int fend = min(nfield, (blockIdx.y + 1) * fpg);  // this CTA's fields: [blockIdx.y fpg, fend)
  // The gathered sites of a warp's column pair (element t = 2 xi + column,
  // t < 2 nx <= Px) are loaded into registers one field pair ahead: the loads
  // of field f + 2 are in flight while field f is transformed and drained.
  constexpr int kPre = (Px + 31) / 32;
  float2 pre[kPre];
  auto gather = [&](int fh) {
    const int l = fh / fc, c = fh - l * fc;
    const float2* xc = x + (size_t)l * ldx + c;
#pragma unroll
    for (int j = 0; j < kPre; ++j) {
      const int t = lane + 32 * j;
      const int m = t < 2 * nx ? socc[(t >> 1) * kTZ + 2 * wp + (t & 1)] : -1;
      pre[j] = m >= 0 ? xc[fc * (size_t)m] : make_float2(0.f, 0.f);
    }
  };
  if (blockIdx.y * fpg + wh < fend) gather(blockIdx.y * fpg + wh);
  for (int f = blockIdx.y * fpg, it = 0; f < fend; f += 2, ++it) {
    const int buf = it & 1;
    const int nh = f + 1 < fend ? 2 : 1;
    if (wh < nh) {
      float2* blk = x2i_block<P>(lines, buf, wh, wp);
#pragma unroll
      for (int j = 0; j < kPre; ++j) {
        const int t = lane + 32 * j;
        if (t < 2 * nx) blk[2 * P::addr(t >> 1) + (t & 1)] = pre[j];
      }
      __syncwarp();
      if (f + 2 + wh < fend) gather(f + 2 + wh);
      sfft::forward_il<P>(blk, twx, lane, nx);
    }
    __syncthreads();
    if (pval) {
      for (int h = 0; h < nh; ++h) {
        const float4* lb = reinterpret_cast<const float4*>(x2i_block<P>(lines, buf, h, tp));
        float4* out = reinterpret_cast<float4*>(t1 + (size_t)(f + h) * Px * rowstride + (size_t)y * nzp + z0 + 2 * tp +
                                                (size_t)tq * rowstride);
        for (int q = tq; q < Px; q += kRowStepX, out += kRowStepX * rowstride / 2) *out = lb[P::addr(q)];
      }
    }
  }
}

template <class P>
__global__ void __launch_bounds__(kTileThreads)
k_pass_e2i(const float2* __restrict__ t1, int nfield, int fpg, int fc, const int* __restrict__ occ,
           const int* __restrict__ tiles, int nx, int ny, int nz, int nzp, int nzt, const float2* __restrict__ twx,
           const float2* __restrict__ x, int ldx, const float2* __restrict__ diag, const float2* __restrict__ jpre,
           float2* __restrict__ y, int ldy, const int* done) {
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int Px = P::N;
  float2* lines = reinterpret_cast<float2*>(smem_raw);
  int* socc = reinterpret_cast<int*>(lines + 4 * kTZ * P::LW);  // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int yy = tile / nzt, z0 = (tile - yy * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wp = warp & (kPairsX - 1), wh = warp / kPairsX;
  const int tp = tid & (kPairsX - 1), tq = tid / kPairsX;
  const bool pval = z0 + 2 * tp < nz;
  const size_t rowstride = (size_t)ny * nzp;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + yy) * nz + z] : -1;
  }
  const int f0 = blockIdx.y * fpg, fend = min(nfield, f0 + fpg);  // this CTA's fields
  // fill fields f, f + 1 (if any): column pair tp, rows tq + 64 k
  auto issue = [&](int f, int buf) {
    const int nh = f + 1 < fend ? 2 : 1;
    for (int h = 0; h < nh; ++h) {
      const float2* g = t1 + (size_t)(f + h) * Px * rowstride + (size_t)yy * nzp + z0 + 2 * tp + (size_t)tq * rowstride;
      float2* lb = x2i_block<P>(lines, buf, h, tp);
      for (int q = tq; q < Px; q += kRowStepX, g += (size_t)kRowStepX * rowstride)
        cp_async<16>(lb + 2 * P::addr(q), pval ? g : t1, pval);
    }
    cp_commit();
  };
  issue(f0, 0);
  for (int f = f0, it = 0; f < fend; f += 2, ++it) {
    const int buf = it & 1;
    const int nh = f + 1 < fend ? 2 : 1;
    if (f + 2 < fend) {
      issue(f + 2, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    if (wh < nh) {
      const int fh = f + wh, l = fh / fc, c = fh - l * fc;
      float2* blk = x2i_block<P>(lines, buf, wh, wp);
      sfft::inverse_il<P>(blk, twx, lane, nx);
      for (int t = lane; t < 2 * nx; t += 32) {
        const int xi = t >> 1, hc = t & 1;
        const int m = socc[xi * kTZ + 2 * wp + hc];
        if (m < 0) continue;
        const size_t r = fc * (size_t)m + c;
        float2 v = blk[2 * P::addr(xi) + hc];
        if (diag != nullptr) v = cadd(v, cmul(diag[r], x[(size_t)l * ldx + r]));
        if (jpre != nullptr) v = cmul(v, jpre[r]);
        y[(size_t)l * ldy + r] = v;
      }
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of fields f + 4, f + 5
  }
}

// Dynamic shared memory of a runtime-plan strided pass with nbuf tile buffers
// (nx > 0: the x passes' occupancy table of the tile).
template <typename T> int smem_tile(int lw, int nx, int nbuf = 2) {
  return nbuf * kTZ * lw * (int)sizeof(typename cplx<T>::type) + nx * kTZ * 4;
}
// Two tile buffers where they fit in a CTA's shared memory, else one.
template <typename T> int tile_buffers(int lw, int nx) { return smem_tile<T>(lw, nx, 2) <= kZSmemMax ? 2 : 1; }

}  // namespace tile
}  // namespace bdda
