// Fused block-MVP passes: y = [diag o x +] A_off x  [o jpre], all RHS at once.
//
// Replaces the reference's per-RHS chain scatter -> BT_pad -> FFTW fwd ->
// Au_til product -> FFTW inv -> BT_reconstruct -> gather -> DIAG add -> jpre
// (mvp_fft/MBT_fft_mvp.cpp:19-32, bl_krylov_mvp_fft/bl_cocg_rq_jacobi_mvp_fft.cpp:43-60)
// by the mathematically identical 2x-padded 3-D FFT convolution with the
// 6-component symmetric Green tensor.  Fields are the 3*L (component, RHS)
// pairs; field f = 3*l + c.
//
// HBM layouts (element = complex T):
//   x, y   : column-major (rows 3*m + c, column l, leading dimension ld) --
//            the reference's Eigen layout of S / AS.
//   occ    : int32 [nx][ny][nz], dipole index of a lattice site or -1.
//   tiles  : int32 list of (y, z-tile) pairs (y*nzt + zt, 8-wide z tiles)
//            holding >= 1 dipole; tmask [ny][nzt] marks them.
//   T1     : [3L][Px][ny][nz]  after the x pass (only rows of listed tiles valid)
//   T2     : [3L][Px][Py][nz]  after the y pass; the z pass works in place
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
#include <algorithm>
#include <type_traits>

#include "fft_core.cuh"

#include "mvp.hpp"

namespace bdda {

namespace {

// ---- cp.async helpers (LDGSTS: global -> shared without registers) --------
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int sz = valid ? BYTES : 0;  // src-size 0: nothing read, destination zero-filled
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ bool skip(const int* done) { return done && *(volatile const int*)done; }

// ---------------------------------------------------------------- pass A
// One CTA per listed (y, z-tile): warp w owns z = z0 + w; loops over fields.
template <typename T>
__global__ void __launch_bounds__(kTileThreads)
k_pass_a(const typename cplx<T>::type* __restrict__ x, int ldx, int nfield, const int* __restrict__ occ,
         const int* __restrict__ tiles, int nx, int ny, int nz, int nzt, AxisPlan px,
         const typename cplx<T>::type* __restrict__ twx, typename cplx<T>::type* __restrict__ t1, const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Px = px.N;
  const int lw = plan_lw<C>(px), sh = plan_sk<C>(px);
  C* lines = reinterpret_cast<C*>(smem_raw);                       // [2][kTZ][lw]
  int* socc = reinterpret_cast<int*>(lines + 2 * kTZ * lw);        // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int y = tile / nzt, z0 = (tile - y * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + y) * nz + z] : -1;
  }
  __syncthreads();
  const size_t rowstride = (size_t)ny * nz;  // T1 stride between x rows
  int l = 0, c = 0;
  for (int f = 0; f < nfield; ++f) {
    C* line = lines + ((f & 1) * kTZ + warp) * lw;
    const C* xc = x + (size_t)l * ldx + c;
    for (int xi = lane; xi < nx; xi += 32) {
      const int m = socc[xi * kTZ + warp];
      line[skw(xi, sh)] = m >= 0 ? xc[3 * (size_t)m] : czero<C>();
    }
    __syncwarp();
    warp_fft<false>(line, twx, px, lane, 32, nx);
    __syncthreads();
    C* out = t1 + (size_t)f * Px * rowstride + (size_t)y * nz + z0;
    const C* lb = lines + (f & 1) * kTZ * lw;
    for (int idx = tid; idx < Px * kTZ; idx += kTileThreads) {
      const int w = idx & 7, q = idx >> 3;
      if (z0 + w < nz) out[(size_t)q * rowstride + w] = lb[w * lw + skw(q, sh)];
    }
    if (++c == 3) { c = 0; ++l; }
  }
}

// ---------------------------------------------------------------- pass B / D
// Persistent CTAs over tasks (field, x, z-tile); lines along y.
// B: T1[f][q][y<ny][z] -> T2[f][q][Py][z]   (rows of empty tiles zero-filled)
// D: T2[f][q][Py][z]   -> T1[f][q][y<ny][z] (rows of listed tiles only)
template <typename T, bool INV>
__global__ void __launch_bounds__(kTileThreads)
k_pass_y(const typename cplx<T>::type* __restrict__ src, typename cplx<T>::type* __restrict__ dst,
         const unsigned char* __restrict__ tmask, int ny, int nz, int nzt, int ntask, AxisPlan py,
         const typename cplx<T>::type* __restrict__ twy, const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Py = py.N;
  const int lw = plan_lw<C>(py), sh = plan_sk<C>(py);
  C* lines = reinterpret_cast<C*>(smem_raw);  // [2][kTZ][lw]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nin = INV ? Py : ny;    // rows read
  const int nout = INV ? ny : Py;   // rows written
  const size_t in_rows = (size_t)nin, out_rows = (size_t)nout;

  auto issue = [&](int task, int buf) {
    const int zt = task % nzt;
    const int r = task / nzt;  // f * Px + q
    const int z0 = zt * kTZ;
    const C* base = src + (size_t)r * in_rows * nz + z0;
    C* lb = lines + buf * kTZ * lw;
    for (int idx = tid; idx < nin * kTZ; idx += kTileThreads) {
      const int w = idx & 7, yy = idx >> 3;
      bool valid = z0 + w < nz;
      if (!INV) valid = valid && tmask[yy * nzt + zt];
      const C* g = valid ? base + (size_t)yy * nz + w : src;
      cp_async<sizeof(C)>(lb + w * lw + skw(yy, sh), g, valid);
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
    C* line = lines + (buf * kTZ + warp) * lw;
    warp_fft<INV>(line, twy, py, lane, 32, INV ? Py : ny);
    __syncthreads();
    const int zt = task % nzt;
    const int r = task / nzt;
    const int z0 = zt * kTZ;
    C* ob = dst + (size_t)r * out_rows * nz + z0;
    const C* lb = lines + buf * kTZ * lw;
    for (int idx = tid; idx < nout * kTZ; idx += kTileThreads) {
      const int w = idx & 7, yy = idx >> 3;
      if (z0 + w >= nz) continue;
      if (INV && !tmask[yy * nzt + zt]) continue;
      ob[(size_t)yy * nz + w] = lb[w * lw + skw(yy, sh)];
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of the next-but-one task
  }
}

// ---------------------------------------------------------------- pass C
// One warp per task (x = q, y = qy, rhs l): the three component lines along z.
template <typename T>
__global__ void __launch_bounds__(kZWarps * 32)
k_pass_c(typename cplx<T>::type* __restrict__ t2, int L, int Px, int Py, int nz, AxisPlan pz,
         const typename cplx<T>::type* __restrict__ twz, const typename cplx<T>::type* __restrict__ ghat,
         const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Pz = pz.N;
  const int lw = plan_lw<C>(pz), sh = plan_sk<C>(pz);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long task = (long long)blockIdx.x * kZWarps + warp;
  const long long ntask = (long long)Px * Py * L;
  if (task >= ntask) return;
  const int l = (int)(task % L);
  const long long line = task / L;  // q * Py + qy
  C* s0 = reinterpret_cast<C*>(smem_raw) + (size_t)warp * 3 * lw;
  C* s1 = s0 + lw;
  C* s2 = s1 + lw;
  const size_t fstride = (size_t)Px * Py * nz;  // between fields
  C* g0 = t2 + (size_t)(3 * l) * fstride + (size_t)line * nz;
  for (int z = lane; z < nz; z += 32) {
    s0[skw(z, sh)] = g0[z];
    s1[skw(z, sh)] = g0[fstride + z];
    s2[skw(z, sh)] = g0[2 * fstride + z];
  }
  __syncwarp();
  warp_fft_lines<false, 3>(s0, lw, twz, pz, lane, 32, nz);
  const C* gl = ghat + (size_t)line * 6 * Pz;
  for (int p = lane; p < Pz; p += 32) {
    const int sp = skw(p, sh);
    const C a0 = s0[sp], a1 = s1[sp], a2 = s2[sp];
    const C gxx = ldg_c(gl + p), gxy = ldg_c(gl + Pz + p), gxz = ldg_c(gl + 2 * Pz + p);
    const C gyy = ldg_c(gl + 3 * Pz + p), gyz = ldg_c(gl + 4 * Pz + p), gzz = ldg_c(gl + 5 * Pz + p);
    s0[sp] = cadd(cadd(cmul(gxx, a0), cmul(gxy, a1)), cmul(gxz, a2));
    s1[sp] = cadd(cadd(cmul(gxy, a0), cmul(gyy, a1)), cmul(gyz, a2));
    s2[sp] = cadd(cadd(cmul(gxz, a0), cmul(gyz, a1)), cmul(gzz, a2));
  }
  __syncwarp();
  warp_fft_lines<true, 3>(s0, lw, twz, pz, lane);
  for (int z = lane; z < nz; z += 32) {
    g0[z] = s0[skw(z, sh)];
    g0[fstride + z] = s1[skw(z, sh)];
    g0[2 * fstride + z] = s2[skw(z, sh)];
  }
}

// ---------------------------------------------------------------- pass E
// One CTA per listed (y, z-tile); loops over fields with the next field's
// tile prefetched by cp.async; scatters the occupied sites.
template <typename T>
__global__ void __launch_bounds__(kTileThreads)
k_pass_e(const typename cplx<T>::type* __restrict__ t1, int nfield, const int* __restrict__ occ,
         const int* __restrict__ tiles, int nx, int ny, int nz, int nzt, AxisPlan px,
         const typename cplx<T>::type* __restrict__ twx, const typename cplx<T>::type* __restrict__ x, int ldx,
         const typename cplx<T>::type* __restrict__ diag, const typename cplx<T>::type* __restrict__ jpre,
         typename cplx<T>::type* __restrict__ y, int ldy, const int* done) {
  using C = typename cplx<T>::type;
  if (skip(done)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Px = px.N;
  const int lw = plan_lw<C>(px), sh = plan_sk<C>(px);
  C* lines = reinterpret_cast<C*>(smem_raw);                       // [2][kTZ][lw]
  int* socc = reinterpret_cast<int*>(lines + 2 * kTZ * lw);        // [nx][kTZ]
  const int tile = tiles[blockIdx.x];
  const int yy = tile / nzt, z0 = (tile - yy * nzt) * kTZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t rowstride = (size_t)ny * nz;
  for (int idx = tid; idx < nx * kTZ; idx += kTileThreads) {
    const int xi = idx >> 3, w = idx & 7, z = z0 + w;
    socc[idx] = z < nz ? occ[((size_t)xi * ny + yy) * nz + z] : -1;
  }
  auto issue = [&](int f, int buf) {
    const C* base = t1 + (size_t)f * Px * rowstride + (size_t)yy * nz + z0;
    C* lb = lines + buf * kTZ * lw;
    for (int idx = tid; idx < Px * kTZ; idx += kTileThreads) {
      const int w = idx & 7, q = idx >> 3;
      const bool valid = z0 + w < nz;
      cp_async<sizeof(C)>(lb + w * lw + skw(q, sh), valid ? base + (size_t)q * rowstride + w : t1, valid);
    }
    cp_commit();
  };
  issue(0, 0);
  int l = 0, c = 0;
  for (int f = 0; f < nfield; ++f) {
    const int buf = f & 1;
    if (f + 1 < nfield) {
      issue(f + 1, buf ^ 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    C* line = lines + (buf * kTZ + warp) * lw;
    warp_fft<true>(line, twx, px, lane);
    for (int xi = lane; xi < nx; xi += 32) {
      const int m = socc[xi * kTZ + warp];
      if (m < 0) continue;
      const size_t r = 3 * (size_t)m + c;
      C v = line[skw(xi, sh)];
      if (diag != nullptr) v = cadd(v, cmul(diag[r], x[(size_t)l * ldx + r]));
      if (jpre != nullptr) v = cmul(v, jpre[r]);
      y[(size_t)l * ldy + r] = v;
    }
    __syncthreads();  // buffer 'buf' is the cp.async target of field f + 2
    if (++c == 3) { c = 0; ++l; }
  }
}

template <typename T> int smem_tile(int lw, int nx) {
  return 2 * kTZ * lw * (int)sizeof(typename cplx<T>::type) + nx * kTZ * 4;
}
template <typename T> int smem_z(int lw) { return kZWarps * 3 * lw * (int)sizeof(typename cplx<T>::type); }

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
  const int nfield = 3 * L;
  const int pbase = sizeof(T) == sizeof(double) ? (kPassA64 - kPassA) : 0;
  if (g.ntiles == 0) return cudaSuccess;  // no dipoles
  const int ntask_y = nfield * g.Px * g.nzt;
  const int grid_y = std::min(ntask_y, num_sms() * 8);
  // A
  if (timer) timer->begin(kPassA + pbase, st);
  k_pass_a<T><<<g.ntiles, kTileThreads, smem_tile<T>(plan_lw<C>(g.px), g.nx), st>>>(x, ldx, nfield, g.occ, g.tiles, g.nx, g.ny,
                                                                       g.nz, g.nzt, g.px, p.twx, t1, done);
  if (timer) timer->end(kPassA + pbase, st);
  // B
  if (timer) timer->begin(kPassB + pbase, st);
  k_pass_y<T, false><<<grid_y, kTileThreads, smem_tile<T>(plan_lw<C>(g.py), 0), st>>>(t1, t2, g.tmask, g.ny, g.nz, g.nzt,
                                                                         ntask_y, g.py, p.twy, done);
  if (timer) timer->end(kPassB + pbase, st);
  // C
  {
    const long long ntask = (long long)g.Px * g.Py * L;
    const unsigned grid = (unsigned)((ntask + kZWarps - 1) / kZWarps);
    if (timer) timer->begin(kPassC + pbase, st);
    bool launched = false;
    if constexpr (std::is_same<T, float>::value) {
      cudaError_t e = cudaSuccess;
      launched = launch_pass_c_static(g, t2, L, p.twz, p.ghat, st, done, &e);
      if (launched && e != cudaSuccess) return e;
    }
    if (!launched)
      k_pass_c<T><<<grid, kZWarps * 32, smem_z<T>(plan_lw<C>(g.pz)), st>>>(t2, L, g.Px, g.Py, g.nz, g.pz, p.twz, p.ghat,
                                                                          done);
    if (timer) timer->end(kPassC + pbase, st);
  }
  // D
  if (timer) timer->begin(kPassD + pbase, st);
  k_pass_y<T, true><<<grid_y, kTileThreads, smem_tile<T>(plan_lw<C>(g.py), 0), st>>>(t2, t1, g.tmask, g.ny, g.nz, g.nzt,
                                                                        ntask_y, g.py, p.twy, done);
  if (timer) timer->end(kPassD + pbase, st);
  // E
  if (timer) timer->begin(kPassE + pbase, st);
  k_pass_e<T><<<g.ntiles, kTileThreads, smem_tile<T>(plan_lw<C>(g.px), g.nx), st>>>(t1, nfield, g.occ, g.tiles, g.nx, g.ny, g.nz,
                                                                       g.nzt, g.px, p.twx, x, ldx, diag, jpre, y, ldy,
                                                                       done);
  if (timer) timer->end(kPassE + pbase, st);
  return cudaGetLastError();
}

template <typename T>
cudaError_t configure_mvp_kernels() {
  const int tile = smem_tile<T>(kMaxLineWords, kMaxLine / 2);
  const int zs = smem_z<T>(kMaxLineWords);
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_pass_a<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_pass_e<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_pass_y<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_pass_y<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile)) != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_pass_c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, zs);
}

template cudaError_t launch_block_mvp<float>(const MvpGeom&, const MvpPrec<float>&, const float2*, int, float2*, int, int,
                                             const float2*, const float2*, float2*, float2*, cudaStream_t, KernelTimer*,
                                             const int*);
template cudaError_t launch_block_mvp<double>(const MvpGeom&, const MvpPrec<double>&, const double2*, int, double2*, int,
                                              int, const double2*, const double2*, double2*, double2*, cudaStream_t,
                                              KernelTimer*, const int*);
template cudaError_t launch_block_mvp<dfl>(const MvpGeom&, const MvpPrec<dfl>&, const dfc*, int, dfc*, int, int,
                                           const dfc*, const dfc*, dfc*, dfc*, cudaStream_t, KernelTimer*, const int*);
template cudaError_t configure_mvp_kernels<float>();
template cudaError_t configure_mvp_kernels<double>();
template cudaError_t configure_mvp_kernels<dfl>();

}  // namespace bdda
