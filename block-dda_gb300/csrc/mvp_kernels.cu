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
//   occ    : int32 [nx*ny*nz], dipole index of a lattice site or -1.
//   lines  : int32 list of (x*ny + y) lattice lines holding >= 1 dipole.
//   lmask  : uint8 [nx*ny], 1 for such lines.
//   T1     : [3L][nx*ny][Pz]   after the z pass (only lines in `lines` valid)
//   T2     : [3L][nx][Py][Pz]  after the y pass; the x pass works in place
//   Ghat   : [Py][ceil(Pz/TZ)][6][Px][TZ] -- Ghat/Ng, tile-contiguous for the
//            x pass, components (xx, xy, xz, yy, yz, zz).
//
// Pass order (forward z, y, x; inverse x, y, z), each a separate kernel:
//   A  z-forward, input pruned to occupied sites           x  -> T1
//   B  y-forward, input pruned to ny rows and to non-empty lines   T1 -> T2
//   C  x-forward, Ghat product, x-inverse, pruned to nx    T2 -> T2 (in place)
//   D  y-inverse, output pruned to ny rows of non-empty lines      T2 -> T1
//   E  z-inverse, gather at occupied sites, + diag o x, o jpre     T1 -> y
#include "fft_core.cuh"
#include "mvp.hpp"

namespace bdda {

namespace {

__host__ __device__ __forceinline__ int odd_stride(int n) { return n | 1; }

// ---------------------------------------------------------------- pass A
template <typename T>
__global__ void __launch_bounds__(kLineWarps * 32)
k_pass_a(const typename cplx<T>::type* __restrict__ x, int ldx, int nfield,
         const int* __restrict__ occ, const int* __restrict__ lines, int nz, int nxy,
         AxisPlan pz, const typename cplx<T>::type* __restrict__ twz,
         typename cplx<T>::type* __restrict__ t1, const int* done) {
  using C = typename cplx<T>::type;
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* smem = reinterpret_cast<C*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int field = blockIdx.y * kLineWarps + warp;
  if (field >= nfield) return;
  const int line = lines[blockIdx.x];
  const int l = field / 3, c = field - 3 * (field / 3);
  C* s = smem + warp * pz.N;
  const C* xc = x + (size_t)l * ldx + c;
  for (int z = lane; z < pz.N; z += 32) {
    C v = czero<C>();
    if (z < nz) {
      const int m = occ[(size_t)line * nz + z];
      if (m >= 0) v = xc[3 * (size_t)m];
    }
    s[z] = v;
  }
  __syncwarp();
  warp_fft<false>(s, twz, pz, lane);
  C* out = t1 + ((size_t)field * nxy + line) * pz.N;
  for (int z = lane; z < pz.N; z += 32) out[z] = s[z];
}

// ---------------------------------------------------------------- pass B / D
// B: T1 -> T2 forward along y.  D: T2 -> T1 inverse along y.
template <typename T, bool INV>
__global__ void __launch_bounds__(TileCfg<T>::TZ * 32)
k_pass_y(const typename cplx<T>::type* __restrict__ src, typename cplx<T>::type* __restrict__ dst,
         const unsigned char* __restrict__ lmask, int nx, int ny, int Pz,
         AxisPlan py, const typename cplx<T>::type* __restrict__ twy, const int* done) {
  using C = typename cplx<T>::type;
  if (done && *(volatile const int*)done) return;
  constexpr int TZ = TileCfg<T>::TZ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* smem = reinterpret_cast<C*>(smem_raw);
  const int Py = py.N;
  const int lds = odd_stride(Py);
  const int z0 = blockIdx.x * TZ;
  const int xi = blockIdx.y;
  const size_t field = blockIdx.z;
  const int tid = threadIdx.x;
  const unsigned char* lm = lmask + (size_t)xi * ny;
  if (!INV) {
    // rows y < ny from T1[field][xi*ny + y][z], zero elsewhere
    const C* base = src + ((size_t)field * nx * ny + (size_t)xi * ny) * Pz;
    for (int idx = tid; idx < Py * TZ; idx += TZ * 32) {
      const int w = idx % TZ, y = idx / TZ, z = z0 + w;
      C v = czero<C>();
      if (y < ny && z < Pz && lm[y]) v = base[(size_t)y * Pz + z];
      smem[w * lds + y] = v;
    }
  } else {
    const C* base = src + ((size_t)field * nx + xi) * (size_t)Py * Pz;
    for (int idx = tid; idx < Py * TZ; idx += TZ * 32) {
      const int w = idx % TZ, y = idx / TZ, z = z0 + w;
      C v = czero<C>();
      if (z < Pz) v = base[(size_t)y * Pz + z];
      smem[w * lds + y] = v;
    }
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  warp_fft<INV>(smem + warp * lds, twy, py, lane);
  __syncthreads();
  if (!INV) {
    C* base = dst + ((size_t)field * nx + xi) * (size_t)Py * Pz;
    for (int idx = tid; idx < Py * TZ; idx += TZ * 32) {
      const int w = idx % TZ, y = idx / TZ, z = z0 + w;
      if (z < Pz) base[(size_t)y * Pz + z] = smem[w * lds + y];
    }
  } else {
    C* base = dst + ((size_t)field * nx * ny + (size_t)xi * ny) * Pz;
    for (int idx = tid; idx < ny * TZ; idx += TZ * 32) {
      const int w = idx % TZ, y = idx / TZ, z = z0 + w;
      if (z < Pz && lm[y]) base[(size_t)y * Pz + z] = smem[w * lds + y];
    }
  }
}

// ---------------------------------------------------------------- pass C
template <typename T>
__global__ void __launch_bounds__(3 * TileCfg<T>::TZ * 32)
k_pass_c(typename cplx<T>::type* __restrict__ t2, int L, int nx, int Py, int Pz,
         AxisPlan px, const typename cplx<T>::type* __restrict__ twx,
         const typename cplx<T>::type* __restrict__ ghat, const int* done) {
  using C = typename cplx<T>::type;
  if (done && *(volatile const int*)done) return;
  constexpr int TZ = TileCfg<T>::TZ;
  constexpr int NT = 3 * TZ * 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* smem = reinterpret_cast<C*>(smem_raw);
  const int Px = px.N;
  const int lds = odd_stride(Px);
  const int zt = blockIdx.x, z0 = zt * TZ;
  const int y = blockIdx.y;
  const int nzt = gridDim.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t pstride = (size_t)Py * Pz;  // x stride in T2
  const C* gb = ghat + ((size_t)y * nzt + zt) * 6 * (size_t)Px * TZ;
  for (int l = 0; l < L; ++l) {
    // load 3 components x TZ columns, rows x < nx; zero-fill to Px
    for (int idx = tid; idx < 3 * Px * TZ; idx += NT) {
      const int w = idx % TZ, t = idx / TZ;
      const int xi = t % Px, c = t / Px, z = z0 + w;
      C v = czero<C>();
      if (xi < nx && z < Pz) v = t2[((size_t)(3 * l + c) * nx + xi) * pstride + (size_t)y * Pz + z];
      smem[(c * TZ + w) * lds + xi] = v;
    }
    __syncthreads();
    warp_fft<false>(smem + warp * lds, twx, px, lane);
    __syncthreads();
    for (int p = tid; p < Px * TZ; p += NT) {
      const int w = p % TZ, q = p / TZ;
      C a0 = smem[(0 * TZ + w) * lds + q];
      C a1 = smem[(1 * TZ + w) * lds + q];
      C a2 = smem[(2 * TZ + w) * lds + q];
      const size_t PT = (size_t)Px * TZ;
      C gxx = gb[0 * PT + p], gxy = gb[1 * PT + p], gxz = gb[2 * PT + p];
      C gyy = gb[3 * PT + p], gyz = gb[4 * PT + p], gzz = gb[5 * PT + p];
      C b0 = cadd(cadd(cmul(gxx, a0), cmul(gxy, a1)), cmul(gxz, a2));
      C b1 = cadd(cadd(cmul(gxy, a0), cmul(gyy, a1)), cmul(gyz, a2));
      C b2 = cadd(cadd(cmul(gxz, a0), cmul(gyz, a1)), cmul(gzz, a2));
      smem[(0 * TZ + w) * lds + q] = b0;
      smem[(1 * TZ + w) * lds + q] = b1;
      smem[(2 * TZ + w) * lds + q] = b2;
    }
    __syncthreads();
    warp_fft<true>(smem + warp * lds, twx, px, lane);
    __syncthreads();
    for (int idx = tid; idx < 3 * nx * TZ; idx += NT) {
      const int w = idx % TZ, t = idx / TZ;
      const int xi = t % nx, c = t / nx, z = z0 + w;
      if (z < Pz) t2[((size_t)(3 * l + c) * nx + xi) * pstride + (size_t)y * Pz + z] = smem[(c * TZ + w) * lds + xi];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- pass E
template <typename T>
__global__ void __launch_bounds__(kLineWarps * 32)
k_pass_e(const typename cplx<T>::type* __restrict__ t1, int nfield, int nz, int nxy,
         const int* __restrict__ occ, const int* __restrict__ lines,
         AxisPlan pz, const typename cplx<T>::type* __restrict__ twz,
         const typename cplx<T>::type* __restrict__ x, int ldx,
         const typename cplx<T>::type* __restrict__ diag,
         const typename cplx<T>::type* __restrict__ jpre,
         typename cplx<T>::type* __restrict__ y, int ldy, const int* done) {
  using C = typename cplx<T>::type;
  if (done && *(volatile const int*)done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* smem = reinterpret_cast<C*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int field = blockIdx.y * kLineWarps + warp;
  if (field >= nfield) return;
  const int line = lines[blockIdx.x];
  const int l = field / 3, c = field - 3 * (field / 3);
  C* s = smem + warp * pz.N;
  const C* in = t1 + ((size_t)field * nxy + line) * pz.N;
  for (int z = lane; z < pz.N; z += 32) s[z] = in[z];
  __syncwarp();
  warp_fft<true>(s, twz, pz, lane);
  for (int z = lane; z < nz; z += 32) {
    const int m = occ[(size_t)line * nz + z];
    if (m < 0) continue;
    const size_t r = 3 * (size_t)m + c;
    C v = s[z];
    if (diag != nullptr) v = cadd(v, cmul(diag[r], x[(size_t)l * ldx + r]));
    if (jpre != nullptr) v = cmul(v, jpre[r]);
    y[(size_t)l * ldy + r] = v;
  }
}

template <typename T>
int smem_line_pass(int Pz) { return kLineWarps * Pz * (int)sizeof(typename cplx<T>::type); }

}  // namespace

// ---------------------------------------------------------------- launcher
template <typename T>
cudaError_t launch_block_mvp(const MvpGeom& g, const MvpPrec<T>& p, const typename cplx<T>::type* x, int ldx,
                             typename cplx<T>::type* y, int ldy, int L,
                             const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre,
                             typename cplx<T>::type* t1, typename cplx<T>::type* t2,
                             cudaStream_t st, KernelTimer* timer, const int* done) {
  using C = typename cplx<T>::type;
  constexpr int TZ = TileCfg<T>::TZ;
  const int nfield = 3 * L;
  const int nxy = g.nx * g.ny;
  const int nzt = (g.Pz + TZ - 1) / TZ;
  if (g.nlines == 0) {
    // no dipoles at all: y = diag o x (o jpre) is empty as well
    return cudaSuccess;
  }
  // A
  {
    dim3 grid(g.nlines, (nfield + kLineWarps - 1) / kLineWarps);
    int sm = smem_line_pass<T>(g.Pz);
    if (timer) timer->begin(kPassA, st);
    k_pass_a<T><<<grid, kLineWarps * 32, sm, st>>>(x, ldx, nfield, g.occ, g.lines, g.nz, nxy, g.pz, p.twz, t1, done);
    if (timer) timer->end(kPassA, st);
  }
  // B
  {
    dim3 grid(nzt, g.nx, nfield);
    int sm = TZ * (g.Py | 1) * (int)sizeof(C);
    if (timer) timer->begin(kPassB, st);
    k_pass_y<T, false><<<grid, TZ * 32, sm, st>>>(t1, t2, g.lmask, g.nx, g.ny, g.Pz, g.py, p.twy, done);
    if (timer) timer->end(kPassB, st);
  }
  // C
  {
    dim3 grid(nzt, g.Py);
    int sm = 3 * TZ * (g.Px | 1) * (int)sizeof(C);
    if (timer) timer->begin(kPassC, st);
    k_pass_c<T><<<grid, 3 * TZ * 32, sm, st>>>(t2, L, g.nx, g.Py, g.Pz, g.px, p.twx, p.ghat, done);
    if (timer) timer->end(kPassC, st);
  }
  // D
  {
    dim3 grid(nzt, g.nx, nfield);
    int sm = TZ * (g.Py | 1) * (int)sizeof(C);
    if (timer) timer->begin(kPassD, st);
    k_pass_y<T, true><<<grid, TZ * 32, sm, st>>>(t2, t1, g.lmask, g.nx, g.ny, g.Pz, g.py, p.twy, done);
    if (timer) timer->end(kPassD, st);
  }
  // E
  {
    dim3 grid(g.nlines, (nfield + kLineWarps - 1) / kLineWarps);
    int sm = smem_line_pass<T>(g.Pz);
    if (timer) timer->begin(kPassE, st);
    k_pass_e<T><<<grid, kLineWarps * 32, sm, st>>>(t1, nfield, g.nz, nxy, g.occ, g.lines, g.pz, p.twz, x, ldx,
                                                   diag, jpre, y, ldy, done);
    if (timer) timer->end(kPassE, st);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t configure_mvp_kernels(int max_px) {
  using C = typename cplx<T>::type;
  constexpr int TZ = TileCfg<T>::TZ;
  cudaError_t e;
  int sm_c = 3 * TZ * (max_px | 1) * (int)sizeof(C);
  e = cudaFuncSetAttribute(k_pass_c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_c > 48 * 1024 ? sm_c : 48 * 1024);
  if (e != cudaSuccess) return e;
  int sm_y = TZ * (kMaxLine | 1) * (int)sizeof(C);
  e = cudaFuncSetAttribute(k_pass_y<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_y > 48 * 1024 ? sm_y : 48 * 1024);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_pass_y<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_y > 48 * 1024 ? sm_y : 48 * 1024);
  if (e != cudaSuccess) return e;
  int sm_l = kLineWarps * kMaxLine * (int)sizeof(C);
  e = cudaFuncSetAttribute(k_pass_a<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_l > 48 * 1024 ? sm_l : 48 * 1024);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_pass_e<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_l > 48 * 1024 ? sm_l : 48 * 1024);
  return e;
}

template cudaError_t launch_block_mvp<float>(const MvpGeom&, const MvpPrec<float>&, const float2*, int, float2*, int, int,
                                             const float2*, const float2*, float2*, float2*, cudaStream_t, KernelTimer*,
                                             const int*);
template cudaError_t launch_block_mvp<double>(const MvpGeom&, const MvpPrec<double>&, const double2*, int, double2*, int,
                                              int, const double2*, const double2*, double2*, double2*, cudaStream_t,
                                              KernelTimer*, const int*);
template cudaError_t configure_mvp_kernels<float>(int);
template cudaError_t configure_mvp_kernels<double>(int);

}  // namespace bdda
