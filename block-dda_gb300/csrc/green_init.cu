// Green-tensor spectrum Ghat on the padded grid, built on the device in FP64.
//
// Replaces application_function + BT_fft + MBT_fft_init
// (mvp_fft/application_function.cpp:21-40, mvp_fft/BT_fft.cpp:8-53,
// mvp_fft/MBT_fft_init.cpp:22-35): instead of the length f^2 prod(2n_i-1) 1-D
// MBT projection, the 3x3 block A(d) = -G(d lf) is evaluated on the 2x-padded
// circulant grid (index j -> offset j for j < n, j - P for j > P - n, zero in
// the gap and at d = 0), its 6 distinct components (9 with the magnetic
// coupling of f = 6) are transformed with a full 3-D FFT in FP64, divided by
// Px*Py*Pz and re-tiled for the fused z pass.
#include <mutex>
#include <vector>

#include "fft_core.cuh"
#include "mvp.hpp"

namespace bdda {

namespace {

__device__ __forceinline__ bool circ_offset(int j, int n, int P, int* d) {
  if (j < n) { *d = j; return true; }
  if (j > P - n) { *d = j - P; return true; }
  return false;
}

// g[comp][jx][jy][jz], comp = xx, xy, xz, yy, yz, zz of A = -G; with nc = 9
// (f = 6) also comp 6..8 = xy, xz, yz of B = -F, F = -k^2 e^{ikr}/r
// (1 - 1/(ikr)) [r^ x] (mvp_fft/application_function.cpp:52-64).
__global__ void k_green_eval(double2* __restrict__ g, int nc, int nx, int ny, int nz, int Px, int Py, int Pz,
                             double lf, double kr, double ki) {
  const size_t ng = (size_t)Px * Py * Pz;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < ng; idx += (size_t)gridDim.x * blockDim.x) {
    const int jz = (int)(idx % Pz);
    const int jy = (int)((idx / Pz) % Py);
    const int jx = (int)(idx / ((size_t)Pz * Py));
    int dx, dy, dz;
    double2 out[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) out[c] = make_double2(0.0, 0.0);
    if (circ_offset(jx, nx, Px, &dx) && circ_offset(jy, ny, Py, &dy) && circ_offset(jz, nz, Pz, &dz) &&
        (dx | dy | dz) != 0) {
      const double rx = dx * lf, ry = dy * lf, rz = dz * lf;
      const double r2 = rx * rx + ry * ry + rz * rz;
      const double r = sqrt(r2);
      // e = exp(i k r) / r with complex k = kr + i ki
      double sn, cs;
      sincos(kr * r, &sn, &cs);
      const double damp = exp(-ki * r) / r;
      const double2 e = make_double2(damp * cs, damp * sn);
      // c1 = k^2 ; c2 = (1 - i k r) / r^2
      const double2 c1 = make_double2(kr * kr - ki * ki, 2.0 * kr * ki);
      const double2 c2 = make_double2((1.0 + ki * r) / r2, (-kr * r) / r2);
      const double u[3] = {rx, ry, rz};
      int c = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int b = a; b < 3; ++b) {
          const double rr = u[a] * u[b] / r2;
          const double dl = (a == b) ? 1.0 : 0.0;
          // G_ab = (c1 (d - rr) - c2 (d - 3 rr)) e ; A = -G
          const double p = dl - rr, q = dl - 3.0 * rr;
          const double2 t = make_double2(c1.x * p - c2.x * q, c1.y * p - c2.y * q);
          const double2 gab = cmul(t, e);
          out[c++] = make_double2(-gab.x, -gab.y);
        }
      }
      if (nc == 9) {
        // fac = -k^2 e (1 - 1/w), w = i k r; B = -F: B_xy = fac u_z, B_xz = -fac u_y, B_yz = fac u_x
        const double2 w = make_double2(-ki * r, kr * r);
        const double w2 = w.x * w.x + w.y * w.y;
        const double2 one_m = make_double2(1.0 - w.x / w2, w.y / w2);  // 1 - conj(w) / |w|^2
        const double2 ce = cmul(c1, e);
        const double2 fac = cmul(make_double2(-ce.x, -ce.y), one_m);
        const double ux = rx / r, uy = ry / r, uz = rz / r;
        out[6] = make_double2(fac.x * uz, fac.y * uz);
        out[7] = make_double2(-fac.x * uy, -fac.y * uy);
        out[8] = make_double2(fac.x * ux, fac.y * ux);
      }
    }
    for (int c = 0; c < nc; ++c) g[(size_t)c * ng + idx] = out[c];
  }
}

// In-place FFT of contiguous lines (length p.N), one warp per line.
constexpr int kInitWarps = 8;
__global__ void __launch_bounds__(kInitWarps * 32)
k_fft_contig(double2* __restrict__ data, size_t nlines, AxisPlan p, const double2* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lw = plan_lw<double2>(p), sh = plan_sk<double2>(p);
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t line = (size_t)blockIdx.x * kInitWarps + warp;
  if (line >= nlines) return;
  double2* s = smem + warp * lw;
  double2* d = data + line * p.N;
  for (int i = lane; i < p.N; i += 32) s[skw(i, sh)] = d[i];
  __syncwarp();
  warp_fft_lines<false, 1, double2, true>(s, 0, tw, p, lane);  // any schedule (z: composite and first-stage radices)
  for (int i = lane; i < p.N; i += 32) d[i] = s[skw(i, sh)];
}

// In-place forward FFT along the middle index of data[A][N][Cc], 8 columns per CTA.
__global__ void __launch_bounds__(kInitWarps * 32)
k_fft_strided(double2* __restrict__ data, size_t Cc, AxisPlan p, const double2* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = p.N;
  const int lw = plan_lw<double2>(p), sh = plan_sk<double2>(p);
  double2* smem = reinterpret_cast<double2*>(smem_raw);
  const size_t c0 = (size_t)blockIdx.x * kInitWarps;
  double2* base = data + (size_t)blockIdx.y * N * Cc;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < N * kInitWarps; idx += kInitWarps * 32) {
    const int w = idx % kInitWarps, i = idx / kInitWarps;
    const size_t c = c0 + w;
    smem[w * lw + skw(i, sh)] = (c < Cc) ? base[(size_t)i * Cc + c] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  warp_fft_lines<false, 1, double2, true>(smem + (tid >> 5) * lw, 0, tw, p, tid & 31);
  __syncthreads();
  for (int idx = tid; idx < N * kInitWarps; idx += kInitWarps * 32) {
    const int w = idx % kInitWarps, i = idx / kInitWarps;
    const size_t c = c0 + w;
    if (c < Cc) base[(size_t)i * Cc + c] = smem[w * lw + skw(i, sh)];
  }
}

// g[comp][qx][qy][qz] / Ng  ->  ghat[qx][qy][comp][green_pos(qz)], nc components
// (rl = 0: natural order along z; else last-radix-major, see green_perm_radix)
template <typename C>
__global__ void k_green_pack(const double2* __restrict__ g, C* __restrict__ out, int nc, int Px, int Py, int Pz,
                             double scale, int rl) {
  const size_t ng = (size_t)Px * Py * Pz;
  const size_t total = (size_t)nc * ng;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int qz = (int)(idx % Pz);
    const size_t t = idx / Pz;
    const int comp = (int)(t % nc);
    const size_t line = t / nc;  // qx * Py + qy
    double2 v = g[(size_t)comp * ng + line * Pz + qz];
    out[idx - qz + green_pos(qz, Pz, rl)] = cmake((decltype(C::x))(v.x * scale), (decltype(C::x))(v.y * scale));
  }
}

}  // namespace

cudaError_t build_green_hat(const MvpGeom& g, double lf, double k_re, double k_im,
                            const double2* twx, const double2* twy, const double2* twz,
                            double2* work, double2* ghat_d, float2* ghat_f, dfc* ghat_df, int gperm, cudaStream_t st) {
  const int Px = g.Px, Py = g.Py, Pz = g.Pz;
  const size_t ng = (size_t)Px * Py * Pz;
  cudaError_t e;
  static std::once_flag once;
  static cudaError_t cfg = cudaSuccess;
  std::call_once(once, [] {
    const int maxsm = kInitWarps * kMaxLineWords * (int)sizeof(double2);
    cfg = cudaFuncSetAttribute(k_fft_contig, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
    if (cfg == cudaSuccess) cfg = cudaFuncSetAttribute(k_fft_strided, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
  });
  if ((e = cfg) != cudaSuccess) return e;
  const int nc = g.f == 6 ? 9 : 6;
  k_green_eval<<<1216, 256, 0, st>>>(work, nc, g.nx, g.ny, g.nz, Px, Py, Pz, lf, k_re, k_im);
  // z lines (contiguous)
  {
    const size_t nlines = (size_t)nc * Px * Py;
    const int sm = kInitWarps * plan_lw<double2>(g.pz) * (int)sizeof(double2);
    k_fft_contig<<<(unsigned)((nlines + kInitWarps - 1) / kInitWarps), kInitWarps * 32, sm, st>>>(work, nlines, g.pz, twz);
  }
  // y lines: data[6*Px][Py][Pz]
  {
    dim3 grid((unsigned)((Pz + kInitWarps - 1) / kInitWarps), nc * Px);
    const int sm = kInitWarps * plan_lw<double2>(g.py) * (int)sizeof(double2);
    k_fft_strided<<<grid, kInitWarps * 32, sm, st>>>(work, (size_t)Pz, g.py, twy);
  }
  // x lines: data[6][Px][Py*Pz]
  {
    const size_t cc = (size_t)Py * Pz;
    dim3 grid((unsigned)((cc + kInitWarps - 1) / kInitWarps), nc);
    const int sm = kInitWarps * plan_lw<double2>(g.px) * (int)sizeof(double2);
    k_fft_strided<<<grid, kInitWarps * 32, sm, st>>>(work, cc, g.px, twx);
  }
  const double scale = 1.0 / (double)ng;
  if (ghat_d) k_green_pack<double2><<<2432, 256, 0, st>>>(work, ghat_d, nc, Px, Py, Pz, scale, 0);
  if (ghat_f) k_green_pack<float2><<<2432, 256, 0, st>>>(work, ghat_f, nc, Px, Py, Pz, scale, gperm);
  if (ghat_df) k_green_pack<dfc><<<2432, 256, 0, st>>>(work, ghat_df, nc, Px, Py, Pz, scale, 0);
  return cudaGetLastError();
}

}  // namespace bdda
