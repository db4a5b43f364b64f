// Internal interfaces of the block-MVP kernels (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "common.cuh"

namespace bdda {

// Warps (one line each) per CTA in the contiguous-axis passes A and E.
constexpr int kLineWarps = 8;

// z-tile width of the strided passes: 8 x c64 = 64 B, 4 x c128 = 64 B rows.
template <typename T> struct TileCfg;
template <> struct TileCfg<float> { static constexpr int TZ = 8; };
template <> struct TileCfg<double> { static constexpr int TZ = 4; };

// Geometry shared by both precisions (device pointers).
struct MvpGeom {
  int nx, ny, nz;
  int Px, Py, Pz;
  AxisPlan px, py, pz;
  int nlines;                 // lattice lines (x, y) that hold >= 1 dipole
  const int* occ;             // [nx*ny*nz] dipole index or -1
  const int* lines;           // [nlines]  x*ny + y
  const unsigned char* lmask; // [nx*ny]
};

// Precision-specific tables (device pointers).
template <typename T> struct MvpPrec {
  using C = typename cplx<T>::type;
  const C* twx;
  const C* twy;
  const C* twz;
  const C* ghat;  // [Py][ceil(Pz/TZ)][6][Px][TZ], already divided by Px*Py*Pz
};

enum KernelId {
  kPassA = 0, kPassB, kPassC, kPassD, kPassE,
  kGram, kUpdate, kSmall, kOther,
  kNumKernelIds
};

// Optional per-kernel CUDA-event timing (accumulated when resolved).
struct KernelTimer {
  struct Pending { int id; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  double ms[kNumKernelIds] = {0};
  long long launches[kNumKernelIds] = {0};
  cudaEvent_t cur_a[kNumKernelIds] = {};
  bool enabled = false;

  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  }
  void begin(int id, cudaStream_t st) {
    launches[id]++;
    if (!enabled) return;
    cur_a[id] = get();
    cudaEventRecord(cur_a[id], st);
  }
  void end(int id, cudaStream_t st) {
    if (!enabled) return;
    cudaEvent_t b = get();
    cudaEventRecord(b, st);
    pending.push_back({id, cur_a[id], b});
  }
  // Call after the stream was synchronised.
  void resolve() {
    for (auto& p : pending) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ms[p.id] += t;
      pool.push_back(p.a); pool.push_back(p.b);
    }
    pending.clear();
  }
  void reset() {
    resolve();
    for (int i = 0; i < kNumKernelIds; ++i) { ms[i] = 0; launches[i] = 0; }
  }
  ~KernelTimer() {
    for (auto& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

template <typename T>
cudaError_t launch_block_mvp(const MvpGeom& g, const MvpPrec<T>& p, const typename cplx<T>::type* x, int ldx,
                             typename cplx<T>::type* y, int ldy, int L,
                             const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre,
                             typename cplx<T>::type* t1, typename cplx<T>::type* t2,
                             cudaStream_t st, KernelTimer* timer, const int* done = nullptr);

template <typename T> cudaError_t configure_mvp_kernels(int max_px);

// Green tensor: build Ghat (FP64 evaluation + FP64 3-D FFT) for both layouts.
// ghat_d: c128 tiles for TZ=TileCfg<double>::TZ; ghat_f: c64 tiles for
// TZ=TileCfg<float>::TZ (either may be null).  work: c128 [6*Px*Py*Pz].
cudaError_t build_green_hat(const MvpGeom& g, double lf, double k_re, double k_im,
                            const double2* twx, const double2* twy, const double2* twz,
                            double2* work, double2* ghat_d, float2* ghat_f, cudaStream_t st);

// Radix schedule + FP64 twiddles for a 5-smooth N <= kMaxLine.
bool make_axis_plan(int N, AxisPlan* p);
void make_twiddles(int N, std::vector<double2>* out);

}  // namespace bdda
