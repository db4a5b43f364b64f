// Shared device/host helpers for the block-DDA GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#if defined(__CUDACC__)
#define BDDA_HD __host__ __device__ __forceinline__
#else
#define BDDA_HD inline
#endif

namespace bdda {

// Complex value types: c64 = float2 (complex FP32), c128 = double2 (complex FP64).
template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };

BDDA_HD float2 cmake(float a, float b) { return make_float2(a, b); }
BDDA_HD double2 cmake(double a, double b) { return make_double2(a, b); }

template <typename C> BDDA_HD C cadd(C a, C b) { return cmake(a.x + b.x, a.y + b.y); }
template <typename C> BDDA_HD C csub(C a, C b) { return cmake(a.x - b.x, a.y - b.y); }
template <typename C> BDDA_HD C cmul(C a, C b) {
  return cmake(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> BDDA_HD C cmulc(C a, C b) {
  return cmake(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// conj(a) * b
template <typename C> BDDA_HD C cconjmul(C a, C b) {
  return cmake(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename C> BDDA_HD C czero() { return cmake(decltype(C::x)(0), decltype(C::x)(0)); }

// Transform length limits of the warp-per-line FFT.
constexpr int kMaxLine = 512;   // longest line one warp transforms
constexpr int kMaxStages = 16;

// Radix schedule of one axis: N = prod(radix[0..nst)), with the per-stage
// constants of the in-place DIF/DIT transform precomputed on the host:
// stage s works on blocks of Ls[s] = N / (radix[0] ... radix[s-1]) points,
// M[s] = Ls[s] / radix[s], twiddle stride N / Ls[s]; invM[s] = 1/M[s] lets a
// lane split its butterfly index t into (t / M, t % M) without an integer
// division (exact for t < 2^12).
struct AxisPlan {
  int N;
  int nst;
  int radix[kMaxStages];
  int M[kMaxStages];
  int tstride[kMaxStages];
  float invM[kMaxStages];
};

}  // namespace bdda
