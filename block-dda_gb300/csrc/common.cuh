// Shared device/host helpers for the block-DDA GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define BDDA_HD __host__ __device__ __forceinline__
#else
#define BDDA_HD inline
#endif

namespace bdda {

// ---------------------------------------------------------------------------
// Double-float scalar: value = hi + lo with |lo| <= ulp(hi)/2 (about 48
// significant bits), computed with FP32 instructions only.  GB300's FP32 pipes
// run ~64x the FP64 rate, so an FFT in double-float arithmetic is several
// times faster than in FP64 while keeping the refinement residual accurate to
// ~1e-14.  Sums use the two-sum of Knuth, products the FMA-based two-product;
// the addition is the short ("sloppy") variant whose error is bounded
// relative to |a| + |b|, which is what FFT error analysis needs.
// ---------------------------------------------------------------------------
struct __align__(8) dfl {
  float hi, lo;
  dfl() = default;
  BDDA_HD constexpr dfl(float h, float l) : hi(h), lo(l) {}
  BDDA_HD constexpr dfl(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  BDDA_HD constexpr dfl(int v) : hi((float)v), lo(0.0f) {}
};
BDDA_HD dfl df_quick_two_sum(float a, float b) {
  const float s = a + b;
  return dfl(s, b - (s - a));
}
BDDA_HD dfl operator+(dfl a, dfl b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return df_quick_two_sum(s, e);
}
BDDA_HD dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
BDDA_HD dfl operator-(dfl a, dfl b) { return a + (-b); }
BDDA_HD dfl operator*(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);  // exact low part of a.hi * b.hi
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_quick_two_sum(p, e);
}
BDDA_HD double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// Complex double-float (16 bytes, the size of a complex FP64 value).
struct __align__(16) dfc {
  dfl x, y;
};

// Double-float without renormalisation, the arithmetic of the double-float
// block MVP.  The leading parts are summed with the exact two-sum and the
// products formed with the FMA two-product, as in dfl, but the result keeps
// the error term as the trailing part (|lo| may exceed ulp(hi) / 2 by the few
// rounding errors of a butterfly chain) instead of being renormalised by a
// quick-two-sum: 8 instead of 11 FP32 instructions per addition, 4 instead of
// 7 per product.  Every result still equals hi + lo to ~2^-44 of the operands'
// magnitude, which bounds the FFT's error in norm as the normalised form
// does; values are read out as hi + lo in FP64.  Layout identical to dfl.
struct __align__(8) dfz {
  float hi, lo;
  dfz() = default;
  BDDA_HD constexpr dfz(float h, float l) : hi(h), lo(l) {}
  BDDA_HD constexpr dfz(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  BDDA_HD constexpr dfz(int v) : hi((float)v), lo(0.0f) {}
};
BDDA_HD dfz operator+(dfz a, dfz b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  return dfz(s, ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo));
}
BDDA_HD dfz operator-(dfz a) { return dfz(-a.hi, -a.lo); }
BDDA_HD dfz operator-(dfz a, dfz b) { return a + (-b); }
BDDA_HD dfz operator*(dfz a, dfz b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dfz(p, e);
}
struct __align__(16) dfzc {
  dfz x, y;
};

// Complex value types: c64 = float2 (complex FP32), c128 = double2 (complex
// FP64), dfc (complex double-float).
template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<dfl> { using type = dfc; };
template <> struct cplx<dfz> { using type = dfzc; };

BDDA_HD float2 cmake(float a, float b) { return make_float2(a, b); }
BDDA_HD double2 cmake(double a, double b) { return make_double2(a, b); }
BDDA_HD dfc cmake(dfl a, dfl b) { dfc c; c.x = a; c.y = b; return c; }
BDDA_HD dfzc cmake(dfz a, dfz b) { dfzc c; c.x = a; c.y = b; return c; }

template <typename C> BDDA_HD C cadd(C a, C b) { return cmake(a.x + b.x, a.y + b.y); }
template <typename C> BDDA_HD C csub(C a, C b) { return cmake(a.x - b.x, a.y - b.y); }

#if defined(__CUDA_ARCH__)
// Complex FP32 values as one two-lane f32x2 operand (sm_100-family
// add/sub/mul/fma.rn.f32x2: both parts in one issue slot, each part rounded as
// the scalar instruction rounds it).  Device code only; the host build and the
// other element types keep the scalar templates above.
namespace f2 {
__device__ __forceinline__ unsigned long long pk(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 up(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ unsigned long long dup(float c) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(c));
  return r;
}
__device__ __forceinline__ float2 add(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
  return up(d);
}
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
  return up(d);
}
// c a (real c)
__device__ __forceinline__ float2 scale(float c, float2 a) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(dup(c)), "l"(pk(a)));
  return up(d);
}
// c a + b (real c), one rounding per part
__device__ __forceinline__ float2 scale_add(float c, float2 a, float2 b) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(dup(c)), "l"(pk(a)), "l"(pk(b)));
  return up(d);
}
}  // namespace f2
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return f2::add(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return f2::sub(a, b); }
#endif

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

// Read-only load of a complex value through the non-coherent cache.
#if defined(__CUDACC__)
__device__ __forceinline__ float2 ldg_c(const float2* p) { return __ldg(p); }
__device__ __forceinline__ double2 ldg_c(const double2* p) { return __ldg(p); }
__device__ __forceinline__ dfc ldg_c(const dfc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  dfc c;
  c.x = dfl(v.x, v.y);
  c.y = dfl(v.z, v.w);
  return c;
}
__device__ __forceinline__ dfzc ldg_c(const dfzc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  dfzc c;
  c.x = dfz(v.x, v.y);
  c.y = dfz(v.z, v.w);
  return c;
}
#else
template <typename C> inline C ldg_c(const C* p) { return *p; }
#endif

// Transform length limits of the warp-per-line FFT.
// Longest line one warp transforms (box sides up to kMaxLine / 2 = 600).  The
// compile-time plan tables cover lengths up to kMaxStaticLine; longer lines
// run the runtime-plan kernels (strided passes single-buffered where two tile
// buffers of 16-byte elements would exceed the shared memory of a CTA).
constexpr int kMaxLine = 1200;
constexpr int kMaxStaticLine = 512;
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
  int sk[2];  // shared-memory skew shift for 8-byte / 16-byte elements (31: no skew)
  int lw[2];  // shared-memory line pitch (elements) for 8-byte / 16-byte elements
};
// Upper bound of AxisPlan::lw (skew shift >= 3, pitch padding < 16).
constexpr int kMaxLineWords = kMaxLine + kMaxLine / 8 + 16;

}  // namespace bdda
