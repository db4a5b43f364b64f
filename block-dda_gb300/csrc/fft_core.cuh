// Warp-per-line in-place mixed-radix FFT in shared memory: register radices
// 2, 3, 4, 5, 8 and the composite 6, 9, 10, 12, 15, 16.
//
// One warp owns one (or NL) line(s) of length N <= kMaxLine held in shared memory.
//
// Forward = decimation in frequency (Gentleman-Sande), natural-order input,
// digit-reversed output.  With N = R_1 R_2 ... R_m, stage s works on blocks
// of length Ls = N / (R_1 ... R_{s-1}), Ms = Ls / R_s; butterfly (b, n1),
// n1 < Ms, reads x[b Ls + n1 + Ms n2] (n2 < R_s), applies the R_s-point DFT
// and the twiddle w_Ls^{n1 k2} and writes back to the same positions
// b Ls + n1 + Ms k2.  Inverse = the adjoint stages in reverse order
// (conjugate twiddle, inverse DFT): digit-reversed input, natural output,
// unnormalised (a round trip scales by N).
//
// A convolution never needs the natural-order spectrum: the Green spectrum is
// produced by the same forward transform, so the pointwise product pairs
// matching (permuted) frequencies and the inverse restores natural order.
// Each butterfly reads and writes the same positions, so a stage needs no
// register staging and only one buffer; lanes take consecutive n1.  Lines
// are stored skewed (skw) with a per-plan shift and pitch, so that the strided
// accesses of the last stages do not collide in shared-memory banks.
//
// Twiddle table (per axis, global memory, read through L1):
//   tw[t] = exp(-2 pi i t / N), t in [0, N), computed in FP64 on the host.
#pragma once

#include "common.cuh"

// The core also compiles as plain C++ (host unit tests run one "lane" that
// walks every butterfly; butterflies of a stage are independent).
#if defined(__CUDACC__)
#define BDDA_FFT_FN __device__ __forceinline__
#define BDDA_LDG(p) ldg_c(p)
#define BDDA_SYNCWARP() __syncwarp()
#else
#define BDDA_FFT_FN inline
#define BDDA_LDG(p) (*(p))
#define BDDA_SYNCWARP() ((void)0)
#endif

namespace bdda {

// ---- radix kernels -------------------------------------------------------
// Forward uses exp(-2 pi i / R); INV uses exp(+2 pi i / R).

template <typename C> BDDA_FFT_FN C mul_i(C a) { return cmake(-a.y, a.x); }     // i a
template <typename C> BDDA_FFT_FN C mul_mi(C a) { return cmake(a.y, -a.x); }    // -i a

template <bool INV, typename C> BDDA_FFT_FN void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <bool INV, typename C> BDDA_FFT_FN void dft3(C* v) {
  using T = decltype(C::x);
  const T s = T(0.86602540378443864676);  // sin(2 pi / 3)
  C t1 = cadd(v[1], v[2]);
  C d = csub(v[1], v[2]);
  C t2, t3;
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(C) == sizeof(float2) && sizeof(T) == sizeof(float)) {  // two-lane f32x2
    t2 = f2::scale_add(-0.5f, t1, v[0]);
    t3 = f2::scale(s, d);
  } else
#endif
  {
    t2 = cmake(v[0].x - T(0.5) * t1.x, v[0].y - T(0.5) * t1.y);
    t3 = cmake(s * d.x, s * d.y);
  }
  v[0] = cadd(v[0], t1);
  C it3 = INV ? mul_i(t3) : mul_mi(t3);
  v[1] = cadd(t2, it3);
  v[2] = csub(t2, it3);
}

template <bool INV, typename C> BDDA_FFT_FN void dft4(C* v) {
  C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  C b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
  C ib1 = INV ? mul_i(b1) : mul_mi(b1);
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = cadd(a1, ib1);
  v[3] = csub(a1, ib1);
}

template <bool INV, typename C> BDDA_FFT_FN void dft5(C* v) {
  using T = decltype(C::x);
  const T c1 = T(0.30901699437494742410);   // cos(2 pi / 5)
  const T c2 = T(-0.80901699437494742410);  // cos(4 pi / 5)
  const T s1 = T(0.95105651629515357212);   // sin(2 pi / 5)
  const T s2 = T(0.58778525229247312917);   // sin(4 pi / 5)
  C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  C a1, a2, b1, b2;
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(C) == sizeof(float2) && sizeof(T) == sizeof(float)) {  // two-lane f32x2
    a1 = f2::scale_add(c2, t2, f2::scale_add(c1, t1, v[0]));
    a2 = f2::scale_add(c1, t2, f2::scale_add(c2, t1, v[0]));
    b1 = f2::scale_add(s2, t4, f2::scale(s1, t3));
    b2 = f2::scale_add(-s1, t4, f2::scale(s2, t3));
  } else
#endif
  {
    a1 = cmake(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    a2 = cmake(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    b1 = cmake(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    b2 = cmake(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  }
  C ib1 = INV ? mul_i(b1) : mul_mi(b1);
  C ib2 = INV ? mul_i(b2) : mul_mi(b2);
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(a1, ib1);
  v[4] = csub(a1, ib1);
  v[2] = cadd(a2, ib2);
  v[3] = csub(a2, ib2);
}

template <bool INV, typename C> BDDA_FFT_FN void dft8(C* v) {
  using T = decltype(C::x);
  const T h = T(0.70710678118654752440);  // 1/sqrt(2)
  C a[4], b[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    a[r] = cadd(v[r], v[r + 4]);
    b[r] = csub(v[r], v[r + 4]);
  }
  // b[r] *= exp(-+ i pi r / 4)
  if (!INV) {
    b[1] = cmake(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
    b[2] = mul_mi(b[2]);
    b[3] = cmake(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
  } else {
    b[1] = cmake(h * (b[1].x - b[1].y), h * (b[1].y + b[1].x));
    b[2] = mul_i(b[2]);
    b[3] = cmake(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));
  }
  dft4<INV>(a);
  dft4<INV>(b);
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    v[2 * m] = a[m];
    v[2 * m + 1] = b[m];
  }
}

// ---- compile-time twiddles for composite register radices -----------------
// cos / sin of 2 pi p / q evaluated at compile time: exact integer reduction
// of p/q to an octant, then Taylor series (|x| <= pi/4, 18 terms) in double.
namespace ct {
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 18; ++k) {
    term *= -x * x / ((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
constexpr double taylor_cos(double x) {
  double term = 1, sum = 1;
  for (int k = 1; k < 18; ++k) {
    term *= -x * x / ((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// angle 2 pi p / q; returns {cos, sin} (double, constexpr)
struct CS { double c, s; };
constexpr CS cossin(long long p, long long q) {
  p %= q;
  if (p < 0) p += q;
  // theta = 2 pi p / q = (pi/4) * (8p/q); octant o = floor(8p/q), remainder r in [0, 1)
  const long long o = (8 * p) / q;
  const double r = (double)(8 * p - o * q) / (double)q;  // in [0,1)
  // phi in [0, pi/4]: reflect odd octants
  const bool odd = (o & 1) != 0;
  const double phi = (odd ? (1.0 - r) : r) * (kPi / 4.0);
  double c = taylor_cos(phi), s = taylor_sin(phi);
  if (odd) { const double t = c; c = s; s = t; }   // angle = (o+1) pi/4 - phi -> swap
  // rotate by (o/2) quarter turns
  switch ((o / 2) & 3) {
    case 0: return {c, s};
    case 1: return {-s, c};
    case 2: return {-c, -s};
    default: return {s, -c};
  }
}
template <int R> struct TwTab {
  double c[R * R > 0 ? R : 1];
  double s[R * R > 0 ? R : 1];
  constexpr TwTab() : c(), s() {
    for (int i = 0; i < R; ++i) {
      const CS v = cossin(i, R);
      c[i] = v.c;
      s[i] = v.s;
    }
  }
};
}  // namespace ct

template <int R, bool INV, typename C> BDDA_FFT_FN void dft(C* v);

// Composite radix R = A * B in registers (natural-order output):
// X[B k1 + k2] = sum_n1 w_A^{n1 k1} w_R^{n1 k2} sum_n2 x[n1 + A n2] w_B^{n2 k2}.
template <int A, int B, bool INV, typename C> BDDA_FFT_FN void dft_ct(C* v) {
  using T = decltype(C::x);
  constexpr int R = A * B;
  constexpr ct::TwTab<R> tw{};
  C y[R];
#pragma unroll
  for (int n1 = 0; n1 < A; ++n1) {
    C u[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) u[n2] = v[n1 + A * n2];
    dft<B, INV>(u);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) {
      const int e = (n1 * k2) % R;
      if (e == 0) {
        y[n1 * B + k2] = u[k2];
      } else {
        const T c = T(tw.c[e]);
        const T sn = INV ? T(tw.s[e]) : T(-tw.s[e]);   // forward: exp(-2 pi i e / R)
        y[n1 * B + k2] = cmake(u[k2].x * c - u[k2].y * sn, u[k2].x * sn + u[k2].y * c);
      }
    }
  }
#pragma unroll
  for (int k2 = 0; k2 < B; ++k2) {
    C u[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) u[n1] = y[n1 * B + k2];
    dft<A, INV>(u);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) v[B * k1 + k2] = u[k1];
  }
}

template <int R, bool INV, typename C> BDDA_FFT_FN void dft(C* v) {
  if constexpr (R == 2) dft2<INV>(v);
  else if constexpr (R == 3) dft3<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else if constexpr (R == 5) dft5<INV>(v);
  else if constexpr (R == 6) dft_ct<2, 3, INV>(v);
  else if constexpr (R == 8) dft8<INV>(v);
  else if constexpr (R == 9) dft_ct<3, 3, INV>(v);
  else if constexpr (R == 10) dft_ct<2, 5, INV>(v);
  else if constexpr (R == 12) dft_ct<4, 3, INV>(v);
  else if constexpr (R == 15) dft_ct<3, 5, INV>(v);
  else if constexpr (R == 16) dft_ct<4, 4, INV>(v);
  // the first-stage radices of the complex FP32 z plans
  else if constexpr (R == 18) dft_ct<2, 9, INV>(v);
  else if constexpr (R == 20) dft_ct<4, 5, INV>(v);
  else if constexpr (R == 24) dft_ct<8, 3, INV>(v);
  else if constexpr (R == 25) dft_ct<5, 5, INV>(v);
  else if constexpr (R == 27) dft_ct<3, 9, INV>(v);
  else if constexpr (R == 30) dft_ct<2, 15, INV>(v);
  else {
    static_assert(R == 32, "register radix");
    dft_ct<4, 8, INV>(v);
  }
}

// ---- shared-memory line layout ---------------------------------------------
// Element i of a line lives at skw(i, sh) = i + (i >> sh) and consecutive
// lines are lw elements apart.  The axis plan picks sh and lw per element
// size (and the radix order) with a bank model, so that the strided butterfly
// accesses, the multi-line stages and the transposed tile loads spread over
// the 32 banks (make_axis_plan).
BDDA_FFT_FN int skw(int i, int sh) { return i + (i >> sh); }
template <typename C> BDDA_HD int plan_sk(const AxisPlan& p) { return p.sk[sizeof(C) == 8 ? 0 : 1]; }
template <typename C> BDDA_HD int plan_lw(const AxisPlan& p) { return p.lw[sizeof(C) == 8 ? 0 : 1]; }

// ---- in-place stages ---------------------------------------------------------
// One stage applied to NL lines of one warp (line j at s + j * lw); the
// butterflies of all lines share one loop so that large radices still fill
// the warp.  nvalid < N (forward first stage only): inputs at positions
// >= nvalid are known zeros and are not read (zero padding needs no fill).
template <int R, bool INV, int NL, typename C>
BDDA_FFT_FN void warp_stage_lines(C* __restrict__ s, int lw, int sh, const C* __restrict__ tw, int M, int tstride,
                                  float invM, int N, int lane, int lanes, int nvalid) {
  const int nb = N / R;
  const int Ls = M * R;
  const float inv_nb = 1.0f / (float)nb;
  for (int t = lane; t < NL * nb; t += lanes) {
    const int j = NL == 1 ? 0 : (int)(((float)t + 0.5f) * inv_nb);
    const int tt = t - j * nb;
    const int b = (int)(((float)tt + 0.5f) * invM);
    const int n1 = tt - b * M;
    const int base = b * Ls + n1;
    C* sl = s + j * lw;
    C v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (nvalid < N) v[i] = (n1 + i * M < nvalid) ? sl[skw(base + i * M, sh)] : czero<C>();
      else v[i] = sl[skw(base + i * M, sh)];
    }
    if (!INV) {
      dft<R, false>(v);
      if (n1 != 0) {
        const int step = n1 * tstride;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmul(v[k], BDDA_LDG(tw + k * step));
      }
    } else {
      if (n1 != 0) {
        const int step = n1 * tstride;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmulc(v[k], BDDA_LDG(tw + k * step));
      }
      dft<R, true>(v);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) sl[skw(base + i * M, sh)] = v[i];
  }
  BDDA_SYNCWARP();
}

// Stage dispatch over the register radices of the plans: 2, 3, 4, 5, 8 and
// the composite 6, 9, 10, 12, 15, 16; with BIG also 18, 20, 24, 25, 27, 30
// and 32, which only the complex FP32 z plans take (their first stage).  The
// kernels that can meet a complex FP32 z plan on this path -- the Green
// spectrum's z transform and the host line transform -- instantiate BIG; the
// MVP's runtime-plan kernels never do (pass C of complex FP32 runs the
// compile-time kernels for every tabled z length, and the other plans hold
// radices <= 16).
template <bool INV, int NL, typename C, bool BIG = false>
BDDA_FFT_FN void warp_stage_lines_dispatch(const AxisPlan& p, int st, C* s, int lw, const C* tw, int lane, int lanes,
                                           int nvalid) {
  const int M = p.M[st], ts = p.tstride[st], sh = plan_sk<C>(p);
  const float iM = p.invM[st];
  switch (p.radix[st]) {
    case 2: warp_stage_lines<2, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 3: warp_stage_lines<3, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 4: warp_stage_lines<4, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 5: warp_stage_lines<5, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 6: warp_stage_lines<6, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 8: warp_stage_lines<8, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 9: warp_stage_lines<9, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 10: warp_stage_lines<10, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 12: warp_stage_lines<12, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 15: warp_stage_lines<15, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 16: warp_stage_lines<16, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    default:
      if constexpr (BIG) {
        switch (p.radix[st]) {
          case 18: warp_stage_lines<18, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          case 20: warp_stage_lines<20, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          case 24: warp_stage_lines<24, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          case 25: warp_stage_lines<25, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          case 27: warp_stage_lines<27, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          case 30: warp_stage_lines<30, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
          default: warp_stage_lines<32, INV, NL>(s, lw, sh, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
        }
      }
      break;
  }
}

// NL lines of one warp transformed together (forward pruned to nvalid inputs):
// forward natural -> digit-reversed (DIF), inverse digit-reversed -> natural
// (DIT, unnormalised).
template <bool INV, int NL, typename C, bool BIG = false>
BDDA_FFT_FN void warp_fft_lines(C* __restrict__ s, int lw, const C* __restrict__ tw, const AxisPlan& p, int lane,
                                int lanes = 32, int nvalid = 1 << 30) {
  if (!INV) {
    for (int st = 0; st < p.nst; ++st)
      warp_stage_lines_dispatch<false, NL, C, BIG>(p, st, s, lw, tw, lane, lanes, st == 0 ? nvalid : p.N);
  } else {
    for (int st = p.nst - 1; st >= 0; --st)
      warp_stage_lines_dispatch<true, NL, C, BIG>(p, st, s, lw, tw, lane, lanes, p.N);
  }
}


}  // namespace bdda

