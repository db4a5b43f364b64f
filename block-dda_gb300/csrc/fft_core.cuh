// Warp-per-line in-place mixed-radix (2,3,4,5,8) FFT in shared memory.
//
// One warp owns one line of length N <= kMaxLine held in shared memory.
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
// are stored with a 128-byte skew (skw) so that the strided accesses of the
// last stages do not collide in shared-memory banks.
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
  C t2 = cmake(v[0].x - T(0.5) * t1.x, v[0].y - T(0.5) * t1.y);
  C d = csub(v[1], v[2]);
  C t3 = cmake(s * d.x, s * d.y);
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
  C a1 = cmake(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  C a2 = cmake(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  C b1 = cmake(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  C b2 = cmake(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
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

template <int R, bool INV, typename C> BDDA_FFT_FN void dft(C* v) {
  if constexpr (R == 2) dft2<INV>(v);
  else if constexpr (R == 3) dft3<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else if constexpr (R == 5) dft5<INV>(v);
  else dft8<INV>(v);
}

// ---- shared-memory line layout ---------------------------------------------
// Element i of a line lives at skw(i) = i + i / (128 bytes / sizeof(C)): one
// pad element per 128 bytes, so the stride-R accesses of the last stages (and
// the transposed tile loads) spread over all banks.
template <typename C> BDDA_FFT_FN int skw(int i) { return i + (i >> (sizeof(C) == 8 ? 4 : 3)); }
// Shared-memory elements one line of n points occupies (rounded to 16 bytes).
template <typename C> BDDA_HD int line_words(int n) { return ((n + (n >> (sizeof(C) == 8 ? 4 : 3)) + 1) + 1) & ~1; }

// ---- one in-place stage, one warp -----------------------------------------
// nvalid < N (forward first stage only): inputs at positions >= nvalid are
// known zeros and are not read (zero padding needs no shared-memory fill).
template <int R, bool INV, typename C>
BDDA_FFT_FN void warp_stage(C* __restrict__ s, const C* __restrict__ tw, int M, int tstride, float invM, int N,
                            int lane, int lanes, int nvalid) {
  const int nb = N / R;
  const int Ls = M * R;
  for (int t = lane; t < nb; t += lanes) {
    const int b = (int)(((float)t + 0.5f) * invM);
    const int n1 = t - b * M;
    const int base = b * Ls + n1;
    C v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (nvalid < N) v[i] = (n1 + i * M < nvalid) ? s[skw<C>(base + i * M)] : czero<C>();
      else v[i] = s[skw<C>(base + i * M)];
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
    for (int i = 0; i < R; ++i) s[skw<C>(base + i * M)] = v[i];
  }
  BDDA_SYNCWARP();
}

template <bool INV, typename C>
BDDA_FFT_FN void warp_stage_dispatch(const AxisPlan& p, int st, C* s, const C* tw, int lane, int lanes, int nvalid) {
  const int M = p.M[st], ts = p.tstride[st];
  const float iM = p.invM[st];
  switch (p.radix[st]) {
    case 2: warp_stage<2, INV>(s, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 3: warp_stage<3, INV>(s, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 4: warp_stage<4, INV>(s, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    case 5: warp_stage<5, INV>(s, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
    default: warp_stage<8, INV>(s, tw, M, ts, iM, p.N, lane, lanes, nvalid); break;
  }
}

// Full in-place transform of one line by one warp.
// INV = false: natural -> digit-reversed (DIF); only the first nvalid inputs
// are read (the rest are taken as zero).  INV = true: digit-reversed ->
// natural (DIT), unnormalised.
template <bool INV, typename C>
BDDA_FFT_FN void warp_fft(C* __restrict__ s, const C* __restrict__ tw, const AxisPlan& p, int lane, int lanes = 32,
                          int nvalid = 1 << 30) {
  if (!INV) {
    for (int st = 0; st < p.nst; ++st) warp_stage_dispatch<false>(p, st, s, tw, lane, lanes, st == 0 ? nvalid : p.N);
  } else {
    for (int st = p.nst - 1; st >= 0; --st) warp_stage_dispatch<true>(p, st, s, tw, lane, lanes, p.N);
  }
}

}  // namespace bdda
