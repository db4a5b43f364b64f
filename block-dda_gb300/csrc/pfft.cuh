// Packed-pair complex FP32 FFT: two lines per thread in the two lanes of
// sm_100-family f32x2 instructions (add / sub / mul / fma .rn.f32x2).
//
// A pair value holds element idx of two lines a and b as two 64-bit register
// pairs, re = {re_a, re_b} and im = {im_a, im_b}.  Every complex operation of
// the transform is then the same operation on both lanes, so one packed
// instruction does the work of two scalar ones; a butterfly element is one
// 16-byte shared-memory access ({re_a, re_b, im_a, im_b}) instead of two
// 8-byte ones, and the index arithmetic is shared by the two lines.
//
// The radix kernels compute the same DFTs as fft_core.cuh (same directions:
// forward exp(-2 pi i / R), inverse exp(+2 pi i / R); same output order), with
// the multiplications by +-i folded into the adjacent additions (packed
// arithmetic has no lane swap).  The stage functions mirror static_fft.cuh
// (same plans, digit order and pruning) on 16-byte elements.
#pragma once

#include "fft_core.cuh"

namespace bdda {
namespace pk {

typedef unsigned long long u64;

// ---- two-lane FP32 primitives ----------------------------------------------
__device__ __forceinline__ u64 p2(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ u64 dup(float a) { return p2(a, a); }
__device__ __forceinline__ void unp(u64 r, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ u64 add(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 sub(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 mul(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// a * b + c
__device__ __forceinline__ u64 fma(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// ---- complex pairs -----------------------------------------------------------
struct cp {
  u64 re, im;
};
__device__ __forceinline__ cp cadd(cp a, cp b) { return {add(a.re, b.re), add(a.im, b.im)}; }
__device__ __forceinline__ cp csub(cp a, cp b) { return {sub(a.re, b.re), sub(a.im, b.im)}; }
__device__ __forceinline__ cp add_i(cp a, cp b) { return {sub(a.re, b.im), add(a.im, b.re)}; }  // a + i b
__device__ __forceinline__ cp sub_i(cp a, cp b) { return {add(a.re, b.im), sub(a.im, b.re)}; }  // a - i b
// a (c + i s) for constants c, s (exact 0 / +-1 parts folded away after unrolling)
__device__ __forceinline__ cp rot(cp a, float c, float s) {
  if (s == 0.0f) {
    if (c == 1.0f) return a;
    return {mul(a.re, dup(c)), mul(a.im, dup(c))};
  }
  if (c == 0.0f) {
    if (s == 1.0f) return {sub(0ull, a.im), a.re};   // i a  (0ull is +0, +0)
    if (s == -1.0f) return {a.im, sub(0ull, a.re)};  // -i a
  }
  return {fma(a.im, dup(-s), mul(a.re, dup(c))), fma(a.re, dup(s), mul(a.im, dup(c)))};
}
// a w and a conj(w) for a twiddle pair table entry {wx, wx, wy, wy}
__device__ __forceinline__ void ld_tw(const float4* p, u64& c, u64& s) {
  asm("ld.global.nc.v2.u64 {%0, %1}, [%2];" : "=l"(c), "=l"(s) : "l"(p));
}
__device__ __forceinline__ cp tw_mul(cp a, u64 c, u64 s) { return {sub(mul(a.re, c), mul(a.im, s)), fma(a.re, s, mul(a.im, c))}; }
__device__ __forceinline__ cp tw_mulc(cp a, u64 c, u64 s) { return {fma(a.im, s, mul(a.re, c)), sub(mul(a.im, c), mul(a.re, s))}; }

// 16-byte shared-memory element {re_a, re_b, im_a, im_b}
__device__ __forceinline__ cp lds(const ulonglong2* p) {
  const ulonglong2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ void sts(ulonglong2* p, cp v) { *p = make_ulonglong2(v.re, v.im); }

// ---- radix kernels -------------------------------------------------------------
template <bool INV> __device__ __forceinline__ void d2(cp* v) {
  const cp a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <bool INV> __device__ __forceinline__ void d3(cp* v) {
  const float s = 0.86602540378443864676f;  // sin(2 pi / 3)
  const cp t1 = cadd(v[1], v[2]);
  const cp t2 = {fma(t1.re, dup(-0.5f), v[0].re), fma(t1.im, dup(-0.5f), v[0].im)};
  const cp d = csub(v[1], v[2]);
  v[0] = cadd(v[0], t1);
  const cp p = {fma(d.im, dup(-s), t2.re), fma(d.re, dup(s), t2.im)};  // t2 + i s d
  const cp m = {fma(d.im, dup(s), t2.re), fma(d.re, dup(-s), t2.im)};  // t2 - i s d
  v[1] = INV ? p : m;
  v[2] = INV ? m : p;
}

template <bool INV> __device__ __forceinline__ void d4(cp* v) {
  const cp a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  const cp b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = INV ? add_i(a1, b1) : sub_i(a1, b1);
  v[3] = INV ? sub_i(a1, b1) : add_i(a1, b1);
}

template <bool INV> __device__ __forceinline__ void d5(cp* v) {
  const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
  const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
  const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
  const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
  const cp t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const cp t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  const cp a1 = {fma(t2.re, dup(c2), fma(t1.re, dup(c1), v[0].re)), fma(t2.im, dup(c2), fma(t1.im, dup(c1), v[0].im))};
  const cp a2 = {fma(t2.re, dup(c1), fma(t1.re, dup(c2), v[0].re)), fma(t2.im, dup(c1), fma(t1.im, dup(c2), v[0].im))};
  const cp b1 = {fma(t4.re, dup(s2), mul(t3.re, dup(s1))), fma(t4.im, dup(s2), mul(t3.im, dup(s1)))};
  const cp b2 = {fma(t4.re, dup(-s1), mul(t3.re, dup(s2))), fma(t4.im, dup(-s1), mul(t3.im, dup(s2)))};
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = INV ? add_i(a1, b1) : sub_i(a1, b1);
  v[4] = INV ? sub_i(a1, b1) : add_i(a1, b1);
  v[2] = INV ? add_i(a2, b2) : sub_i(a2, b2);
  v[3] = INV ? sub_i(a2, b2) : add_i(a2, b2);
}

template <bool INV> __device__ __forceinline__ void d8(cp* v) {
  const float h = 0.70710678118654752440f;  // 1/sqrt(2)
  cp a[4], b[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    a[r] = cadd(v[r], v[r + 4]);
    b[r] = csub(v[r], v[r + 4]);
  }
  // b[1] *= exp(-+ i pi / 4), b[3] *= exp(-+ 3 i pi / 4); b[2] *= -+i folded below
  if (!INV) {
    b[1] = {mul(add(b[1].re, b[1].im), dup(h)), mul(sub(b[1].im, b[1].re), dup(h))};
    b[3] = {mul(sub(b[3].im, b[3].re), dup(h)), mul(add(b[3].re, b[3].im), dup(-h))};
  } else {
    b[1] = {mul(sub(b[1].re, b[1].im), dup(h)), mul(add(b[1].re, b[1].im), dup(h))};
    b[3] = {mul(add(b[3].re, b[3].im), dup(-h)), mul(sub(b[3].re, b[3].im), dup(h))};
  }
  d4<INV>(a);
  // radix 4 on b with b[2] pre-multiplied by -+i
  const cp e0 = INV ? add_i(b[0], b[2]) : sub_i(b[0], b[2]);
  const cp e1 = INV ? sub_i(b[0], b[2]) : add_i(b[0], b[2]);
  const cp f0 = cadd(b[1], b[3]), f1 = csub(b[1], b[3]);
  b[0] = cadd(e0, f0);
  b[2] = csub(e0, f0);
  b[1] = INV ? add_i(e1, f1) : sub_i(e1, f1);
  b[3] = INV ? sub_i(e1, f1) : add_i(e1, f1);
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    v[2 * m] = a[m];
    v[2 * m + 1] = b[m];
  }
}

template <int R, bool INV> __device__ __forceinline__ void dft(cp* v);

// composite R = A * B in registers, natural-order output (as fft_core.cuh dft_ct)
template <int A, int B, bool INV> __device__ __forceinline__ void dct(cp* v) {
  constexpr int R = A * B;
  constexpr ct::TwTab<R> tw{};
  cp y[R];
#pragma unroll
  for (int n1 = 0; n1 < A; ++n1) {
    cp u[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) u[n2] = v[n1 + A * n2];
    dft<B, INV>(u);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) {
      const int e = (n1 * k2) % R;
      const float c = (float)tw.c[e];
      const float s = INV ? (float)tw.s[e] : (float)-tw.s[e];
      y[n1 * B + k2] = e == 0 ? u[k2] : rot(u[k2], c, s);
    }
  }
#pragma unroll
  for (int k2 = 0; k2 < B; ++k2) {
    cp u[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) u[n1] = y[n1 * B + k2];
    dft<A, INV>(u);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) v[B * k1 + k2] = u[k1];
  }
}

template <int R, bool INV> __device__ __forceinline__ void dft(cp* v) {
  if constexpr (R == 2) d2<INV>(v);
  else if constexpr (R == 3) d3<INV>(v);
  else if constexpr (R == 4) d4<INV>(v);
  else if constexpr (R == 5) d5<INV>(v);
  else if constexpr (R == 6) dct<2, 3, INV>(v);
  else if constexpr (R == 8) d8<INV>(v);
  else if constexpr (R == 9) dct<3, 3, INV>(v);
  else if constexpr (R == 10) dct<2, 5, INV>(v);
  else if constexpr (R == 12) dct<4, 3, INV>(v);
  else if constexpr (R == 15) dct<3, 5, INV>(v);
  else dct<4, 4, INV>(v);  // 16
}

// ---- stages on 16-byte shared-memory elements (compile-time plan P) -------------
// NP line pairs per warp; pair j's element idx at sm[j * P::LW + P::addr(idx)].
// tw: staged twiddle pair table ({wx, wx, wy, wy} entries, same layout as
// sfft's staged table: stage s at P::TWO(s), entry (k - 1) M_s + n1).
template <class P, int s, bool INV, int NP>
__device__ __forceinline__ void stage(ulonglong2* __restrict__ sm, const float4* __restrict__ tw, int lane, int nv) {
  constexpr int R = P::rad[s];
  constexpr int M = P::M(s);
  constexpr int Ls = M * R;
  constexpr int B = P::N / R;
  constexpr int T = NP * B;
  constexpr int off = (s == P::nst - 1) ? 1 : (M / P::Rl) * P::S;
  constexpr bool prune_in = !INV && s == 0;
  constexpr bool prune_out = INV && s == 0;
  for (int t = lane; t < T; t += 32) {
    const int j = NP == 1 ? 0 : t / B;
    const int u = t - j * B;
    const int b = u / M, n1 = u - b * M;
    const int idx0 = b * Ls + n1;
    ulonglong2* p = sm + j * P::LW + P::addr(idx0);
    cp v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_in) v[i] = (2 * i < R && idx0 + i * M < nv) ? lds(p + i * off) : cp{0ull, 0ull};
      else v[i] = lds(p + i * off);
    }
    if (!INV) {
      dft<R, false>(v);
      if (M > 1 && n1 != 0) {
        const float4* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) {
          u64 c, sn;
          ld_tw(tws + (k - 1) * M, c, sn);
          v[k] = tw_mul(v[k], c, sn);
        }
      }
    } else {
      if (M > 1 && n1 != 0) {
        const float4* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) {
          u64 c, sn;
          ld_tw(tws + (k - 1) * M, c, sn);
          v[k] = tw_mulc(v[k], c, sn);
        }
      }
      dft<R, true>(v);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_out) {
        if (2 * i < R && idx0 + i * M < nv) sts(p + i * off, v[i]);
      } else {
        sts(p + i * off, v[i]);
      }
    }
  }
  __syncwarp();
}

// First forward stage reading the two lines of each pair from global memory:
// pair j's lines at ga + j * gstride and ga + j * gstride + boff, elements
// idx < nv (the zero padding is never read).
template <class P, int NP>
__device__ __forceinline__ void stage0_from_global(ulonglong2* __restrict__ sm, const float4* __restrict__ tw, int lane,
                                                   int nv, const float2* __restrict__ ga, size_t gstride, ptrdiff_t boff) {
  constexpr int R = P::rad[0];
  constexpr int M = P::M(0);
  constexpr int T = NP * M;
  constexpr int off = (P::nst == 1) ? 1 : (M / P::Rl) * P::S;
  for (int t = lane; t < T; t += 32) {
    const int j = NP == 1 ? 0 : t / M;
    const int n1 = t - j * M;
    const float2* g = ga + (size_t)j * gstride + n1;
    cp v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (2 * i < R && n1 + i * M < nv) {  // nv <= N / 2, as in sfft::stage
        const float2 x = g[i * M], y = g[i * M + boff];
        v[i] = {p2(x.x, y.x), p2(x.y, y.y)};
      } else {
        v[i] = {0ull, 0ull};
      }
    }
    dft<R, false>(v);
    if (M > 1 && n1 != 0) {
#pragma unroll
      for (int k = 1; k < R; ++k) {
        u64 c, sn;
        ld_tw(tw + (k - 1) * M + n1, c, sn);
        v[k] = tw_mul(v[k], c, sn);
      }
    }
    ulonglong2* p = sm + j * P::LW + P::addr(n1);
#pragma unroll
    for (int i = 0; i < R; ++i) sts(p + i * off, v[i]);
  }
  __syncwarp();
}

// Last inverse stage writing the pairs' lines to global memory (elements
// idx < nv; the second line only when write_b).
template <class P, int NP>
__device__ __forceinline__ void stage0_to_global(const ulonglong2* __restrict__ sm, const float4* __restrict__ tw,
                                                 int lane, int nv, float2* __restrict__ ga, size_t gstride,
                                                 ptrdiff_t boff, bool write_b) {
  constexpr int R = P::rad[0];
  constexpr int M = P::M(0);
  constexpr int T = NP * M;
  constexpr int off = (P::nst == 1) ? 1 : (M / P::Rl) * P::S;
  for (int t = lane; t < T; t += 32) {
    const int j = NP == 1 ? 0 : t / M;
    const int n1 = t - j * M;
    const ulonglong2* p = sm + j * P::LW + P::addr(n1);
    cp v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = lds(p + i * off);
    if (M > 1 && n1 != 0) {
#pragma unroll
      for (int k = 1; k < R; ++k) {
        u64 c, sn;
        ld_tw(tw + (k - 1) * M + n1, c, sn);
        v[k] = tw_mulc(v[k], c, sn);
      }
    }
    dft<R, true>(v);
    float2* g = ga + (size_t)j * gstride + n1;
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (2 * i < R && n1 + i * M < nv) {
        float ra, rb, ia, ib;
        unp(v[i].re, ra, rb);
        unp(v[i].im, ia, ib);
        g[i * M] = make_float2(ra, ia);
        if (write_b) g[i * M + boff] = make_float2(rb, ib);
      }
  }
  __syncwarp();
}

// Forward stages s .. end - 1.
template <class P, int NP, int s, int end>
__device__ __forceinline__ void forward_to(ulonglong2* sm, const float4* tw, int lane, int nv) {
  if constexpr (s < end) {
    stage<P, s, false, NP>(sm, tw, lane, nv);
    forward_to<P, NP, s + 1, end>(sm, tw, lane, nv);
  }
}

// Last forward stage, Green product and first inverse stage of a task's three
// line pairs in one sweep (the packed form of sfft::middle3): butterfly b of
// the last stage (M = 1, no twiddles) in all three component pairs, the
// symmetric 3 x 3 spectrum (last-radix-major, green_pos) of each of its R
// frequencies applied in registers, the inverse DFT, one store.  Used for
// R <= 5 (3 R pair elements, 12 R registers; zpacked::supported).
template <class P>
__device__ __forceinline__ void middle3(ulonglong2* __restrict__ sm, const float2* __restrict__ gl, int lane) {
  constexpr int R = P::Rl;
  constexpr int B = P::N / R;
  constexpr int m[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int b = lane; b < B; b += 32) {
    const int idx0 = b * R;
    ulonglong2* p = sm + P::addr(idx0);
    cp e[3][R];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int i = 0; i < R; ++i) e[c][i] = lds(p + c * P::LW + i);
      dft<R, false>(e[c]);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      u64 gr[6], gi[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float2 g = ldg_c(gl + c * P::N + i * B + b);
        gr[c] = dup(g.x);
        gi[c] = dup(g.y);
      }
      cp o3[3];
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        // re' = sum re_d gr - sum im_d gi ; im' = sum im_d gr + re_d gi
        u64 ar = mul(e[0][i].re, gr[m[o][0]]);
        ar = fma(e[1][i].re, gr[m[o][1]], ar);
        ar = fma(e[2][i].re, gr[m[o][2]], ar);
        u64 ai = mul(e[0][i].im, gi[m[o][0]]);
        ai = fma(e[1][i].im, gi[m[o][1]], ai);
        ai = fma(e[2][i].im, gi[m[o][2]], ai);
        u64 bi = mul(e[0][i].im, gr[m[o][0]]);
        bi = fma(e[1][i].im, gr[m[o][1]], bi);
        bi = fma(e[2][i].im, gr[m[o][2]], bi);
        bi = fma(e[0][i].re, gi[m[o][0]], bi);
        bi = fma(e[1][i].re, gi[m[o][1]], bi);
        bi = fma(e[2][i].re, gi[m[o][2]], bi);
        o3[o] = cp{sub(ar, ai), bi};
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) e[c][i] = o3[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dft<R, true>(e[c]);
#pragma unroll
      for (int i = 0; i < R; ++i) sts(p + c * P::LW + i, e[c][i]);
    }
  }
  __syncwarp();
}

template <class P, int NP, int s = 0>
__device__ __forceinline__ void forward(ulonglong2* sm, const float4* tw, int lane, int nv) {
  if constexpr (s < P::nst) {
    stage<P, s, false, NP>(sm, tw, lane, nv);
    forward<P, NP, s + 1>(sm, tw, lane, nv);
  }
}
template <class P, int NP, int s = P::nst - 1, int last = 0>
__device__ __forceinline__ void inverse(ulonglong2* sm, const float4* tw, int lane, int nv) {
  if constexpr (s >= last) {
    stage<P, s, true, NP>(sm, tw, lane, nv);
    inverse<P, NP, s - 1, last>(sm, tw, lane, nv);
  }
}

}  // namespace pk
}  // namespace bdda
