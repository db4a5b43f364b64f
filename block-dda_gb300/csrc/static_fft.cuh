// Warp FFT with a compile-time plan (complex FP32 block-MVP passes).
//
// The same in-place DIF forward / DIT inverse transform pair as the runtime
// core (fft_core.cuh: same butterflies, twiddles and digit order for the same
// radix sequence), with the plan as a type: the radix sequence, the padded
// shared-memory layout and the line pitch are template constants, so each
// butterfly element is a per-butterfly base address plus an immediate offset
// and the index arithmetic divides by constants.
//
// Twiddles come from a staged table (stage_twiddles, built on the host from
// the plan's radices): for each stage its factors, k-major, so that the lanes
// of a butterfly loop -- adjacent n1 -- load adjacent entries for each k.
//
// Layout: element idx = q * R_last + r of a line lives at q * S + r.  Every
// stage s before the last steps through its butterfly in multiples of R_last
// (M_s is a multiple of it), so its elements are (M_s / R_last) * S apart; the
// last stage's are adjacent.  Lines are LW elements apart.  The plans come
// from zplans.inc / zwplans.inc / tplans.inc / yplans.inc (gen_zplans.py).
#pragma once

#include "fft_core.cuh"

namespace bdda {
namespace sfft {

// Twiddle / spectrum load: TS = the table was staged in shared memory (a
// plain load), else an L1-cached global load.
template <bool TS, typename C> __device__ __forceinline__ C ldt(const C* p) {
  if constexpr (TS) return *p;
  else return ldg_c(p);
}

template <int N_, int S_, int LW_, int... R>
struct Plan {
  static constexpr int N = N_, S = S_, LW = LW_, nst = sizeof...(R);
  static constexpr int rad[nst] = {R...};
  static constexpr int Rl = rad[nst - 1];
  // product of the radices after stage s (the butterfly span M_s)
  static constexpr int M(int s) {
    int m = 1;
    for (int t = s + 1; t < nst; ++t) m *= rad[t];
    return m;
  }
  __device__ static __forceinline__ int addr(int idx) { return (idx / Rl) * S + idx % Rl; }
  // Offset of stage s in the staged twiddle table (stage_twiddles): stage s
  // holds w^(k n1 N / (M_s R_s)) at (k - 1) M_s + n1, k = 1 .. R_s - 1, n1 < M_s.
  static constexpr int TWO(int s) {
    int o = 0;
    for (int t = 0; t < s; ++t) o += (rad[t] - 1) * M(t);
    return o;
  }
};

// One stage over NL lines of a warp.  Forward (DIF): DFT then twiddle;
// inverse (DIT, the adjoint): conjugate twiddle then inverse DFT.  The forward
// first stage reads only inputs idx < nv (the rest are zero padding); the
// inverse last stage writes only outputs idx < nv (the rest are discarded).
// Every caller has nv <= N / 2 (a padded line is at least twice the box
// side), so in those stages (span M = N / R) the butterfly elements i with
// 2 i >= R are padding in every butterfly: compile-time zero inputs and dead
// outputs, whose DFT arithmetic the compiler folds away.
template <class P, int s, bool INV, int NL, typename C = float2, bool TS = false>
__device__ __forceinline__ void stage(C* __restrict__ sm, const C* __restrict__ tw, int lane, int nv) {
  constexpr int R = P::rad[s];
  constexpr int M = P::M(s);
  constexpr int Ls = M * R;
  constexpr int B = P::N / R;    // butterflies per line
  constexpr int T = NL * B;      // butterflies of the warp
  constexpr int off = (s == P::nst - 1) ? 1 : (M / P::Rl) * P::S;
  constexpr bool prune_in = !INV && s == 0;
  constexpr bool prune_out = INV && s == 0;
  for (int t = lane; t < T; t += 32) {
    const int j = NL == 1 ? 0 : t / B;
    const int u = t - j * B;
    const int b = u / M, n1 = u - b * M;
    const int idx0 = b * Ls + n1;
    C* p = sm + j * P::LW + P::addr(idx0);
    C v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_in) v[i] = (2 * i < R && idx0 + i * M < nv) ? p[i * off] : czero<C>();
      else v[i] = p[i * off];
    }
    if (!INV) {
      dft<R, false>(v);
      if (M > 1 && n1 != 0) {
        const C* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmul(v[k], ldt<TS>(tws + (k - 1) * M));
      }
    } else {
      if (M > 1 && n1 != 0) {
        const C* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmulc(v[k], ldt<TS>(tws + (k - 1) * M));
      }
      dft<R, true>(v);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_out) {
        if (2 * i < R && idx0 + i * M < nv) p[i * off] = v[i];
      } else {
        p[i * off] = v[i];
      }
    }
  }
  __syncwarp();
}

// First forward stage with its inputs read from global memory instead of
// shared memory: line j's element idx < nv at gsrc[j * gstride + idx] (the
// zero padding past nv is never read), results stored to the padded shared
// line as stage<P, 0, false, NL> stores them.
template <class P, int NL, typename C = float2, bool TS = false>
__device__ __forceinline__ void stage0_from_global(C* __restrict__ sm, const C* __restrict__ tw, int lane,
                                                   int nv, const C* __restrict__ gsrc, size_t gstride) {
  constexpr int R = P::rad[0];
  constexpr int M = P::M(0);       // butterflies per line (Ls = N)
  constexpr int T = NL * M;
  constexpr int off = (P::nst == 1) ? 1 : (M / P::Rl) * P::S;
  for (int t = lane; t < T; t += 32) {
    const int j = NL == 1 ? 0 : t / M;
    const int n1 = t - j * M;
    const C* g = gsrc + (size_t)j * gstride + n1;
    C v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = (2 * i < R && n1 + i * M < nv) ? g[i * M] : czero<C>();
    dft<R, false>(v);
    if (M > 1 && n1 != 0) {
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul(v[k], ldt<TS>(tw + (k - 1) * M + n1));
    }
    C* p = sm + j * P::LW + P::addr(n1);
#pragma unroll
    for (int i = 0; i < R; ++i) p[i * off] = v[i];
  }
  __syncwarp();
}

// Last inverse stage with its outputs written to global memory: line j's
// element idx < nv to gdst[j * gstride + idx] (the rest are discarded).
template <class P, int NL, typename C = float2, bool TS = false>
__device__ __forceinline__ void stage0_to_global(const C* __restrict__ sm, const C* __restrict__ tw,
                                                 int lane, int nv, C* __restrict__ gdst, size_t gstride) {
  constexpr int R = P::rad[0];
  constexpr int M = P::M(0);
  constexpr int T = NL * M;
  constexpr int off = (P::nst == 1) ? 1 : (M / P::Rl) * P::S;
  for (int t = lane; t < T; t += 32) {
    const int j = NL == 1 ? 0 : t / M;
    const int n1 = t - j * M;
    const C* p = sm + j * P::LW + P::addr(n1);
    C v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = p[i * off];
    if (M > 1 && n1 != 0) {
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmulc(v[k], ldt<TS>(tw + (k - 1) * M + n1));
    }
    dft<R, true>(v);
    C* g = gdst + (size_t)j * gstride + n1;
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (2 * i < R && n1 + i * M < nv) g[i * M] = v[i];
  }
  __syncwarp();
}

// Forward transform of NL lines: natural order in, digit-reversed out, only
// the first nv inputs read.
template <class P, int NL, int s = 0, typename C = float2>
__device__ __forceinline__ void forward(C* sm, const C* tw, int lane, int nv) {
  if constexpr (s < P::nst) {
    stage<P, s, false, NL, C>(sm, tw, lane, nv);
    forward<P, NL, s + 1, C>(sm, tw, lane, nv);
  }
}

// Forward transform whose input lines are in global memory (see stage0_from_global).
template <class P, int NL, typename C = float2>
__device__ __forceinline__ void forward_from_global(C* sm, const C* tw, int lane, int nv, const C* gsrc, size_t gstride) {
  stage0_from_global<P, NL, C>(sm, tw, lane, nv, gsrc, gstride);
  forward<P, NL, 1, C>(sm, tw, lane, nv);
}

// Forward stages s .. end - 1 of NL lines.
template <class P, int NL, int s, int end, typename C = float2, bool TS = false>
__device__ __forceinline__ void forward_to(C* sm, const C* tw, int lane, int nv) {
  if constexpr (s < end) {
    stage<P, s, false, NL, C, TS>(sm, tw, lane, nv);
    forward_to<P, NL, s + 1, end, C, TS>(sm, tw, lane, nv);
  }
}

// Last forward stage, Green product and first inverse stage of the three
// component lines of a z task in one sweep over shared memory.  The last
// forward stage has M = 1: butterfly b holds the R adjacent elements b R ..
// b R + R - 1 (at P::addr(b R) + i) and takes no twiddles, and so does the
// first inverse stage on the same elements; in between, each of the R
// frequencies is multiplied by the symmetric 3 x 3 Green spectrum (components
// xx xy xz yy yz zz, A = -G of mvp_fft/application_function.cpp:36-40), stored
// last-radix-major (frequency b R + i of component c at gl[c Pz + i (Pz / R) +
// b], green_pos), so for each (c, i) the lanes' loads are adjacent.  A thread
// does all three lines of its butterfly, so the spectrum is applied in
// registers: one shared-memory load and store per element instead of the
// separate stages' three of each.
template <class P, typename C, bool GS = false>
__device__ __forceinline__ void middle3(C* __restrict__ sm, const C* __restrict__ gl, int lane) {
  constexpr int R = P::Rl;
  constexpr int B = P::N / R;
  for (int b = lane; b < B; b += 32) {
    const int idx0 = b * R;
    C* p = sm + P::addr(idx0);
    C e0[R], e1[R], e2[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      e0[i] = p[i];
      e1[i] = p[P::LW + i];
      e2[i] = p[2 * P::LW + i];
    }
    dft<R, false>(e0);
    dft<R, false>(e1);
    dft<R, false>(e2);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const C* g = gl + i * B + b;
      const C gxx = ldt<GS>(g), gxy = ldt<GS>(g + P::N), gxz = ldt<GS>(g + 2 * P::N);
      const C gyy = ldt<GS>(g + 3 * P::N), gyz = ldt<GS>(g + 4 * P::N), gzz = ldt<GS>(g + 5 * P::N);
      const C x = e0[i], y = e1[i], z = e2[i];
      e0[i] = cadd(cadd(cmul(gxx, x), cmul(gxy, y)), cmul(gxz, z));
      e1[i] = cadd(cadd(cmul(gxy, x), cmul(gyy, y)), cmul(gyz, z));
      e2[i] = cadd(cadd(cmul(gxz, x), cmul(gyz, y)), cmul(gzz, z));
    }
    dft<R, true>(e0);
    dft<R, true>(e1);
    dft<R, true>(e2);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      p[i] = e0[i];
      p[P::LW + i] = e1[i];
      p[2 * P::LW + i] = e2[i];
    }
  }
  __syncwarp();
}

// Inverse transform (unnormalised): digit-reversed in, natural order out,
// only the first nv outputs written.
template <class P, int NL, int s = P::nst - 1, int last = 0, typename C = float2, bool TS = false>
__device__ __forceinline__ void inverse(C* sm, const C* tw, int lane, int nv) {
  if constexpr (s >= last) {
    stage<P, s, true, NL, C, TS>(sm, tw, lane, nv);
    inverse<P, NL, s - 1, last, C, TS>(sm, tw, lane, nv);
  }
}

// Inverse transform whose output lines go to global memory (see stage0_to_global).
template <class P, int NL, typename C = float2>
__device__ __forceinline__ void inverse_to_global(C* sm, const C* tw, int lane, int nv, C* gdst, size_t gstride) {
  inverse<P, NL, P::nst - 1, 1, C>(sm, tw, lane, nv);
  stage0_to_global<P, NL, C>(sm, tw, lane, nv, gdst, gstride);
}

// ---- two lines interleaved element by element ---------------------------------
// Element idx of line h (0 or 1) at sm[2 * P::addr(idx) + h]: a 16-byte pair
// per element, so a tile can be staged two columns per 16-byte copy.  Lane
// parity selects the line (t = 2 u + h), so the lanes of a butterfly's two
// lines touch adjacent words.
template <class P, int s, bool INV>
__device__ __forceinline__ void stage_il(float2* __restrict__ sm, const float2* __restrict__ tw, int lane, int nv) {
  constexpr int R = P::rad[s];
  constexpr int M = P::M(s);
  constexpr int Ls = M * R;
  constexpr int B = P::N / R;
  constexpr int T = 2 * B;
  constexpr int off = 2 * ((s == P::nst - 1) ? 1 : (M / P::Rl) * P::S);
  constexpr bool prune_in = !INV && s == 0;
  constexpr bool prune_out = INV && s == 0;
  for (int t = lane; t < T; t += 32) {
    const int h = t & 1;
    const int u = t >> 1;
    const int b = u / M, n1 = u - b * M;
    const int idx0 = b * Ls + n1;
    float2* p = sm + 2 * P::addr(idx0) + h;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_in) v[i] = (2 * i < R && idx0 + i * M < nv) ? p[i * off] : make_float2(0.f, 0.f);
      else v[i] = p[i * off];
    }
    if (!INV) {
      dft<R, false>(v);
      if (M > 1 && n1 != 0) {
        const float2* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmul(v[k], ldg_c(tws + (k - 1) * M));
      }
    } else {
      if (M > 1 && n1 != 0) {
        const float2* tws = tw + P::TWO(s) + n1;
#pragma unroll
        for (int k = 1; k < R; ++k) v[k] = cmulc(v[k], ldg_c(tws + (k - 1) * M));
      }
      dft<R, true>(v);
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (prune_out) {
        if (2 * i < R && idx0 + i * M < nv) p[i * off] = v[i];
      } else {
        p[i * off] = v[i];
      }
    }
  }
  __syncwarp();
}

template <class P, int s = 0>
__device__ __forceinline__ void forward_il(float2* sm, const float2* tw, int lane, int nv) {
  if constexpr (s < P::nst) {
    stage_il<P, s, false>(sm, tw, lane, nv);
    forward_il<P, s + 1>(sm, tw, lane, nv);
  }
}
template <class P, int s = P::nst - 1>
__device__ __forceinline__ void inverse_il(float2* sm, const float2* tw, int lane, int nv) {
  if constexpr (s >= 0) {
    stage_il<P, s, true>(sm, tw, lane, nv);
    inverse_il<P, s - 1>(sm, tw, lane, nv);
  }
}

}  // namespace sfft
}  // namespace bdda
