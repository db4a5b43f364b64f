// Spectral product of the fused z pass at one frequency of one (x, y, rhs)
// task, in place on the task's component lines (line c at s + c * lw, element
// offset a).  The Green spectrum of the (x, y) line holds nc = 6 or 9
// components of Pz frequencies each (gl[comp * Pz + p]):
//   f = 3: A = -G, symmetric, components xx xy xz yy yz zz;  E' = A E
//          (mvp_fft/application_function.cpp:36-40)
//   f = 6: also B = -F, antisymmetric, components xy xz yz (B_yx = -B_xy ...);
//          [E'; M'] = [[A, B], [-B, A]] [E; M], the block
//          [[-G, -F], [F, -G]] of mvp_fft/application_function.cpp:53-68.
#pragma once

#include "common.cuh"

namespace bdda {

// GS: the spectrum was staged in shared memory (plain loads), else L1-cached
// global loads.
template <typename C, bool GS = false>
__device__ __forceinline__ void z_product(C* __restrict__ s, int lw, int a, const C* __restrict__ gl, int Pz, int p,
                                          bool six) {
  auto ld = [](const C* q) -> C {
    if constexpr (GS) return *q;
    else return ldg_c(q);
  };
  const C e0 = s[a], e1 = s[lw + a], e2 = s[2 * lw + a];
  const C gxx = ld(gl + p), gxy = ld(gl + Pz + p), gxz = ld(gl + 2 * Pz + p);
  const C gyy = ld(gl + 3 * Pz + p), gyz = ld(gl + 4 * Pz + p), gzz = ld(gl + 5 * Pz + p);
  C ox = cadd(cadd(cmul(gxx, e0), cmul(gxy, e1)), cmul(gxz, e2));
  C oy = cadd(cadd(cmul(gxy, e0), cmul(gyy, e1)), cmul(gyz, e2));
  C oz = cadd(cadd(cmul(gxz, e0), cmul(gyz, e1)), cmul(gzz, e2));
  if (six) {
    const C m0 = s[3 * lw + a], m1 = s[4 * lw + a], m2 = s[5 * lw + a];
    const C bxy = ld(gl + 6 * Pz + p), bxz = ld(gl + 7 * Pz + p), byz = ld(gl + 8 * Pz + p);
    // E' = A E + B M
    ox = cadd(ox, cadd(cmul(bxy, m1), cmul(bxz, m2)));
    oy = cadd(oy, csub(cmul(byz, m2), cmul(bxy, m0)));
    oz = csub(oz, cadd(cmul(bxz, m0), cmul(byz, m1)));
    // M' = A M - B E
    const C px = csub(cadd(cadd(cmul(gxx, m0), cmul(gxy, m1)), cmul(gxz, m2)), cadd(cmul(bxy, e1), cmul(bxz, e2)));
    const C py = cadd(csub(cadd(cmul(gxy, m0), cmul(gyy, m1)), cmul(byz, e2)), cadd(cmul(gyz, m2), cmul(bxy, e0)));
    const C pz = cadd(cadd(cadd(cmul(gxz, m0), cmul(gyz, m1)), cmul(gzz, m2)), cadd(cmul(bxz, e0), cmul(byz, e1)));
    s[3 * lw + a] = px;
    s[4 * lw + a] = py;
    s[5 * lw + a] = pz;
  }
  s[a] = ox;
  s[lw + a] = oy;
  s[2 * lw + a] = oz;
}

}  // namespace bdda
