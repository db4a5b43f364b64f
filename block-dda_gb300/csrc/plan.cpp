// FFT radix schedules and FP64 twiddle tables (host), plus a host entry point
// that runs the exact device FFT core on the CPU for unit tests.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/bdda.h"
#include "fft_core.cuh"
#include "mvp.hpp"

namespace bdda {

namespace {
// Fewest stages using register radices from `allowed` (largest first on ties
// of stage count, then the smallest largest radix for lane occupancy).
void best_factorization(int N, const std::vector<int>& allowed, std::vector<int>& cur, std::vector<int>& best) {
  if (N == 1) {
    if (best.empty() || cur.size() < best.size() ||
        (cur.size() == best.size() && *std::max_element(cur.begin(), cur.end()) < *std::max_element(best.begin(), best.end())))
      best = cur;
    return;
  }
  if (!best.empty() && cur.size() + 1 > best.size()) return;
  for (int r : allowed) {
    if (N % r) continue;
    if (!cur.empty() && r > cur.back()) continue;  // non-increasing order: each multiset once
    cur.push_back(r);
    best_factorization(N / r, allowed, cur, best);
    cur.pop_back();
  }
}
}  // namespace

bool make_axis_plan(int N, AxisPlan* p, int max_radix) {
  if (N < 1 || N > kMaxLine) return false;
  int t = N;
  for (int q : {2, 3, 5})
    while (t % q == 0) t /= q;
  if (t != 1) return false;
  p->N = N;
  p->nst = 0;
  if (max_radix <= 8) {
    int a = 0, b = 0, c = 0;
    t = N;
    while (t % 2 == 0) { t /= 2; ++a; }
    while (t % 3 == 0) { t /= 3; ++b; }
    while (t % 5 == 0) { t /= 5; ++c; }
    auto push = [&](int r) { p->radix[p->nst++] = r; };
    while (a >= 3) { push(8); a -= 3; }
    if (a == 2) push(4);
    if (a == 1) push(2);
    for (int i = 0; i < c; ++i) push(5);
    for (int i = 0; i < b; ++i) push(3);
  } else {
    const std::vector<int> allowed = {16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};
    std::vector<int> cur, best;
    best_factorization(N, allowed, cur, best);
    for (int r : best) p->radix[p->nst++] = r;
  }
  if (p->nst == 0) p->radix[p->nst++] = N == 1 ? 1 : N;  // N == 1 is rejected by callers
  int Ls = N;
  for (int s = 0; s < p->nst; ++s) {
    p->M[s] = Ls / p->radix[s];
    p->tstride[s] = N / Ls;
    p->invM[s] = 1.0f / (float)p->M[s];
    Ls = p->M[s];
  }
  return p->nst <= kMaxStages;
}

void make_twiddles(int N, std::vector<double2>* out) {
  out->resize(N);
  const double two_pi = 6.283185307179586476925286766559;
  for (int t = 0; t < N; ++t) {
    // angle reduced to the first octant-friendly form through exact integer symmetry
    long long num = t;  // exp(-2 pi i t / N)
    double c, s;
    if (4 * num == N) { c = 0.0; s = 1.0; }
    else if (2 * num == N) { c = -1.0; s = 0.0; }
    else if (4 * num == 3LL * N) { c = 0.0; s = -1.0; }
    else if (num == 0) { c = 1.0; s = 0.0; }
    else {
      const double ang = two_pi * (double)num / (double)N;
      c = std::cos(ang);
      s = std::sin(ang);
    }
    (*out)[t] = make_double2(c, -s);
  }
}

}  // namespace bdda

extern "C" {

// Runs the device FFT core (one "lane") on a host line: forward (natural ->
// digit-reversed) or inverse (digit-reversed -> natural, unnormalised).
// data: N interleaved complex values; prec 1 = FP64, 2 = FP32, 3 = double-float arithmetic
// (values are rounded to float and back).  nvalid in (0, N): the forward
// transform reads only the first nvalid inputs and takes the rest as zero
// (the pad slots hold poison values to prove it).  Returns the number of stages, or
// a negative value for an unsupported N.  Radices are written to radix (<= 16).
int bdda_host_fft_line(int N, int inverse, int prec, int nvalid, double* data, int* radix) {
  bdda::AxisPlan p;
  const int max_radix = (radix && radix[0] > 8) ? radix[0] : 8;
  if (!bdda::make_axis_plan(N, &p, max_radix)) return -1;
  std::vector<double2> tw;
  bdda::make_twiddles(N, &tw);
  // nvalid: forward transforms read only the first nvalid inputs (zero padding)
  const int nv = (nvalid > 0 && nvalid < N) ? nvalid : (1 << 30);
  if (prec == 1) {
    std::vector<double2> s(bdda::line_words<double2>(N), make_double2(1e300, 1e300));
    for (int i = 0; i < N; ++i) s[bdda::skw<double2>(i)] = make_double2(data[2 * i], data[2 * i + 1]);
    if (inverse) bdda::warp_fft_lines<true, 1>(s.data(), 0, tw.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1>(s.data(), 0, tw.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const double2 v = s[bdda::skw<double2>(i)];
      data[2 * i] = v.x; data[2 * i + 1] = v.y;
    }
  } else if (prec == 3) {
    std::vector<bdda::dfc> s(bdda::line_words<bdda::dfc>(N), bdda::cmake(bdda::dfl(1e30), bdda::dfl(1e30))), t(N);
    for (int i = 0; i < N; ++i) {
      s[bdda::skw<bdda::dfc>(i)] = bdda::cmake(bdda::dfl(data[2 * i]), bdda::dfl(data[2 * i + 1]));
      t[i] = bdda::cmake(bdda::dfl(tw[i].x), bdda::dfl(tw[i].y));
    }
    if (inverse) bdda::warp_fft_lines<true, 1>(s.data(), 0, t.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1>(s.data(), 0, t.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const bdda::dfc v = s[bdda::skw<bdda::dfc>(i)];
      data[2 * i] = bdda::df_to_double(v.x); data[2 * i + 1] = bdda::df_to_double(v.y);
    }
  } else {
    std::vector<float2> s(bdda::line_words<float2>(N), make_float2(1e30f, 1e30f)), t(N);
    for (int i = 0; i < N; ++i) {
      s[bdda::skw<float2>(i)] = make_float2((float)data[2 * i], (float)data[2 * i + 1]);
      t[i] = make_float2((float)tw[i].x, (float)tw[i].y);
    }
    if (inverse) bdda::warp_fft_lines<true, 1>(s.data(), 0, t.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1>(s.data(), 0, t.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const float2 v = s[bdda::skw<float2>(i)];
      data[2 * i] = v.x; data[2 * i + 1] = v.y;
    }
  }
  if (radix)
    for (int i = 0; i < p.nst; ++i) radix[i] = p.radix[i];
  return p.nst;
}

}  // extern "C"
