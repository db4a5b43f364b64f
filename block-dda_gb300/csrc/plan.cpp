// FFT radix schedules and FP64 twiddle tables (host), plus a host entry point
// that runs the exact device FFT core on the CPU for unit tests.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/bdda.h"
#include "fft_core.cuh"
#include "mvp.hpp"

namespace bdda {

namespace {
// Fewest stages using register radices from `allowed`.
int min_stages(int N, const std::vector<int>& allowed, int depth, int best) {
  if (N == 1) return depth;
  if (depth + 1 >= best) return best;
  for (int r : allowed)
    if (N % r == 0) best = std::min(best, min_stages(N / r, allowed, depth + 1, best));
  return best;
}

// Every ordered radix sequence of exactly `len` stages with product N.
void sequences(int N, const std::vector<int>& allowed, int len, std::vector<int>& cur,
               std::vector<std::vector<int>>& out) {
  if ((int)cur.size() == len) {
    if (N == 1) out.push_back(cur);
    return;
  }
  for (int r : allowed) {
    if (N % r) continue;
    cur.push_back(r);
    sequences(N / r, allowed, len, cur, out);
    cur.pop_back();
  }
}

// ---- shared-memory bank model ----------------------------------------------
// 32 banks of 4 bytes.  8-byte accesses of a warp are served per half-warp and
// 16-byte accesses per quarter-warp; a group takes as many wavefronts as the
// largest number of distinct 4-byte words that fall into one bank.  (This
// reproduces the shared-memory wavefront counts ncu reports for the passes.)
int wavefronts(const int* addr, int n, int esize) {
  const int g = 128 / esize, wpe = esize / 4;
  int total = 0;
  for (int g0 = 0; g0 < n; g0 += g) {
    int cnt[32] = {0};
    int words[32][16];
    int worst = 0;
    const int g1 = std::min(n, g0 + g);
    for (int l = g0; l < g1; ++l)
      for (int k = 0; k < wpe; ++k) {
        const int w = addr[l] * wpe + k, b = w & 31;
        bool seen = false;
        for (int q = 0; q < cnt[b] && !seen; ++q) seen = words[b][q] == w;
        if (!seen) {
          words[b][cnt[b]++] = w;
          worst = std::max(worst, cnt[b]);
        }
      }
    total += worst;
  }
  return total;
}

int skew(int i, int sh) { return i + (i >> sh); }

// Butterfly loads of one transform over NL lines of pitch lw, lanes mapped as
// warp_stage_lines maps them (the stores repeat the same addresses).
long stage_cost(int N, const std::vector<int>& rad, int NL, int lw, int sh, int esize) {
  long c = 0;
  int addr[32];
  int Ls = N;
  for (int R : rad) {
    const int M = Ls / R, nb = N / R;
    for (int t0 = 0; t0 < NL * nb; t0 += 32) {
      const int n = std::min(32, NL * nb - t0);
      for (int i = 0; i < R; ++i) {
        for (int l = 0; l < n; ++l) {
          const int t = t0 + l, j = t / nb, tt = t - j * nb, b = tt / M, n1 = tt - b * M;
          addr[l] = j * lw + skew(b * Ls + n1 + i * M, sh);
        }
        c += wavefronts(addr, n, esize);
      }
    }
    Ls = M;
  }
  return c;
}

// Tile transposes of the strided passes: idx -> line idx & 7, position idx >> 3.
long tile_cost(int N, int lw, int sh, int esize) {
  long c = 0;
  int addr[32];
  for (int i0 = 0; i0 < 8 * N; i0 += 32) {
    const int n = std::min(32, 8 * N - i0);
    for (int l = 0; l < n; ++l) addr[l] = ((i0 + l) & 7) * lw + skew((i0 + l) >> 3, sh);
    c += wavefronts(addr, n, esize);
  }
  return c;
}

// Contiguous per-line accesses (loads, stores and the spectral product of the z pass).
long contig_cost(int N, int NL, int lw, int sh, int esize) {
  long c = 0;
  int addr[32];
  for (int j = 0; j < NL; ++j)
    for (int z0 = 0; z0 < N; z0 += 32) {
      const int n = std::min(32, N - z0);
      for (int l = 0; l < n; ++l) addr[l] = j * lw + skew(z0 + l, sh);
      c += wavefronts(addr, n, esize);
    }
  return c;
}

constexpr int kNoSkew = 31;
const int kShifts[] = {kNoSkew, 3, 4, 5, 6, 7, 8};

// Modelled wavefronts per line of the pass that uses the plan: single-line
// plans serve the tile passes (one forward or inverse transform + a tile fill
// and drain), three-line plans the fused z pass (forward + inverse + the
// contiguous load, product and store).
long plan_cost(int N, const std::vector<int>& rad, bool three, int lw, int sh, int esize) {
  if (three) return 2 * stage_cost(N, rad, 3, lw, sh, esize) + 2 * contig_cost(N, 3, lw, sh, esize);
  return stage_cost(N, rad, 1, lw, sh, esize) + tile_cost(N, lw, sh, esize);
}

struct Layout { long cost; int sh, lw; };

Layout best_layout(int N, const std::vector<int>& rad, bool three, int esize) {
  Layout best{-1, kNoSkew, N};
  const int dmax = esize == 8 ? 16 : 8;
  for (int sh : kShifts)
    for (int d = 0; d < dmax; ++d) {
      const int lw = skew(N - 1, sh) + 1 + d;
      const long c = plan_cost(N, rad, three, lw, sh, esize);
      if (best.cost < 0 || c < best.cost) best = {c, sh, lw};
    }
  return best;
}

struct PlanChoice { std::vector<int> rad; Layout l8, l16; };

// Radix sequences of the compile-time plans: the complex FP32 fused z pass
// (three-line plans, first-stage radices up to 32) ...
struct PlanRow { int N, S, LW; int rad[kMaxStages]; };
constexpr PlanRow kZPlans[] = {
#define BDDA_ZPLAN(I, N, S, LW, ...) {N, S, LW, {__VA_ARGS__}},
#include "zplans.inc"
#undef BDDA_ZPLAN
};
// ... the 16-byte (FP64 / double-float) z passes (radices <= 16) ...
constexpr PlanRow kZWPlans[] = {
#define BDDA_ZWPLAN(I, N, S, LW, ...) {N, S, LW, {__VA_ARGS__}},
#include "zwplans.inc"
#undef BDDA_ZWPLAN
};
// ... and of the strided x / y passes (single-line plans).
constexpr PlanRow kTPlans[] = {
#define BDDA_TPLAN(I, N, S, LW, ...) {N, S, LW, {__VA_ARGS__}},
#include "tplans.inc"
#undef BDDA_TPLAN
};

template <size_t K>
bool table_radices(const PlanRow (&tab)[K], int N, std::vector<int>* rad) {
  for (const PlanRow& z : tab)
    if (z.N == N) {
      rad->clear();
      for (int s = 0; s < kMaxStages && z.rad[s] > 0; ++s) rad->push_back(z.rad[s]);
      return true;
    }
  return false;
}

// Radix order, skew and pitch by the bank model: among the fewest-stage radix
// sequences, the one whose best 8-byte layout takes the fewest wavefronts
// (complex FP32 is the hot precision); the 16-byte layout is then fitted to it.
// Radix sequence: the compile-time tables' for complex FP32 and for every
// z axis (each element width its own z table, and so its own Green spectrum
// order); otherwise (16-byte tile passes) the fewest-stage sequence of radices
// <= 8 whose best 16-byte layout takes the fewest wavefronts.  Then the best
// layout of each element width for that sequence.
PlanChoice choose_plan(int N, bool three, bool wide) {
  PlanChoice best;
  const bool tabled = three ? table_radices(wide ? kZWPlans : kZPlans, N, &best.rad)
                            : (!wide && table_radices(kTPlans, N, &best.rad));
  if (!tabled) {
    const std::vector<int> allowed = three ? std::vector<int>{16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2}
                                           : std::vector<int>{8, 5, 4, 3, 2};
    const int es = wide ? 16 : 8;
    const int len = min_stages(N, allowed, 0, 64);
    std::vector<std::vector<int>> seqs;
    std::vector<int> cur;
    sequences(N, allowed, len, cur, seqs);
    // coarse pass: every sequence and shift at the minimal pitch; the best few then get every pitch
    struct Cand { long cost; size_t s; };
    std::vector<Cand> cand;
    for (size_t i = 0; i < seqs.size(); ++i) {
      long c = -1;
      for (int sh : kShifts) {
        const long v = plan_cost(N, seqs[i], three, skew(N - 1, sh) + 1, sh, es);
        if (c < 0 || v < c) c = v;
      }
      cand.push_back({c, i});
    }
    std::stable_sort(cand.begin(), cand.end(), [](const Cand& a, const Cand& b) { return a.cost < b.cost; });
    long bc = -1;
    for (size_t k = 0; k < cand.size() && k < 4; ++k) {
      const Layout l = best_layout(N, seqs[cand[k].s], three, es);
      if (bc < 0 || l.cost < bc) {
        best.rad = seqs[cand[k].s];
        bc = l.cost;
      }
    }
  }
  best.l8 = best_layout(N, best.rad, three, 8);
  best.l16 = best_layout(N, best.rad, three, 16);
  return best;
}
}  // namespace

bool make_axis_plan(int N, AxisPlan* p, bool three, bool wide) {
  if (N < 2 || N > kMaxLine) return false;
  int t = N;
  for (int q : {2, 3, 5})
    while (t % q == 0) t /= q;
  if (t != 1) return false;
  static std::mutex mu;
  static std::map<std::tuple<int, bool, bool>, PlanChoice> cache;
  PlanChoice ch;
  {
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(N, three, wide);
    auto it = cache.find(key);
    if (it == cache.end()) it = cache.emplace(key, choose_plan(N, three, wide)).first;
    ch = it->second;
  }
  if ((int)ch.rad.size() > kMaxStages) return false;
  p->N = N;
  p->nst = (int)ch.rad.size();
  int Ls = N;
  for (int s = 0; s < p->nst; ++s) {
    p->radix[s] = ch.rad[s];
    p->M[s] = Ls / p->radix[s];
    p->tstride[s] = N / Ls;
    p->invM[s] = 1.0f / (float)p->M[s];
    Ls = p->M[s];
  }
  p->sk[0] = ch.l8.sh;
  p->lw[0] = ch.l8.lw;
  p->sk[1] = ch.l16.sh;
  p->lw[1] = ch.l16.lw;
  return p->lw[0] <= kMaxLineWords && p->lw[1] <= kMaxLineWords;
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

void stage_twiddles(const AxisPlan& p, std::vector<double2>* out) {
  std::vector<double2> w;
  make_twiddles(p.N, &w);
  out->clear();
  int Ls = p.N;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.radix[s], M = Ls / R, ts = p.N / Ls;
    for (int k = 1; k < R; ++k)
      for (int n1 = 0; n1 < M; ++n1) out->push_back(w[(size_t)k * n1 * ts]);  // k n1 ts < N
    Ls = M;
  }
}

}  // namespace bdda

extern "C" {

// Runs the device FFT core (one "lane") on a host line: forward (natural ->
// digit-reversed) or inverse (digit-reversed -> natural, unnormalised).
// data: N interleaved complex values; prec 1 = FP64, 2 = FP32, 3 = double-float arithmetic
// (values are rounded to float and back).  nvalid in (0, N): the forward
// transform reads only the first nvalid inputs and takes the rest as zero
// (the pad slots hold poison values to prove it).  radix[0] > 8 on input: the
// z-axis schedule, else the x / y one, each for the element width of prec;
// radix[1] = 1 on input: the complex FP32 schedule in any arithmetic (its
// Green spectrum is transformed in FP64).  Returns the number of stages, or a
// negative value for an unsupported N.  Radices are written to radix (<= 32).
int bdda_host_fft_line(int N, int inverse, int prec, int nvalid, double* data, int* radix) {
  bdda::AxisPlan p;
  const bool three = radix && radix[0] > 8;
  const bool wide = (radix && radix[1] == 1) ? false : prec != 2;
  if (!bdda::make_axis_plan(N, &p, three, wide)) return -1;
  std::vector<double2> tw;
  bdda::make_twiddles(N, &tw);
  // nvalid: forward transforms read only the first nvalid inputs (zero padding)
  const int nv = (nvalid > 0 && nvalid < N) ? nvalid : (1 << 30);
  if (prec == 1) {
    const int sh = bdda::plan_sk<double2>(p);
    std::vector<double2> s(bdda::plan_lw<double2>(p), make_double2(1e300, 1e300));
    for (int i = 0; i < N; ++i) s[bdda::skw(i, sh)] = make_double2(data[2 * i], data[2 * i + 1]);
    if (inverse) bdda::warp_fft_lines<true, 1, double2, true>(s.data(), 0, tw.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1, double2, true>(s.data(), 0, tw.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const double2 v = s[bdda::skw(i, sh)];
      data[2 * i] = v.x; data[2 * i + 1] = v.y;
    }
  } else if (prec == 3) {  // the double-float MVP's arithmetic (dfz)
    const int sh = bdda::plan_sk<bdda::dfzc>(p);
    std::vector<bdda::dfzc> s(bdda::plan_lw<bdda::dfzc>(p), bdda::cmake(bdda::dfz(1e30), bdda::dfz(1e30))), t(N);
    for (int i = 0; i < N; ++i) {
      s[bdda::skw(i, sh)] = bdda::cmake(bdda::dfz(data[2 * i]), bdda::dfz(data[2 * i + 1]));
      t[i] = bdda::cmake(bdda::dfz(tw[i].x), bdda::dfz(tw[i].y));
    }
    if (inverse) bdda::warp_fft_lines<true, 1, bdda::dfzc, true>(s.data(), 0, t.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1, bdda::dfzc, true>(s.data(), 0, t.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const bdda::dfzc v = s[bdda::skw(i, sh)];
      data[2 * i] = (double)v.x.hi + (double)v.x.lo; data[2 * i + 1] = (double)v.y.hi + (double)v.y.lo;
    }
  } else {
    const int sh = bdda::plan_sk<float2>(p);
    std::vector<float2> s(bdda::plan_lw<float2>(p), make_float2(1e30f, 1e30f)), t(N);
    for (int i = 0; i < N; ++i) {
      s[bdda::skw(i, sh)] = make_float2((float)data[2 * i], (float)data[2 * i + 1]);
      t[i] = make_float2((float)tw[i].x, (float)tw[i].y);
    }
    if (inverse) bdda::warp_fft_lines<true, 1, float2, true>(s.data(), 0, t.data(), p, 0, 1);
    else bdda::warp_fft_lines<false, 1, float2, true>(s.data(), 0, t.data(), p, 0, 1, nv);
    for (int i = 0; i < N; ++i) {
      const float2 v = s[bdda::skw(i, sh)];
      data[2 * i] = v.x; data[2 * i + 1] = v.y;
    }
  }
  if (radix)
    for (int i = 0; i < p.nst; ++i) radix[i] = p.radix[i];
  return p.nst;
}

}  // extern "C"
