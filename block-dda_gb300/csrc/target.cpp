// Host-side target model: polarizability, aggregates, incident fields, cross sections.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/bdda.h"

namespace bdda {
void set_error(const std::string& msg);
}

namespace {

using cd = std::complex<double>;

// Mie coefficients a1, b1 of a sphere (Bohren & Huffman 1983, eqs. 4.53, 4.88 with
// mu/mu_m factors for magnetic spheres, Kerker et al. 1983).  Logarithmic derivative
// D_n(y) by downward recurrence from a start index well above |y|; psi_n(x) and
// xi_n(x) by the (stable for the orders used here) upward recurrence.  Polarizability
// needs only n = 1, so 16 + |y| terms are plenty for the start of the recurrence.
void mie_a1b1(double wl0, double rp, cd eps_p, cd mu_p, cd eps_m, cd mu_m, cd* a1, cd* b1) {
  const double k0 = 2.0 * M_PI / wl0;
  const cd m_m = std::sqrt(eps_m * mu_m);
  const cd m_p = std::sqrt(eps_p * mu_p);
  const cd x = m_m * k0 * rp;        // size parameter in the medium
  const cd mr = m_p / m_m;           // relative refractive index
  const cd y = mr * x;
  // D_1(y): D_{n-1} = n/y - 1/(D_n + n/y)
  const int nstart = 16 + (int)std::ceil(std::abs(y)) + (int)std::ceil(4.0 * std::cbrt(std::abs(y)));
  cd D(0.0, 0.0);
  for (int nn = nstart; nn > 1; --nn) D = (double)nn / y - 1.0 / (D + (double)nn / y);
  const cd D1 = D;  // D_1
  // Riccati-Bessel psi_n(x) = x j_n(x), chi_n(x) = x y_n(x) (y_n spherical Neumann),
  // xi_n = psi_n + i chi_n (outgoing);  n = 0, 1
  // psi_1 = r_1 psi_0 with r_n = psi_n / psi_{n-1} from the continued fraction
  // r_n = 1 / ((2n+1)/x - r_{n+1}) (no cancellation for small x)
  cd r(0.0, 0.0);
  for (int nn = nstart; nn >= 1; --nn) r = 1.0 / ((2.0 * nn + 1.0) / x - r);
  const cd psi0 = std::sin(x), psi1 = r * psi0;
  const cd chi0 = -std::cos(x), chi1 = -std::cos(x) / x - std::sin(x);
  const cd xi0 = psi0 + cd(0, 1) * chi0, xi1 = psi1 + cd(0, 1) * chi1;
  const cd fa = (mu_p / (mu_m * mr)) * D1 + 1.0 / x;
  const cd fb = (mu_m * mr / mu_p) * D1 + 1.0 / x;
  *a1 = (fa * psi1 - psi0) / (fa * xi1 - xi0);
  *b1 = (fb * psi1 - psi0) / (fb * xi1 - xi0);
}

// Efficiencies of a sphere in a non-absorbing medium (Bohren & Huffman 1983,
// eqs. 4.61-4.62): Qsca = 2/x^2 sum (2n+1)(|a_n|^2 + |b_n|^2), Qext = 2/x^2
// sum (2n+1) Re(a_n + b_n), n <= x + 4 x^(1/3) + 2 (Wiscombe 1980).  a_n, b_n
// as for n = 1 above; psi_n from the ratios psi_n / psi_{n-1} (downward
// continued fraction, stable for every n), chi_n upward (its stable direction).
bool mie_q(double wl0, double rp, cd eps_p, cd mu_p, cd eps_m, cd mu_m, double* qsca, double* qabs, double* qext) {
  const double k0 = 2.0 * M_PI / wl0;
  const cd m_m = std::sqrt(eps_m * mu_m);
  if (std::abs(m_m.imag()) > 0.0) return false;
  const cd m_p = std::sqrt(eps_p * mu_p);
  const double x = m_m.real() * k0 * rp;
  const cd mr = m_p / m_m;
  const cd y = mr * x;
  const int nstop = (int)(x + 4.0 * std::cbrt(x) + 2.0);
  const int nmx = std::max(nstop, (int)std::ceil(std::abs(y))) + 16;
  std::vector<cd> D(nmx + 1), r(nmx + 2);
  D[nmx] = cd(0.0, 0.0);
  for (int n = nmx; n > 0; --n) D[n - 1] = (double)n / y - 1.0 / (D[n] + (double)n / y);
  r[nmx + 1] = cd(0.0, 0.0);
  for (int n = nmx; n >= 1; --n) r[n] = 1.0 / ((2.0 * n + 1.0) / x - r[n + 1]);
  double psi_m1 = std::sin(x), chi_m1 = -std::cos(x);  // n = 0
  double psi = (r[1] * psi_m1).real(), chi = -std::cos(x) / x - std::sin(x);  // n = 1
  double ssca = 0.0, sext = 0.0;
  for (int n = 1; n <= nstop; ++n) {
    const cd xi(psi, chi), xi_m1(psi_m1, chi_m1);
    const cd fa = (mu_p / (mu_m * mr)) * D[n] + (double)n / x;
    const cd fb = (mu_m * mr / mu_p) * D[n] + (double)n / x;
    const cd an = (fa * psi - psi_m1) / (fa * xi - xi_m1);
    const cd bn = (fb * psi - psi_m1) / (fb * xi - xi_m1);
    ssca += (2.0 * n + 1.0) * (std::norm(an) + std::norm(bn));
    sext += (2.0 * n + 1.0) * (an + bn).real();
    const double psi_n1 = (r[n + 1] * psi).real();
    const double chi_n1 = (2.0 * n + 1.0) / x * chi - chi_m1;
    psi_m1 = psi; psi = psi_n1;
    chi_m1 = chi; chi = chi_n1;
  }
  *qsca = 2.0 / (x * x) * ssca;
  *qext = 2.0 / (x * x) * sext;
  *qabs = *qext - *qsca;
  return true;
}

// splitmix64 + uniform double in [0,1)
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ULL + 0x2545F4914F6CDD1DULL) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Key {
  static uint64_t pack(int x, int y, int z) {
    return ((uint64_t)(uint32_t)(x + (1 << 20)) << 42) | ((uint64_t)(uint32_t)(y + (1 << 20)) << 21) |
           (uint64_t)(uint32_t)(z + (1 << 20));
  }
};

}  // namespace

extern "C" {

int bdda_mie_a1b1(double wl0, double r_p, const double eps_p[2], const double mu_p[2], const double eps_m[2],
                  const double mu_m[2], double a1[2], double b1[2]) {
  if (!(wl0 > 0) || !(r_p > 0) || !eps_p || !mu_p || !eps_m || !mu_m || !a1 || !b1) {
    bdda::set_error("bad Mie arguments");
    return BDDA_ERR_INVALID;
  }
  cd a, b;
  mie_a1b1(wl0, r_p, cd(eps_p[0], eps_p[1]), cd(mu_p[0], mu_p[1]), cd(eps_m[0], eps_m[1]), cd(mu_m[0], mu_m[1]), &a, &b);
  a1[0] = a.real(); a1[1] = a.imag();
  b1[0] = b.real(); b1[1] = b.imag();
  return BDDA_OK;
}

int bdda_mie_q(double wl0, double r_p, const double eps_p[2], const double mu_p[2], const double eps_m[2],
               const double mu_m[2], double q[3]) {
  if (!(wl0 > 0) || !(r_p > 0) || !eps_p || !mu_p || !eps_m || !mu_m || !q) {
    bdda::set_error("bad Mie arguments");
    return BDDA_ERR_INVALID;
  }
  if (!mie_q(wl0, r_p, cd(eps_p[0], eps_p[1]), cd(mu_p[0], mu_p[1]), cd(eps_m[0], eps_m[1]), cd(mu_m[0], mu_m[1]),
             &q[0], &q[1], &q[2])) {
    bdda::set_error("Mie efficiencies need a non-absorbing medium");
    return BDDA_ERR_INVALID;
  }
  return BDDA_OK;
}

// Tunable particle-cluster aggregation on the simple cubic lattice.  Monomers are
// lattice sites (spacing 1 = monomer radius a).  Monomer N+1 is attached to a
// face-adjacent empty site of the cluster whose distance G from the current
// centre of mass best matches the tunable-aggregation rule (Filippov et al.
// 2000): G^2 = (N+1)^2/N Rg(N+1)^2 - (N+1) Rg(N)^2 with Rg(N) = a (N/kf)^(1/Df)
// (point monomers), chosen among a seeded random sample of frontier sites.
int bdda_aggregate(int nocc, double kf, double Df, unsigned long long seed, int n[3], int* address) {
  if (nocc < 1 || !(kf > 0) || !(Df > 0) || !n || !address) {
    bdda::set_error("bad aggregate arguments");
    return BDDA_ERR_INVALID;
  }
  Rng rng(seed);
  std::vector<int> xs, ys, zs;
  xs.reserve(nocc); ys.reserve(nocc); zs.reserve(nocc);
  std::unordered_map<uint64_t, int> occ;      // site -> 1
  std::vector<uint64_t> frontier;             // empty sites adjacent to the cluster
  std::unordered_map<uint64_t, int> fpos;     // frontier site -> index
  occ.reserve((size_t)nocc * 2);
  fpos.reserve((size_t)nocc * 8);
  const int nb[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  double sx = 0, sy = 0, sz = 0, sxx = 0;  // sums for centre of mass and Rg
  auto add_site = [&](int x, int y, int z) {
    const uint64_t k = Key::pack(x, y, z);
    occ[k] = 1;
    auto it = fpos.find(k);
    if (it != fpos.end()) {
      const int i = it->second;
      const uint64_t last = frontier.back();
      frontier[i] = last;
      fpos[last] = i;
      frontier.pop_back();
      fpos.erase(k);
    }
    for (auto& d : nb) {
      const uint64_t q = Key::pack(x + d[0], y + d[1], z + d[2]);
      if (occ.count(q) || fpos.count(q)) continue;
      fpos[q] = (int)frontier.size();
      frontier.push_back(q);
    }
    xs.push_back(x); ys.push_back(y); zs.push_back(z);
    sx += x; sy += y; sz += z;
    sxx += (double)x * x + (double)y * y + (double)z * z;
  };
  auto unpack = [](uint64_t k, int* x, int* y, int* z) {
    *z = (int)(k & ((1u << 21) - 1)) - (1 << 20);
    *y = (int)((k >> 21) & ((1u << 21) - 1)) - (1 << 20);
    *x = (int)((k >> 42) & ((1u << 21) - 1)) - (1 << 20);
  };
  add_site(0, 0, 0);
  auto rg = [&](double N) { return std::pow(N / kf, 1.0 / Df); };
  const int kSample = 48;
  while ((int)xs.size() < nocc) {
    const double N = (double)xs.size();
    const double cx = sx / N, cy = sy / N, cz = sz / N;
    const double g2 = (N + 1) * (N + 1) / N * rg(N + 1) * rg(N + 1) - (N + 1) * rg(N) * rg(N);
    const double g = std::sqrt(std::max(0.0, g2));
    uint64_t best = frontier[0];
    double bestd = 1e300;
    const int m = (int)frontier.size();
    const int tries = std::min(kSample, m);
    for (int t = 0; t < tries; ++t) {
      const uint64_t q = frontier[(size_t)(rng.uniform() * m) % m];
      int x, y, z;
      unpack(q, &x, &y, &z);
      const double d = std::sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
      const double e = std::fabs(d - g);
      if (e < bestd) { bestd = e; best = q; }
    }
    int x, y, z;
    unpack(best, &x, &y, &z);
    add_site(x, y, z);
  }
  int mn[3] = {xs[0], ys[0], zs[0]}, mx[3] = {xs[0], ys[0], zs[0]};
  for (int i = 0; i < nocc; ++i) {
    mn[0] = std::min(mn[0], xs[i]); mx[0] = std::max(mx[0], xs[i]);
    mn[1] = std::min(mn[1], ys[i]); mx[1] = std::max(mx[1], ys[i]);
    mn[2] = std::min(mn[2], zs[i]); mx[2] = std::max(mx[2], zs[i]);
  }
  for (int d = 0; d < 3; ++d) n[d] = mx[d] - mn[d] + 1;
  for (int i = 0; i < nocc; ++i) {
    const long long a = (long long)n[1] * n[2] * (xs[i] - mn[0]) + (long long)n[2] * (ys[i] - mn[1]) + (zs[i] - mn[2]);
    address[i] = (int)a;
  }
  return BDDA_OK;
}

int bdda_incident_fields(const int n[3], double lf, const int* address, int nocc, double k, int L, const double* uinc,
                         const double* einc, double* B, int ldb) {
  if (!n || !address || !uinc || !einc || !B || nocc < 1 || L < 1 || ldb < 3 * nocc) {
    bdda::set_error("bad incident-field arguments");
    return BDDA_ERR_INVALID;
  }
  const long long nyz = (long long)n[1] * n[2];
  for (int l = 0; l < L; ++l) {
    const double* u = uinc + 3 * l;
    const cd e[3] = {cd(einc[6 * l + 0], einc[6 * l + 1]), cd(einc[6 * l + 2], einc[6 * l + 3]),
                     cd(einc[6 * l + 4], einc[6 * l + 5])};
    for (int m = 0; m < nocc; ++m) {
      const long long a = address[m];
      const long long ix = a / nyz, iy = (a - nyz * ix) / n[2], iz = a - nyz * ix - (long long)n[2] * iy;
      const double ph = k * lf * (u[0] * ix + u[1] * iy + u[2] * iz);
      const cd p(std::cos(ph), std::sin(ph));
      for (int c = 0; c < 3; ++c) {
        const cd v = e[c] * p;
        const size_t r = (size_t)l * ldb + 3 * (size_t)m + c;
        B[2 * r] = v.real();
        B[2 * r + 1] = v.imag();
      }
    }
  }
  return BDDA_OK;
}

int bdda_cross_sections(double k, const double alpha0[2], const double* E, int lde, const double* P, int ldp, int nrows, int L,
                        double* out) {
  if (!alpha0 || !E || !P || !out || nrows < 1 || L < 1 || lde < nrows || ldp < nrows) {
    bdda::set_error("bad cross-section arguments");
    return BDDA_ERR_INVALID;
  }
  const cd a0(alpha0[0], alpha0[1]);
  const double absfac = std::imag(std::conj(1.0 / a0)) - 2.0 * k * k * k / 3.0;
  for (int l = 0; l < L; ++l) {
    cd dot(0, 0);
    double p2 = 0.0;
    for (int r = 0; r < nrows; ++r) {
      const cd e(E[2 * ((size_t)l * lde + r)], E[2 * ((size_t)l * lde + r) + 1]);
      const cd p(P[2 * ((size_t)l * ldp + r)], P[2 * ((size_t)l * ldp + r) + 1]);
      dot += std::conj(e) * p;
      p2 += std::norm(p);
    }
    const double cext = 4.0 * M_PI * k * dot.imag();
    const double cabs = 4.0 * M_PI * k * absfac * p2;
    out[3 * l + 0] = cext;
    out[3 * l + 1] = cabs;
    out[3 * l + 2] = cext - cabs;
  }
  return BDDA_OK;
}

int bdda_incident_fields_eh(const int n[3], double lf, const int* address, int nocc, double k, int L,
                            const double* uinc, const double* einc, const double* hinc, double* B, int ldb) {
  if (!n || !address || !uinc || !einc || !hinc || !B || nocc < 1 || L < 1 || ldb < 6 * nocc) {
    bdda::set_error("bad incident-field arguments");
    return BDDA_ERR_INVALID;
  }
  const long long nyz = (long long)n[1] * n[2];
  for (int l = 0; l < L; ++l) {
    const double* u = uinc + 3 * l;
    cd eh[6];
    for (int c = 0; c < 3; ++c) {
      eh[c] = cd(einc[6 * l + 2 * c], einc[6 * l + 2 * c + 1]);
      eh[3 + c] = cd(hinc[6 * l + 2 * c], hinc[6 * l + 2 * c + 1]);
    }
    for (int m = 0; m < nocc; ++m) {
      const long long a = address[m];
      const long long ix = a / nyz, iy = (a - nyz * ix) / n[2], iz = a - nyz * ix - (long long)n[2] * iy;
      const double ph = k * lf * (u[0] * ix + u[1] * iy + u[2] * iz);
      const cd p(std::cos(ph), std::sin(ph));
      for (int c = 0; c < 6; ++c) {
        const cd v = eh[c] * p;
        const size_t r = (size_t)l * ldb + 6 * (size_t)m + c;
        B[2 * r] = v.real();
        B[2 * r + 1] = v.imag();
      }
    }
  }
  return BDDA_OK;
}

int bdda_cross_sections_eh(double k, const double alpha_e0[2], const double alpha_h0[2], const double* EH, int lde,
                           const double* PM, int ldp, int nocc, int L, double* out) {
  if (!alpha_e0 || !alpha_h0 || !EH || !PM || !out || nocc < 1 || L < 1 || lde < 6 * nocc || ldp < 6 * nocc) {
    bdda::set_error("bad cross-section arguments");
    return BDDA_ERR_INVALID;
  }
  const double we = std::imag(std::conj(1.0 / cd(alpha_e0[0], alpha_e0[1]))) - 2.0 * k * k * k / 3.0;
  const double wh = std::imag(std::conj(1.0 / cd(alpha_h0[0], alpha_h0[1]))) - 2.0 * k * k * k / 3.0;
  for (int l = 0; l < L; ++l) {
    cd dot(0, 0);
    double pe = 0.0, pm = 0.0;
    for (int r = 0; r < 6 * nocc; ++r) {
      const cd e(EH[2 * ((size_t)l * lde + r)], EH[2 * ((size_t)l * lde + r) + 1]);
      const cd p(PM[2 * ((size_t)l * ldp + r)], PM[2 * ((size_t)l * ldp + r) + 1]);
      dot += std::conj(e) * p;
      if (r % 6 < 3) pe += std::norm(p);
      else pm += std::norm(p);
    }
    const double cext = 4.0 * M_PI * k * dot.imag();
    const double cabs = 4.0 * M_PI * k * (we * pe + wh * pm);
    out[3 * l + 0] = cext;
    out[3 * l + 1] = cabs;
    out[3 * l + 2] = cext - cabs;
  }
  return BDDA_OK;
}

}  // extern "C"
