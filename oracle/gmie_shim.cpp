// C shim over the reference's own Mie code (gmie/gmie_coeff.cpp, gmie/gmie.cpp),
// compiled from the reference sources where they lie by oracle/Makefile.
// Test infrastructure only: it produces golden Mie coefficients and sphere
// efficiencies for tests/golden; nothing in the product links it.
#include <complex>
#include <tuple>
#include <vector>

std::tuple<std::vector<std::complex<double>>, std::vector<std::complex<double>>,
           std::vector<std::complex<double>>, std::vector<std::complex<double>>>
gmie_coeff(const double& wl_0, const double& r_p, const std::complex<double>& eper_p,
           const std::complex<double>& mper_p, const std::complex<double>& eper_m,
           const std::complex<double>& mper_m);

std::tuple<double, double, double, std::vector<std::complex<double>>, std::vector<std::complex<double>>>
gmie(const double& wl_0, const double& r_p, const int& nang, const std::complex<double>& eper_p,
     const std::complex<double>& mper_p, const std::complex<double>& eper_m,
     const std::complex<double>& mper_m);

extern "C" {

// a1, b1 (first partial-wave coefficients) as {re, im} pairs.
int ref_gmie_a1b1(double wl0, double rp, double ep_re, double ep_im, double mp_re, double mp_im,
                  double em_re, double em_im, double mm_re, double mm_im, double* a1, double* b1) {
  std::vector<std::complex<double>> a, b, c, d;
  std::tie(a, b, c, d) = gmie_coeff(wl0, rp, {ep_re, ep_im}, {mp_re, mp_im}, {em_re, em_im}, {mm_re, mm_im});
  if (a.empty()) return 1;
  a1[0] = a[0].real(); a1[1] = a[0].imag();
  b1[0] = b[0].real(); b1[1] = b[0].imag();
  return 0;
}

// Qsca, Qabs, Qext of a sphere.
int ref_gmie_q(double wl0, double rp, double ep_re, double ep_im, double mp_re, double mp_im,
               double em_re, double em_im, double mm_re, double mm_im, double* q3) {
  double qs, qa, qe;
  std::vector<std::complex<double>> s1, s2;
  int nang = 3;
  std::tie(qs, qa, qe, s1, s2) = gmie(wl0, rp, nang, {ep_re, ep_im}, {mp_re, mp_im}, {em_re, em_im}, {mm_re, mm_im});
  q3[0] = qs; q3[1] = qa; q3[2] = qe;
  return 0;
}

}
