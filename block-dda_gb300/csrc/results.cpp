// Result sections in the reference's DDA_result.dat text format.
//
// Restates Result_manager::add_to_result_queue (Result_manager.cpp:10-133:
// particle or core/coat properties, Csca = Cext - Cabs, SSA, MAC),
// Basic_Stats (Basic_Stats.hpp: mean, sample standard deviation from the mean
// of squares), the section writer operator<< (Result_manager.cpp:178-245) and
// the volume-equivalent Mie MAC line the reference's main program appends
// (Result_manager.cpp:137-176, block_DDA_main.cpp:169-183).  Numbers go
// through std::ostream with its default formatting, as the reference's do.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/bdda.h"

namespace bdda {
void set_error(const std::string& msg);
}

namespace {

using cd = std::complex<double>;

struct Stats {
  double mean, std;
};

// Basic_Stats.hpp: var = (mean of squares - mean^2) N / (N - 1)
Stats basic_stats(const std::vector<double>& v) {
  const int N = (int)v.size();
  double sum = 0.0, sq = 0.0;
  for (double x : v) sum += x;
  for (double x : v) sq += x * x;
  const double mean = sum / N;
  const double var = (sq / N - mean * mean) * N * 1.0 / (N - 1.0);
  return {mean, std::sqrt(var)};
}

}  // namespace

extern "C" int bdda_format_result(const bdda_result_record* r, char* buf, int cap, int* len) {
  if (!r || !len || r->L < 1 || !r->cext || !r->cabs || !(r->wl0 > 0) || !(r->volume_core > 0)) {
    bdda::set_error("bad result record");
    return BDDA_ERR_INVALID;
  }
  const double um3_to_cm3 = 1.0e-12, um2_to_m2 = 1.0e-12;
  const cd eper_core(r->eper_core[0], r->eper_core[1]), mper_core(r->mper_core[0], r->mper_core[1]);
  const double mass = r->volume_core * um3_to_cm3 * r->density_core;
  const double ve_radius = std::cbrt(r->volume_core * 3.0 / (4.0 * M_PI));
  std::vector<double> csca(r->L), mac(r->L), ssa(r->L);
  for (int l = 0; l < r->L; ++l) {
    csca[l] = r->cext[l] - r->cabs[l];
    ssa[l] = (r->cext[l] - r->cabs[l]) / r->cext[l];
    mac[l] = r->cabs[l] * um2_to_m2 / mass;
  }
  const Stats s_csca = basic_stats(csca), s_mac = basic_stats(mac), s_ssa = basic_stats(ssa);
  const cd eper_m(r->eper_medium[0], r->eper_medium[1]), mper_m(r->mper_medium[0], r->mper_medium[1]);
  std::ostringstream os;
  os << "####################### Start of result section #######################" << '\n';
  os << "wl0_index" << '\t' << r->wl0_index << '\n';
  os << "target_index" << '\t' << r->target_index << '\n';
  os << '\n';
  os << "----------------- Incident wave properties -------------------" << '\n';
  os << "wl0" << '\t' << r->wl0 << '\n' << "N_inc" << '\t' << r->N_inc << '\n';
  os << '\n';
  os << "-------------------- Medium properties -----------------------" << '\n';
  os << "eper_medium" << '\t' << eper_m << '\n' << "mper_medium" << '\t' << mper_m << '\n';
  os << '\n';
  os << "-------------------- Target properties ----------------------" << '\n';
  os << "target_fname" << '\t' << (r->target_fname ? r->target_fname : "") << '\n';
  os << "is_homogeneous" << '\t' << (r->is_homogeneous ? 1 : 0) << '\n';
  if (r->is_homogeneous) {
    os << "eper_particle" << '\t' << eper_core << '\n'
       << "mper_particle" << '\t' << mper_core << '\n'
       << "volume_particle" << '\t' << r->volume_core << '\n'
       << "mass_particle" << '\t' << mass << '\n'
       << "density_particle" << '\t' << r->density_core << '\n'
       << "ve_radius_particle" << '\t' << ve_radius << '\n';
  } else {
    os << "eper_core" << '\t' << eper_core << '\n'
       << "mper_core" << '\t' << mper_core << '\n'
       << "volume_core" << '\t' << r->volume_core << '\n'
       << "mass_core" << '\t' << mass << '\n'
       << "density_core" << '\t' << r->density_core << '\n'
       << "ve_radius_core" << '\t' << ve_radius << '\n'
       << "eper_coat" << '\t' << cd(r->eper_coat[0], r->eper_coat[1]) << '\n'
       << "mper_coat" << '\t' << cd(r->mper_coat[0], r->mper_coat[1]) << '\n'
       << "volume_coat" << '\t' << r->volume_coat << '\n'
       << "coat_to_core_vratio" << '\t' << r->volume_coat / r->volume_core << '\n';
  }
  os << '\n';
  os << "----------------- Computed optical properties -----------------" << '\n';
  os << "mean_Csca" << '\t' << s_csca.mean << '\n'
     << "std_Csca" << '\t' << s_csca.std << '\n'
     << "mean_MAC" << '\t' << s_mac.mean << '\n'
     << "std_MAC" << '\t' << s_mac.std << '\n'
     << "mean_SSA" << '\t' << s_ssa.mean << '\n'
     << "std_SSA" << '\t' << s_ssa.std << '\n';
  os << '\n';
  os << "------------------- Computational info --------------------" << '\n';
  os << "f" << '\t' << r->f << '\n';
  os << "nx" << '\t' << r->nx << '\n';
  os << "ny" << '\t' << r->ny << '\n';
  os << "nz" << '\t' << r->nz << '\n';
  os << "num_element_cuboid" << '\t' << r->nx * r->ny * r->nz << '\n';
  os << "num_element_occupy" << '\t' << r->num_element_occupy << '\n';
  os << "DDA_solver_time" << '\t' << r->solver_time << '\n'
     << "DDA_solver_time_per_Ninc" << '\t' << r->solver_time / r->N_inc << '\n';
  os << '\n';
  os << "************************ End of result section ***********************" << '\n';
  if (r->append_mac_mie) {
    double q[3];
    const int rc = bdda_mie_q(r->wl0, ve_radius, r->eper_core, r->mper_core, r->eper_medium, r->mper_medium, q);
    if (rc != BDDA_OK) return rc;
    const double cabs_mie = q[1] * M_PI * ve_radius * ve_radius;
    os << "MAC_mie" << '\t' << cabs_mie * um2_to_m2 / mass << '\n' << '\n';
  }
  const std::string out = os.str();
  *len = (int)out.size();
  if (buf && cap > 0) {
    const size_t nc = std::min<size_t>(out.size(), (size_t)cap - 1);
    std::memcpy(buf, out.data(), nc);
    buf[nc] = '\0';
    if (out.size() >= (size_t)cap) {
      bdda::set_error("result buffer too small");
      return BDDA_ERR_INVALID;
    }
  }
  return BDDA_OK;
}
