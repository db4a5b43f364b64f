// Target ingestion on the host: target files, shape targets, material tables
// and per-dipole polarizabilities with a cache.
//
// Restates Target_manager::add_to_target_queue (Target_manager.cpp:84-202),
// Material (Material.cpp:10-124), Target::vol_eq_radius_element
// (Target.cpp:13-19), Target_manager::set_polarizability
// (Target_manager.cpp:215-260) and the DIAG_A assembly of
// Solver::prepare_DDA_matrix (Solver.cpp:28-56).  Differences: errors return
// codes instead of exit(); blank and '#' lines are skipped; the Mie
// coefficients are computed once per distinct (element volume, material)
// instead of once per dipole.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/bdda.h"

namespace bdda {
void set_error(const std::string& msg);
}

using cd = std::complex<double>;

struct bdda_material {
  bool constant = true;
  cd eper{1.0, 0.0}, mper{1.0, 0.0};  // constant materials
  std::vector<double> wl0;            // table materials, ascending
  std::vector<cd> eper_t, mper_t;
  double density = 0.0;
};

namespace {

bool blank_or_comment(const std::string& line) {
  size_t i = line.find_first_not_of(" \t\r\n");
  return i == std::string::npos || line[i] == '#';
}

// "re", "(re)" or "(re,im)" (the forms std::complex extraction accepts).
bool parse_complex(std::istringstream& iss, cd* out) {
  std::string tok;
  if (!(iss >> tok)) return false;
  try {
    if (tok.front() != '(') {
      *out = cd(std::stod(tok), 0.0);
      return true;
    }
    if (tok.back() != ')') return false;
    const std::string body = tok.substr(1, tok.size() - 2);
    const size_t comma = body.find(',');
    if (comma == std::string::npos) {
      *out = cd(std::stod(body), 0.0);
    } else {
      *out = cd(std::stod(body.substr(0, comma)), std::stod(body.substr(comma + 1)));
    }
    return true;
  } catch (...) {
    return false;
  }
}

// Target_manager::is_in_target_volume (Target_manager.cpp:8-82).
bool in_shape(int shape, double x, double y, double z, const double* s) {
  switch (shape) {
    case BDDA_SHAPE_SPHERE: {
      const double r = s[0] / 2.0;
      return std::sqrt((x - r) * (x - r) + (y - r) * (y - r) + (z - r) * (z - r)) <= r;
    }
    case BDDA_SHAPE_CUBE:
    case BDDA_SHAPE_CUBOID:
      return x <= s[0] && y <= s[1] && z <= s[2];
    case BDDA_SHAPE_ELLIPSOID: {
      const double a = s[0] / 2.0, b = s[1] / 2.0, c = s[2] / 2.0;
      return (x - a) * (x - a) / (a * a) + (y - b) * (y - b) / (b * b) + (z - c) * (z - c) / (c * c) <= 1.0;
    }
    case BDDA_SHAPE_CYLINDER: {
      const double r = s[0] / 2.0, l = s[2];
      return std::sqrt((x - r) * (x - r) + (y - r) * (y - r)) <= r && z <= l;
    }
    default: {  // BDDA_SHAPE_ROUNDED_CYLINDER
      const double r = s[0] / 2.0;
      // Target_manager.cpp:58-74: below the lower cap centre a sphere test;
      // above it the reference's second test (r < z || z < l - r) is always
      // true, so the rest is a plain cylinder (the upper cap is never rounded).
      if (z <= r) return std::sqrt((x - r) * (x - r) + (y - r) * (y - r) + (z - r) * (z - r)) <= r;
      return std::sqrt((x - r) * (x - r) + (y - r) * (y - r)) <= r;
    }
  }
}

}  // namespace

extern "C" {

int bdda_read_target_file(const char* path, double scale_factor, int n[3], double* lf, int* nocc, int capacity,
                          int* address, double* vol, int* material) {
  if (!path || !n || !lf || !nocc || capacity < 0) {
    bdda::set_error("bad target-file arguments");
    return BDDA_ERR_INVALID;
  }
  std::ifstream in(path);
  if (!in) {
    bdda::set_error(std::string("cannot open target file ") + path);
    return BDDA_ERR_INVALID;
  }
  std::vector<std::string> head;
  std::string line;
  while (head.size() < 5 && std::getline(in, line))
    if (!blank_or_comment(line)) head.push_back(line);
  if (head.size() < 5) {
    bdda::set_error(std::string("truncated header in ") + path);
    return BDDA_ERR_INVALID;
  }
  try {
    (void)std::stod(head[0]);  // pp radius, aggregate volume, coating volume (not used)
    (void)std::stod(head[1]);
    (void)std::stod(head[2]);
    std::istringstream nn(head[3]);
    if (!(nn >> n[0] >> n[1] >> n[2]) || n[0] < 1 || n[1] < 1 || n[2] < 1) throw std::invalid_argument("n");
    *lf = std::stod(head[4]) * scale_factor;
  } catch (...) {
    bdda::set_error(std::string("wrong header format in ") + path);
    return BDDA_ERR_INVALID;
  }
  const double s3 = scale_factor * scale_factor * scale_factor;
  const long long nc = (long long)n[0] * n[1] * n[2];
  int count = 0;
  while (std::getline(in, line)) {
    if (blank_or_comment(line)) continue;
    std::istringstream iss(line);
    long long a;
    double v;
    int mat;
    if (!(iss >> a >> v >> mat)) {
      bdda::set_error(std::string("wrong data format in ") + path + ": " + line);
      return BDDA_ERR_INVALID;
    }
    if (a < 0 || a >= nc) {
      bdda::set_error("lattice address outside the box in " + std::string(path));
      return BDDA_ERR_INVALID;
    }
    if (mat != 0 && mat != 1) {
      bdda::set_error("unknown material index " + std::to_string(mat) + " in " + path);
      return BDDA_ERR_INVALID;
    }
    if (count < capacity) {
      if (address) address[count] = (int)a;
      if (vol) vol[count] = v * s3;
      if (material) material[count] = mat;
    }
    ++count;
  }
  *nocc = count;
  if (count > capacity && capacity > 0) {
    bdda::set_error("target file has " + std::to_string(count) + " rows, capacity " + std::to_string(capacity));
    return BDDA_ERR_INVALID;
  }
  return BDDA_OK;
}

int bdda_shape_target(int shape, int nmax, const double side_lengths[3], int n[3], double* lf, int* nocc, int capacity,
                      int* address) {
  if (!side_lengths || !n || !lf || !nocc || nmax < 1 || capacity < 0 || shape < BDDA_SHAPE_SPHERE ||
      shape > BDDA_SHAPE_ROUNDED_CYLINDER) {
    bdda::set_error("bad shape-target arguments");
    return BDDA_ERR_INVALID;
  }
  double mx = side_lengths[0];
  for (int i = 0; i < 3; ++i) {
    if (!(side_lengths[i] > 0.0)) {
      bdda::set_error("side lengths must be positive");
      return BDDA_ERR_INVALID;
    }
    mx = std::max(mx, side_lengths[i]);
  }
  *lf = mx / nmax;
  for (int i = 0; i < 3; ++i) n[i] = (int)std::ceil(nmax * (side_lengths[i] / mx));
  int count = 0;
  for (int ix = 0; ix < n[0]; ++ix)
    for (int iy = 0; iy < n[1]; ++iy)
      for (int iz = 0; iz < n[2]; ++iz)
        if (in_shape(shape, *lf * ix, *lf * iy, *lf * iz, side_lengths)) {
          if (address && count < capacity) address[count] = n[1] * n[2] * ix + n[2] * iy + iz;
          ++count;
        }
  *nocc = count;
  if (count > capacity && capacity > 0) {
    bdda::set_error("shape target has " + std::to_string(count) + " sites, capacity " + std::to_string(capacity));
    return BDDA_ERR_INVALID;
  }
  return BDDA_OK;
}

int bdda_material_load(const char* path, double density, bdda_material** out) {
  if (!path || !out) {
    bdda::set_error("bad material arguments");
    return BDDA_ERR_INVALID;
  }
  *out = nullptr;
  std::ifstream in(path);
  if (!in) {
    bdda::set_error(std::string("cannot open material file ") + path);
    return BDDA_ERR_INVALID;
  }
  std::unique_ptr<bdda_material> m(new bdda_material());
  m->constant = false;
  m->density = density;
  std::string line;
  while (std::getline(in, line)) {
    if (blank_or_comment(line)) continue;
    std::istringstream iss(line);
    double w;
    cd e, u;
    if (!(iss >> w) || !parse_complex(iss, &e) || !parse_complex(iss, &u)) {
      bdda::set_error(std::string("wrong data format in ") + path + ": " + line);
      return BDDA_ERR_INVALID;
    }
    if (!m->wl0.empty() && !(w > m->wl0.back())) {
      bdda::set_error(std::string("wavelengths not ascending in ") + path);
      return BDDA_ERR_INVALID;
    }
    m->wl0.push_back(w);
    m->eper_t.push_back(e);
    m->mper_t.push_back(u);
  }
  if (m->wl0.empty()) {
    bdda::set_error(std::string("no material data in ") + path);
    return BDDA_ERR_INVALID;
  }
  *out = m.release();
  return BDDA_OK;
}

int bdda_material_constant(const double eper[2], const double mper[2], double density, bdda_material** out) {
  if (!eper || !mper || !out) {
    bdda::set_error("bad material arguments");
    return BDDA_ERR_INVALID;
  }
  bdda_material* m = new bdda_material();
  m->eper = cd(eper[0], eper[1]);
  m->mper = cd(mper[0], mper[1]);
  m->density = density;
  *out = m;
  return BDDA_OK;
}

int bdda_material_eval(const bdda_material* m, double wl0, double eper[2], double mper[2], double* density) {
  if (!m) {
    bdda::set_error("null material");
    return BDDA_ERR_INVALID;
  }
  if (density) *density = m->density;
  if (!eper && !mper) return BDDA_OK;  // density only
  cd e = m->eper, u = m->mper;
  if (!m->constant) {
    const std::vector<double>& w = m->wl0;
    if (!(wl0 >= w.front() && wl0 <= w.back())) {
      bdda::set_error("wavelength outside the material table");
      return BDDA_ERR_INVALID;
    }
    size_t i = 0;
    while (i + 1 < w.size() && !(w[i] <= wl0 && wl0 <= w[i + 1])) ++i;
    if (i + 1 < w.size()) {
      // Material.cpp:97-102, same operation order
      e = m->eper_t[i] + (m->eper_t[i + 1] - m->eper_t[i]) / (w[i + 1] - w[i]) * (wl0 - w[i]);
      u = m->mper_t[i] + (m->mper_t[i + 1] - m->mper_t[i]) / (w[i + 1] - w[i]) * (wl0 - w[i]);
    } else {  // single-row table at exactly its wavelength
      e = m->eper_t[0];
      u = m->mper_t[0];
    }
  }
  if (eper) { eper[0] = e.real(); eper[1] = e.imag(); }
  if (mper) { mper[0] = u.real(); mper[1] = u.imag(); }
  return BDDA_OK;
}

int bdda_material_destroy(bdda_material* m) {
  delete m;
  return BDDA_OK;
}

int bdda_polarizabilities(double wl0, int nocc, const double* vol, const int* material,
                          const bdda_material* const* mats, int nmat, double* alpha_e, double* alpha_h,
                          int* mie_evaluations) {
  if (!(wl0 > 0.0) || nocc < 1 || !vol || !mats || nmat < 1 || !alpha_e) {
    bdda::set_error("bad polarizability arguments");
    return BDDA_ERR_INVALID;
  }
  const double k = 2.0 * M_PI / wl0;  // vacuum medium
  const double k3 = k * k * k;
  std::vector<cd> eper(nmat), mper(nmat);
  for (int j = 0; j < nmat; ++j) {
    double e[2], u[2];
    const int rc = bdda_material_eval(mats[j], wl0, e, u, nullptr);
    if (rc != BDDA_OK) return rc;
    eper[j] = cd(e[0], e[1]);
    mper[j] = cd(u[0], u[1]);
  }
  std::map<std::pair<double, int>, std::pair<cd, cd>> cache;  // (element volume, material) -> (alpha_E, alpha_H)
  const double one[2] = {1.0, 0.0};
  for (int i = 0; i < nocc; ++i) {
    const int mi = material ? material[i] : 0;
    if (mi < 0 || mi >= nmat) {
      bdda::set_error("material index outside the material list");
      return BDDA_ERR_INVALID;
    }
    auto key = std::make_pair(vol[i], mi);
    auto it = cache.find(key);
    if (it == cache.end()) {
      const double rp = std::cbrt(vol[i] * 3.0 / (4.0 * M_PI));  // Target.cpp:15
      const double ep[2] = {eper[mi].real(), eper[mi].imag()}, mp[2] = {mper[mi].real(), mper[mi].imag()};
      double a1[2], b1[2];
      const int rc = bdda_mie_a1b1(wl0, rp, ep, mp, one, one, a1, b1);
      if (rc != BDDA_OK) return rc;
      const cd i3(0.0, 3.0);
      it = cache.emplace(key, std::make_pair(i3 * cd(a1[0], a1[1]) / (2.0 * k3), i3 * cd(b1[0], b1[1]) / (2.0 * k3)))
               .first;
    }
    alpha_e[2 * i] = it->second.first.real();
    alpha_e[2 * i + 1] = it->second.first.imag();
    if (alpha_h) {
      alpha_h[2 * i] = it->second.second.real();
      alpha_h[2 * i + 1] = it->second.second.imag();
    }
  }
  if (mie_evaluations) *mie_evaluations = (int)cache.size();
  return BDDA_OK;
}

int bdda_diag_a(int f, int nocc, const double* alpha_e, const double* alpha_h, double* diag) {
  if ((f != 3 && f != 6) || nocc < 1 || !alpha_e || !diag || (f == 6 && !alpha_h)) {
    bdda::set_error("bad DIAG_A arguments");
    return BDDA_ERR_INVALID;
  }
  for (int m = 0; m < nocc; ++m) {
    const cd de = 1.0 / cd(alpha_e[2 * m], alpha_e[2 * m + 1]);
    const cd dh = f == 6 ? 1.0 / cd(alpha_h[2 * m], alpha_h[2 * m + 1]) : de;
    for (int c = 0; c < f; ++c) {
      const cd v = c < 3 ? de : dh;
      diag[2 * ((size_t)f * m + c)] = v.real();
      diag[2 * ((size_t)f * m + c) + 1] = v.imag();
    }
  }
  return BDDA_OK;
}

}  // extern "C"
