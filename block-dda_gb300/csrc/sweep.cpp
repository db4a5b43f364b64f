// Wavelength x target sweep: the reference's experiment loop
// (block_DDA_main.cpp:138-163: for every wavelength and target, optical
// constants, polarizabilities, incident fields, DDA matrix, solve, cross
// sections) as one library call.
//
// The reference re-creates its Solver (FFT plans, Green spectrum) for every
// (wavelength, target).  Here the loop runs target-major: one operator per
// target whose spectrum alone is rebuilt per wavelength
// (bdda_op_set_wavenumber), and with warm_start each wavelength's refinement
// starts from the target's solution at the previous wavelength.  Results are
// stored [wavelength][target] as the reference's result queue orders them.
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "../../include/bdda.h"

namespace bdda {
void set_error(const std::string& msg);
}

extern "C" int bdda_sweep(const bdda_sweep_spec* s, double* cross, bdda_sweep_result* res) {
  if (!s || !cross || !res || (s->f != 3 && s->f != 6) || s->n_wl < 1 || !s->wl0 || s->n_targets < 1 ||
      !s->targets || s->nmat < 1 || !s->materials || s->L < 1 || s->L > 32 || !s->uinc || !s->einc ||
      (s->f == 6 && !s->hinc)) {
    bdda::set_error("bad sweep specification");
    return BDDA_ERR_INVALID;
  }
  if (s->warm_start && !(s->opts.true_tol > 0)) {
    bdda::set_error("warm_start needs opts.true_tol > 0");
    return BDDA_ERR_INVALID;
  }
  const int f = s->f, L = s->L;
  int first_error = BDDA_OK;
  for (int t = 0; t < s->n_targets; ++t) {
    const bdda_sweep_target& tg = s->targets[t];
    const int nocc = tg.nocc, nrow = f * nocc;
    if (nocc < 1 || !tg.address || !tg.vol) {
      bdda::set_error("bad sweep target");
      return BDDA_ERR_INVALID;
    }
    bdda_op* op = nullptr;
    const double k0 = 2.0 * M_PI / s->wl0[0];
    int rc = bdda_op_create(&op, tg.n, f, tg.lf, k0, 0.0, s->prec ? s->prec : BDDA_PREC_FP64 | BDDA_PREC_FP32 | BDDA_PREC_DF64);
    if (rc == BDDA_OK) rc = bdda_op_set_dipoles(op, tg.address, nocc);
    if (rc != BDDA_OK) {
      bdda_op_destroy(op);
      return rc;
    }
    std::vector<double> ae(2 * nocc), ah(2 * nocc), diag(2 * (size_t)nrow), B(2 * (size_t)nrow * L),
        X(2 * (size_t)nrow * L, 0.0), out(3 * (size_t)L);
    bool have_x = false;
    for (int w = 0; w < s->n_wl; ++w) {
      const double wl0 = s->wl0[w], k = 2.0 * M_PI / wl0;
      bdda_sweep_result& r = res[(size_t)w * s->n_targets + t];
      r = bdda_sweep_result{};
      rc = w == 0 ? BDDA_OK : bdda_op_set_wavenumber(op, k, 0.0);
      int nev = 0;
      if (rc == BDDA_OK)
        rc = bdda_polarizabilities(wl0, nocc, tg.vol, tg.material, s->materials, s->nmat, ae.data(), ah.data(), &nev);
      if (rc == BDDA_OK) rc = bdda_diag_a(f, nocc, ae.data(), ah.data(), diag.data());
      if (rc == BDDA_OK)
        rc = f == 3 ? bdda_incident_fields(tg.n, tg.lf, tg.address, nocc, k, L, s->uinc, s->einc, B.data(), nrow)
                    : bdda_incident_fields_eh(tg.n, tg.lf, tg.address, nocc, k, L, s->uinc, s->einc, s->hinc,
                                              B.data(), nrow);
      bdda_solve_opts o = s->opts;
      o.warm_start = s->warm_start && have_x ? 1 : 0;
      bdda_solve_stats st{};
      if (rc == BDDA_OK) rc = bdda_solve(op, &o, diag.data(), B.data(), nrow, X.data(), nrow, L, &st);
      const bool solved = rc == BDDA_OK || rc == BDDA_ERR_NOT_CONVERGED;
      if (solved) {
        have_x = true;
        const int rc2 = f == 3 ? bdda_cross_sections(k, ae.data(), B.data(), nrow, X.data(), nrow, nrow, L, out.data())
                               : bdda_cross_sections_eh(k, ae.data(), ah.data(), B.data(), nrow, X.data(), nrow,
                                                        nocc, L, out.data());
        if (rc2 != BDDA_OK) rc = rc2;
        for (int i = 0; i < 3 * L; ++i) cross[((size_t)w * s->n_targets + t) * 3 * L + i] = out[i];
      }
      r.status = rc;
      r.iterations = st.iterations;
      r.refinements = st.refinements;
      r.true_res_max = st.true_res_max;
      r.final_err = st.final_err;
      r.ms_solve = st.ms_solve;
      r.mie_evaluations = nev;
      r.alpha_e0[0] = ae[0];
      r.alpha_e0[1] = ae[1];
      r.alpha_h0[0] = f == 6 ? ah[0] : 0.0;
      r.alpha_h0[1] = f == 6 ? ah[1] : 0.0;
      if (rc != BDDA_OK && first_error == BDDA_OK) first_error = rc;
      if (!solved) have_x = false;
    }
    bdda_op_destroy(op);
  }
  return first_error;
}
