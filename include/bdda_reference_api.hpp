// bdda_reference_api.hpp -- the reference's C++ entry points over the C ABI.
//
// Drop-in replacements, same names, argument meaning and layouts, for the
// functions nmoteki/block-DDA declares in MBT_utils.hpp:1-6,
// bl_krylov_mvp_fft/DDA_linear_solvers.hpp:1-6 and
// bl_krylov_mvp_fft/linear_algebra_addon.hpp:1, as called from
// Solver.cpp:55,64,71.  Header-only; link with libbdda.so.
//
// Differences a caller sees:
//  * MBT_fft_init returns an operator token (MbtOperator) instead of the
//    Au_til vector; pass it back wherever the reference passes Au_til.
//  * fftw_plan arguments are accepted and ignored (the operator owns its
//    device FFT plans); a stand-in typedef is used when <fftw3.h> is absent.
//  * Errors throw bdda_ref::Error (the reference calls exit()).
//  * Non-convergence is not an error, as in the reference; call
//    bdda_ref::last_stats() for the iteration count and status.
//  * Vectors/matrices are Eigen types when <Eigen/Dense> is available, else
//    the minimal column-major stand-ins below with the same member names used
//    by the reference (size, rows, cols, data, operator()).
#pragma once

#include <complex>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "bdda.h"

#if __has_include(<fftw3.h>)
#include <fftw3.h>
#else
typedef struct bdda_fftw_plan_stub* fftw_plan;
#endif

#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
namespace bdda_ref {
using VectorXi = Eigen::VectorXi;
using VectorXcd = Eigen::VectorXcd;
using MatrixXcd = Eigen::MatrixXcd;
}  // namespace bdda_ref
#else
namespace bdda_ref {
// Column-major stand-ins (Eigen's default storage order).
struct VectorXi {
  std::vector<int> v;
  VectorXi() = default;
  explicit VectorXi(int n) : v(n) {}
  VectorXi(std::initializer_list<int> l) : v(l) {}
  int size() const { return (int)v.size(); }
  int& operator()(int i) { return v[i]; }
  int operator()(int i) const { return v[i]; }
  const int* data() const { return v.data(); }
  long long prod() const { long long p = 1; for (int x : v) p *= x; return p; }
};
struct VectorXcd {
  std::vector<std::complex<double>> v;
  VectorXcd() = default;
  explicit VectorXcd(int n) : v(n) {}
  int size() const { return (int)v.size(); }
  std::complex<double>& operator()(int i) { return v[i]; }
  const std::complex<double>& operator()(int i) const { return v[i]; }
  std::complex<double>* data() { return v.data(); }
  const std::complex<double>* data() const { return v.data(); }
};
struct MatrixXcd {
  int r = 0, c = 0;
  std::vector<std::complex<double>> v;
  MatrixXcd() = default;
  MatrixXcd(int rows, int cols) : r(rows), c(cols), v((size_t)rows * cols) {}
  int rows() const { return r; }
  int cols() const { return c; }
  std::complex<double>& operator()(int i, int j) { return v[(size_t)j * r + i]; }
  const std::complex<double>& operator()(int i, int j) const { return v[(size_t)j * r + i]; }
  std::complex<double>* data() { return v.data(); }
  const std::complex<double>* data() const { return v.data(); }
};
}  // namespace bdda_ref
#endif

namespace bdda_ref {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != BDDA_OK && rc != BDDA_ERR_NOT_CONVERGED) throw Error(rc, bdda_last_error());
}

// What MBT_fft_init returns: the device operator of one box and wavenumber.
struct MbtOperator {
  std::shared_ptr<bdda_op> op;
  std::vector<int> dipoles;  // address list currently set on the operator
};

inline bdda_solve_stats& last_stats() {
  thread_local bdda_solve_stats s{};
  return s;
}

// MBT_fft_init (mvp_fft/MBT_fft_init.cpp:10-42): build the Green spectrum.
inline MbtOperator MBT_fft_init(const VectorXi& n, const int& f, const double& lf, const std::complex<double>& k,
                                fftw_plan& /*plan_fwd*/) {
  if (n.size() != 3) throw Error(BDDA_ERR_INVALID, "n must hold 3 box sizes");
  const int nn[3] = {n(0), n(1), n(2)};
  bdda_op* raw = nullptr;
  check(bdda_op_create(&raw, nn, f, lf, k.real(), k.imag(), BDDA_PREC_FP64 | BDDA_PREC_FP32));
  MbtOperator m;
  m.op = std::shared_ptr<bdda_op>(raw, [](bdda_op* p) { bdda_op_destroy(p); });
  return m;
}

// MBT_fft_mvp (mvp_fft/MBT_fft_mvp.cpp:8-43): off-diagonal product on the
// cuboid vector of length f * nx * ny * nz.  Safe to call from several host
// threads on one operator (the reference's OpenMP loop).
inline VectorXcd MBT_fft_mvp(const VectorXi& /*n*/, const int& /*f*/, const MbtOperator& Au_til, const VectorXcd& p_hat,
                             fftw_plan& /*plan_fwd*/, fftw_plan& /*plan_inv*/) {
  VectorXcd q(p_hat.size());
  check(bdda_mbt_fft_mvp(Au_til.op.get(), reinterpret_cast<const double*>(p_hat.data()),
                         reinterpret_cast<double*>(q.data())));
  return q;
}

namespace detail {
inline MatrixXcd solve(int solver, bool jacobi, const std::vector<int>& address, const MbtOperator& Au_til,
                       const VectorXcd& DIAG_A, const MatrixXcd& B, double tol, int itermax) {
  MbtOperator& m = const_cast<MbtOperator&>(Au_til);
  if (m.dipoles != address) {
    check(bdda_op_set_dipoles(m.op.get(), address.data(), (int)address.size()));
    m.dipoles = address;
  }
  bdda_solve_opts o;
  bdda_solve_opts_default(&o);
  o.solver = solver;
  o.jacobi = jacobi ? 1 : 0;
  o.precision = BDDA_SOLVE_FP64;
  o.tol = tol;
  o.itermax = itermax;
  MatrixXcd X(B.rows(), B.cols());
  check(bdda_solve(m.op.get(), &o, reinterpret_cast<const double*>(DIAG_A.data()),
                   reinterpret_cast<const double*>(B.data()), (int)B.rows(), reinterpret_cast<double*>(X.data()),
                   (int)X.rows(), (int)B.cols(), &last_stats()));
  return X;
}
}  // namespace detail

#define BDDA_REF_SOLVER(NAME, ID, JAC)                                                                              \
  inline MatrixXcd NAME(const VectorXi& /*n*/, const int& /*f*/, const std::vector<int>& address,                  \
                        const MbtOperator& Au_til, const VectorXcd& DIAG_A, const MatrixXcd& B, const double& tol,  \
                        const int& itermax, fftw_plan& /*plan_fwd*/, fftw_plan& /*plan_inv*/) {                    \
    return detail::solve(ID, JAC, address, Au_til, DIAG_A, B, tol, itermax);                                       \
  }

// bl_krylov_mvp_fft/DDA_linear_solvers.hpp:1-6
BDDA_REF_SOLVER(bl_cocg_rq_mvp_fft, BDDA_SOLVER_COCG_RQ, false)
BDDA_REF_SOLVER(bl_cocg_rq_jacobi_mvp_fft, BDDA_SOLVER_COCG_RQ, true)
BDDA_REF_SOLVER(bl_bicgstab_mvp_fft, BDDA_SOLVER_BICGSTAB, false)
BDDA_REF_SOLVER(bl_bicgstab_jacobi_mvp_fft, BDDA_SOLVER_BICGSTAB, true)
BDDA_REF_SOLVER(bl_bicggr_mvp_fft, BDDA_SOLVER_BICGGR, false)
BDDA_REF_SOLVER(bl_bicggr_jacobi_mvp_fft, BDDA_SOLVER_BICGGR, true)
#undef BDDA_REF_SOLVER

// qr_reduced (bl_krylov_mvp_fft/qr_reduced.cpp:9-31)
inline std::tuple<MatrixXcd, MatrixXcd> qr_reduced(const MatrixXcd& A) {
  MatrixXcd Q(A.rows(), A.cols()), R(A.cols(), A.cols());
  check(bdda_qr_reduced(reinterpret_cast<const double*>(A.data()), (int)A.rows(), (int)A.cols(), (int)A.rows(),
                        reinterpret_cast<double*>(Q.data()), (int)Q.rows(), reinterpret_cast<double*>(R.data())));
  return std::make_tuple(Q, R);
}

}  // namespace bdda_ref
