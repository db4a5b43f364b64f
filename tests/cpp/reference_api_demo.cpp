// Calls the reference-named C++ entry points (include/bdda_reference_api.hpp)
// the way Solver::prepare_DDA_matrix / DDA_solve do (Solver.cpp:28-83), on
// inputs written by tests/test_gpu_reference_api.py, and writes the results
// back for comparison with the oracle.
//
// input file (little-endian): int nx, ny, nz, nocc, L; double lf, k_re, k_im, tol;
//   int itermax; int address[nocc]; complex diag[3 nocc]; complex B[3 nocc * L]
//   (column-major); complex p_hat[3 nx ny nz]
// output file: complex q_hat[3 nx ny nz]; complex X[3 nocc * L]; complex Q, R of qr_reduced(B);
//   int iterations
#include <cstdio>
#include <fstream>
#include <vector>

#include "bdda_reference_api.hpp"

using namespace bdda_ref;

template <typename T> static void rd(std::ifstream& f, T* p, size_t n) { f.read(reinterpret_cast<char*>(p), sizeof(T) * n); }
template <typename T> static void wr(std::ofstream& f, const T* p, size_t n) { f.write(reinterpret_cast<const char*>(p), sizeof(T) * n); }

int main(int argc, char** argv) {
  if (argc != 3) { std::fprintf(stderr, "usage: %s in out\n", argv[0]); return 2; }
  std::ifstream in(argv[1], std::ios::binary);
  int hdr[5];
  rd(in, hdr, 5);
  double dv[4];
  rd(in, dv, 4);
  int itermax;
  rd(in, &itermax, 1);
  const int nocc = hdr[3], L = hdr[4];
  std::vector<int> address(nocc);
  rd(in, address.data(), nocc);
  VectorXcd diag(3 * nocc);
  rd(in, diag.data(), 3 * nocc);
  MatrixXcd B(3 * nocc, L);
  rd(in, B.data(), (size_t)3 * nocc * L);
  VectorXi n(3);
  n(0) = hdr[0]; n(1) = hdr[1]; n(2) = hdr[2];
  VectorXcd p(3 * hdr[0] * hdr[1] * hdr[2]);
  rd(in, p.data(), p.size());
  fftw_plan plan_fwd{}, plan_inv{};
  try {
    const int f = 3;
    MbtOperator Au_til = MBT_fft_init(n, f, dv[0], std::complex<double>(dv[1], dv[2]), plan_fwd);
    VectorXcd q = MBT_fft_mvp(n, f, Au_til, p, plan_fwd, plan_inv);
    MatrixXcd X = bl_cocg_rq_jacobi_mvp_fft(n, f, address, Au_til, diag, B, dv[3], itermax, plan_fwd, plan_inv);
    const int iters = last_stats().iterations;
    auto qr = qr_reduced(B);
    std::ofstream out(argv[2], std::ios::binary);
    wr(out, q.data(), q.size());
    wr(out, X.data(), (size_t)X.rows() * X.cols());
    wr(out, std::get<0>(qr).data(), (size_t)3 * nocc * L);
    wr(out, std::get<1>(qr).data(), (size_t)L * L);
    wr(out, &iters, 1);
  } catch (const Error& e) {
    std::fprintf(stderr, "bdda error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
