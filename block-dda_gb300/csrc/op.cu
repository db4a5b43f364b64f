// Operator lifecycle and MVP entry points of the C ABI.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bdda.h"
#include "op.hpp"

namespace bdda {

namespace {
thread_local std::string g_err;
}

void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }

static int cuda_fail(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? BDDA_ERR_NOMEM : BDDA_ERR_CUDA;
}
#define BDDA_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
  } while (0)

static int smooth235(int v) {
  for (;; ++v) {
    int t = v;
    for (int p : {2, 3, 5})
      while (t % p == 0) t /= p;
    if (t == 1) return v;
  }
}

Op::~Op() {
  if (stream) cudaStreamDestroy(stream);
}

int build_occupancy(Op* op, const int* address, int nocc, Occupancy* o) {
  const int nx = op->n[0], ny = op->n[1], nz = op->n[2];
  const size_t nc = (size_t)nx * ny * nz;
  std::vector<int> occ(nc, -1);
  std::vector<unsigned char> lmask((size_t)nx * ny, 0);
  if (address == nullptr) nocc = (int)nc;
  for (int m = 0; m < nocc; ++m) {
    const long long a = address ? address[m] : m;
    if (a < 0 || a >= (long long)nc) {
      set_error("dipole address out of the lattice box");
      return BDDA_ERR_INVALID;
    }
    if (occ[a] >= 0) {
      set_error("duplicate dipole address " + std::to_string(a));
      return BDDA_ERR_INVALID;
    }
    occ[a] = m;
    lmask[a / nz] = 1;
  }
  std::vector<int> lines;
  for (size_t i = 0; i < lmask.size(); ++i)
    if (lmask[i]) lines.push_back((int)i);
  o->nocc = nocc;
  o->nlines = (int)lines.size();
  BDDA_CUDA(o->occ.ensure(nc * sizeof(int)));
  BDDA_CUDA(o->lmask.ensure(lmask.size()));
  BDDA_CUDA(o->lines.ensure(std::max<size_t>(1, lines.size()) * sizeof(int)));
  BDDA_CUDA(cudaMemcpy(o->occ.p, occ.data(), nc * sizeof(int), cudaMemcpyHostToDevice));
  BDDA_CUDA(cudaMemcpy(o->lmask.p, lmask.data(), lmask.size(), cudaMemcpyHostToDevice));
  if (!lines.empty()) BDDA_CUDA(cudaMemcpy(o->lines.p, lines.data(), lines.size() * sizeof(int), cudaMemcpyHostToDevice));
  return BDDA_OK;
}

template <typename T>
int op_block_mvp(Op* op, const Occupancy& o, const typename cplx<T>::type* x, int ldx, typename cplx<T>::type* y, int ldy,
                 int L, const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre, cudaStream_t st,
                 const int* done) {
  using C = typename cplx<T>::type;
  const int pi = std::is_same<T, double>::value ? 0 : 1;
  const int need = std::is_same<T, double>::value ? BDDA_PREC_FP64 : BDDA_PREC_FP32;
  if (!(op->prec & need)) {
    set_error("operator was created without the tables of this precision");
    return BDDA_ERR_INVALID;
  }
  if (L < 1 || ldx < 3 * o.nocc || ldy < 3 * o.nocc) {
    set_error("bad L or leading dimension");
    return BDDA_ERR_INVALID;
  }
  const size_t nf = 3 * (size_t)L;
  const size_t t1 = nf * op->n[0] * op->n[1] * op->P[2] * sizeof(C);
  const size_t t2 = nf * op->n[0] * (size_t)op->P[1] * op->P[2] * sizeof(C);
  BDDA_CUDA(op->t1[pi].ensure(t1));
  BDDA_CUDA(op->t2[pi].ensure(t2));
  MvpGeom g = op->geom(o);
  cudaError_t e = launch_block_mvp<T>(g, op->tables<T>(), x, ldx, y, ldy, L, diag, jpre, op->t1[pi].as<C>(),
                                      op->t2[pi].as<C>(), st, &op->timer, done);
  op->kernel_launches += 5;
  if (e != cudaSuccess) return cuda_fail(e, "block MVP launch");
  return BDDA_OK;
}

template int op_block_mvp<double>(Op*, const Occupancy&, const double2*, int, double2*, int, int, const double2*,
                                  const double2*, cudaStream_t, const int*);
template int op_block_mvp<float>(Op*, const Occupancy&, const float2*, int, float2*, int, int, const float2*,
                                 const float2*, cudaStream_t, const int*);

}  // namespace bdda

using namespace bdda;

extern "C" {

const char* bdda_last_error(void) { return bdda::last_error(); }

int bdda_op_create(bdda_op** out, const int n[3], int f, double lf, double k_re, double k_im, int prec) {
  if (!out || !n) { set_error("null argument"); return BDDA_ERR_INVALID; }
  *out = nullptr;
  if (f != 3) { set_error("unknown f value (only f=3 is supported)"); return BDDA_ERR_INVALID; }
  if ((prec & (BDDA_PREC_FP64 | BDDA_PREC_FP32)) == 0) { set_error("no precision requested"); return BDDA_ERR_INVALID; }
  for (int i = 0; i < 3; ++i)
    if (n[i] < 1 || n[i] > kMaxLine / 2) {
      set_error("lattice box dimension outside 1..256");
      return BDDA_ERR_INVALID;
    }
  if (!(lf > 0.0)) { set_error("lattice spacing must be positive"); return BDDA_ERR_INVALID; }
  std::unique_ptr<bdda_op> op(new bdda_op());
  op->f = f;
  op->lf = lf;
  op->kr = k_re;
  op->ki = k_im;
  op->prec = prec;
  for (int i = 0; i < 3; ++i) {
    op->n[i] = n[i];
    op->P[i] = smooth235(2 * n[i]);
    if (!make_axis_plan(op->P[i], &op->plan[i])) { set_error("no FFT plan for the padded grid"); return BDDA_ERR_INVALID; }
  }
  BDDA_CUDA(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  // twiddles
  for (int i = 0; i < 3; ++i) {
    std::vector<double2> tw;
    make_twiddles(op->P[i], &tw);
    BDDA_CUDA(op->tw64[i].ensure(tw.size() * sizeof(double2)));
    BDDA_CUDA(cudaMemcpy(op->tw64[i].p, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice));
    std::vector<float2> tf(tw.size());
    for (size_t t = 0; t < tw.size(); ++t) tf[t] = make_float2((float)tw[t].x, (float)tw[t].y);
    BDDA_CUDA(op->tw32[i].ensure(tf.size() * sizeof(float2)));
    BDDA_CUDA(cudaMemcpy(op->tw32[i].p, tf.data(), tf.size() * sizeof(float2), cudaMemcpyHostToDevice));
  }
  BDDA_CUDA(configure_mvp_kernels<double>(kMaxLine));  // largest line, so every live operator fits
  BDDA_CUDA(configure_mvp_kernels<float>(kMaxLine));
  // Green spectrum
  const int Px = op->P[0], Py = op->P[1], Pz = op->P[2];
  const size_t ng = (size_t)Px * Py * Pz;
  DevBuf work;
  BDDA_CUDA(work.ensure(6 * ng * sizeof(double2)));
  const int nzt_d = (Pz + TileCfg<double>::TZ - 1) / TileCfg<double>::TZ;
  const int nzt_f = (Pz + TileCfg<float>::TZ - 1) / TileCfg<float>::TZ;
  if (prec & BDDA_PREC_FP64) BDDA_CUDA(op->ghat64.ensure((size_t)Py * nzt_d * 6 * Px * TileCfg<double>::TZ * sizeof(double2)));
  if (prec & BDDA_PREC_FP32) BDDA_CUDA(op->ghat32.ensure((size_t)Py * nzt_f * 6 * Px * TileCfg<float>::TZ * sizeof(float2)));
  MvpGeom g = op->geom(op->dip);
  BDDA_CUDA(build_green_hat(g, lf, k_re, k_im, op->tw64[0].as<double2>(), op->tw64[1].as<double2>(),
                            op->tw64[2].as<double2>(), work.as<double2>(), op->ghat64.as<double2>(),
                            op->ghat32.as<float2>(), op->stream));
  BDDA_CUDA(cudaStreamSynchronize(op->stream));
  *out = op.release();
  return BDDA_OK;
}

int bdda_op_destroy(bdda_op* op) {
  delete op;
  return BDDA_OK;
}

int bdda_op_set_dipoles(bdda_op* op, const int* address, int nocc) {
  if (!op || (address == nullptr && nocc != 0) || nocc < 0) {
    set_error("bad dipole list");
    return BDDA_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(op->mu);
  return build_occupancy(op, address, nocc, &op->dip);
}

int bdda_op_info(const bdda_op* op, int P[3], int* nocc, int* nlines) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  if (P) for (int i = 0; i < 3; ++i) P[i] = op->P[i];
  if (nocc) *nocc = op->dip.nocc;
  if (nlines) *nlines = op->dip.nlines;
  return BDDA_OK;
}

int bdda_mbt_fft_mvp(bdda_op* op, const double* p_hat, double* q_hat) {
  if (!op || !p_hat || !q_hat) { set_error("null argument"); return BDDA_ERR_INVALID; }
  if (!(op->prec & BDDA_PREC_FP64)) { set_error("MBT_fft_mvp needs the FP64 tables"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  if (op->cub.nocc == 0) {
    int rc = build_occupancy(op, nullptr, 0, &op->cub);
    if (rc) return rc;
  }
  const size_t nrow = 3 * (size_t)op->cub.nocc;
  DevBuf x, y;
  BDDA_CUDA(x.ensure(nrow * sizeof(double2)));
  BDDA_CUDA(y.ensure(nrow * sizeof(double2)));
  BDDA_CUDA(cudaMemcpyAsync(x.p, p_hat, nrow * sizeof(double2), cudaMemcpyHostToDevice, op->stream));
  int rc = op_block_mvp<double>(op, op->cub, x.as<double2>(), (int)nrow, y.as<double2>(), (int)nrow, 1, nullptr, nullptr,
                                op->stream);
  if (rc) return rc;
  BDDA_CUDA(cudaMemcpyAsync(q_hat, y.p, nrow * sizeof(double2), cudaMemcpyDeviceToHost, op->stream));
  BDDA_CUDA(cudaStreamSynchronize(op->stream));
  return BDDA_OK;
}

int bdda_op_mvp_device(bdda_op* op, int prec, const void* x, int ldx, void* y, int ldy, int L, const void* diag,
                       const void* jpre, void* stream) {
  if (!op || !x || !y) { set_error("null argument"); return BDDA_ERR_INVALID; }
  if (op->dip.nocc == 0) { set_error("no dipoles set on the operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : op->stream;
  if (prec == BDDA_PREC_FP64)
    return op_block_mvp<double>(op, op->dip, (const double2*)x, ldx, (double2*)y, ldy, L, (const double2*)diag,
                                (const double2*)jpre, st);
  if (prec == BDDA_PREC_FP32)
    return op_block_mvp<float>(op, op->dip, (const float2*)x, ldx, (float2*)y, ldy, L, (const float2*)diag,
                               (const float2*)jpre, st);
  set_error("prec must be BDDA_PREC_FP64 or BDDA_PREC_FP32");
  return BDDA_ERR_INVALID;
}

int bdda_op_set_timing(bdda_op* op, int enable) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->timer.enabled = enable != 0;
  return BDDA_OK;
}

int bdda_op_kernel_stats(bdda_op* op, double* ms, long long* launches, int n, int reset) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  cudaStreamSynchronize(op->stream);
  cudaDeviceSynchronize();
  op->timer.resolve();
  const int m = std::min(n, (int)kNumKernelIds);
  for (int i = 0; i < m; ++i) {
    if (ms) ms[i] = op->timer.ms[i];
    if (launches) launches[i] = op->timer.launches[i];
  }
  if (reset) op->timer.reset();
  return m;
}

}  // extern "C"
