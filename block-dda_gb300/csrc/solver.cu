// Block Krylov solvers on the device, FP64 refinement loop and qr_reduced.
//
// Every Krylov iteration is a fixed sequence of kernel launches with no host
// round trip: block MVP passes, tall-skinny Gram reductions, one-CTA FP64
// L x L steps (LU solves, Cholesky factors of CholQR2, stopping test) and row
// transforms.  The stopping test runs on the device and raises
// SolverCtl::done; every later kernel of the solve returns at entry, so the
// host only polls the control block every few iterations.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/bdda.h"
#include "krylov_kernels.cuh"
#include "op.hpp"
#include "small.cuh"

namespace bdda {

// Iteration cap of an FP32 inner solve of a mixed refinement (the FP64
// fallback of the refinement loop takes over where FP32 Krylov stalls).
constexpr int kMixedInnerCap = 200;

// ---------------------------------------------------------------------------
// small-state slots (each L x L complex FP64, column-major)
// ---------------------------------------------------------------------------
enum Slot {
  kXi = 0, kAlpha, kNAlpha, kAXi, kR1, kR1Inv, kR2Inv, kTau, kQtQ, kBeta, kM, kM2, kZetaI, kNZetaI, kIdent, kNIdent,
  kNumSlots
};

// One poll cycle of block COCG-RQ (the iterations between two reads of the
// control block) captured as a CUDA graph: ~18 launches per iteration become
// one graph launch, which is what bounds small systems.  It is replayed while
// every argument its kernels were captured with is unchanged (the key); the
// iteration index and the tolerance are read from the control block.
struct CycleGraph {
  struct Key {
    const void *op, *X, *Bp, *Q, *diag, *jpre;
    cudaStream_t st;
    unsigned long long dip_epoch, op_bufs, work_bufs;
    int solver, n, L, full, cycle;
    unsigned timing;
  };
  Key key;
  cudaGraphExec_t exec = nullptr;
  int mvps = 0;  // block MVPs one replay runs
  TimerRec rec;  // launch counts and timed pairs of one replay
  CycleGraph() { std::memset(&key, 0, sizeof key); }
  CycleGraph(const CycleGraph&) = delete;
  CycleGraph& operator=(const CycleGraph&) = delete;
  bool matches(const Key& k) const { return exec != nullptr && std::memcmp(&key, &k, sizeof k) == 0; }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    mvps = 0;
    rec.clear();
    std::memset(&key, 0, sizeof key);
  }
  ~CycleGraph() { reset(); }
};

struct SolverWork {
  int n = 0, L = 0;
  DevBuf blk64[10], blk32[10];   // 0-7 Krylov blocks, 8 right-hand side, 9 solution
  DevBuf X64, R64, Y64;
  DevBuf xdf, ydf, diagdf;      // double-float residual MVP (mixed solves)
  DevBuf jpre64, diag32, jpre32;
  DevBuf gpart;                 // per-CTA Gram partials [G][L*L], or [G][2 L*L] for gram2
  DevBuf partials, partials2;   // reduced Gram matrices (c128) [L*L]
  DevBuf vpart;                 // dot / norm partials
  DevBuf colf;                  // FP64 [2][L]: column scaling of the inner right-hand side and its inverse
  DevBuf small;                 // c128 [kNumSlots][L*L] + scalars
  DevBuf ctl;                   // SolverCtl
  DevBuf hist;                  // double[itermax]
  CycleGraph cycle[2];          // COCG-RQ poll cycle per precision (0 FP64, 1 FP32)
  SolverCtl ctl_host_buf{};           // pageable: the poll copy completes before returning
  SolverCtl* ctl_host = &ctl_host_buf;

  unsigned long long buffer_sig() const {
    unsigned long long h = 0;
    for (int i = 0; i < 10; ++i) h = sig_add(sig_add(h, blk64[i]), blk32[i]);
    for (const DevBuf* b : {&X64, &R64, &Y64, &xdf, &ydf, &diagdf, &jpre64, &diag32, &jpre32, &gpart, &partials,
                            &partials2, &vpart, &colf, &small, &ctl, &hist})
      h = sig_add(h, *b);
    return h;
  }
};

namespace {

int cuda_fail(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? BDDA_ERR_NOMEM : BDDA_ERR_CUDA;
}
#define BDDA_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
  } while (0)
#define BDDA_TRY(call)           \
  do {                           \
    int _rc = (call);            \
    if (_rc != BDDA_OK) return _rc; \
  } while (0)

inline int gram_grid(int n) { return std::max(1, std::min(2 * 152, (n + 63) / 64)); }
inline int vec_grid(size_t total) { return (int)std::max<size_t>(1, std::min<size_t>(608, (total + 255) / 256)); }

__device__ __forceinline__ double2* slot(double2* st, int s, int L) { return st + (size_t)s * L * L; }

// ---------------------------------------------------------------------------
// one-CTA steps
// ---------------------------------------------------------------------------
struct SmallSmem {
  // dynamic smem carve-up: 6 matrices + reduction scratch
  static size_t bytes(int L) { return 6 * (size_t)L * L * sizeof(double2) + (2 + kMaxL) * sizeof(int); }
};

#define SMALL_PROLOGUE                                                                              \
  using M = typename SmallMat<R>::M;                                                                \
  extern __shared__ __align__(16) unsigned char smem_raw[];                                         \
  M* m0 = reinterpret_cast<M*>(smem_raw);                                                           \
  M* m1 = m0 + L * L;                                                                               \
  [[maybe_unused]] M* m2 = m1 + L * L;                                                              \
  [[maybe_unused]] M* m3 = m2 + L * L;                                                              \
  [[maybe_unused]] M* m4 = m3 + L * L;                                                              \
  [[maybe_unused]] M* m5 = m4 + L * L;                                                              \
  [[maybe_unused]] int* piv = reinterpret_cast<int*>(m5 + L * L);                                   \
  [[maybe_unused]] int* colperm = piv + 2;                                                          \
  const int LL = L * L;

__device__ void fail(SolverCtl* ctl) {
  if (threadIdx.x == 0) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; }
}

// Deterministic sum of vpart[0..count) by one CTA of 256 threads (fixed tree).
__device__ double block_sum_256(const double* __restrict__ vpart, int count) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < count; i += 256) s += vpart[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// Identity helpers and ||B|| from column-norm partials.  256 threads.
__global__ void __launch_bounds__(256) k_small_init(const double* __restrict__ vpart, int nparts, int L, double2* st, SolverCtl* ctl,
                                                    double tol) {
  const int LL = L * L;
  for (int e = threadIdx.x; e < LL; e += blockDim.x) {
    const int i = e % L, j = e / L;
    slot(st, kIdent, L)[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    slot(st, kNIdent, L)[e] = make_double2(i == j ? -1.0 : 0.0, 0.0);
  }
  const double s = block_sum_256(vpart, nparts * L);
  if (threadIdx.x == 0) {
    ctl->bnorm = sqrt(s);
    ctl->done = 0;
    ctl->status = 0;
    ctl->iter = 0;
    ctl->err = 1.0;
    ctl->tol = tol;
    if (!(s > 0.0) || !isfinite(s)) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; }
  }
}

// Cholesky factor and its inverse of the Gram matrix in m0 (into m1, m2).
// In double-float the matrix is first scaled by an exact power of two so that
// its largest diagonal is O(1) (the double-float exponent range is FP32's),
// and the factors are scaled back; FP64 factors it as it is.
template <typename R>
__device__ bool chol_and_inverse(typename SmallMat<R>::M* m0, typename SmallMat<R>::M* m1, typename SmallMat<R>::M* m2,
                                 int L) {
  if constexpr (std::is_same<R, dfl>::value) {
    __shared__ int e2;
    if (threadIdx.x < 32) {  // largest diagonal (leading parts), one warp, FP32
      float mx = threadIdx.x < L ? fabsf(m0[threadIdx.x * (L + 1)].x.hi) : 0.0f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (threadIdx.x == 0) e2 = mx > 0.0f && isfinite(mx) ? ilogbf(mx) / 2 : 0;  // H / 4^e2 has diagonals O(1)
    }
    __syncthreads();
    const float sh = ldexpf(1.0f, -2 * e2);
    for (int e = threadIdx.x; e < L * L; e += blockDim.x) {
      m0[e].x = dfl(m0[e].x.hi * sh, m0[e].x.lo * sh);
      m0[e].y = dfl(m0[e].y.hi * sh, m0[e].y.lo * sh);
    }
    __syncthreads();
    if (!sm_cholesky<R>(m1, m0, L)) return false;
    sm_tri_inv<R>(m2, m1, L);
    const float sr = ldexpf(1.0f, e2), si = ldexpf(1.0f, -e2);  // R = R' 2^e2, R^-1 = R'^-1 2^-e2
    for (int e = threadIdx.x; e < L * L; e += blockDim.x) {
      m1[e].x = dfl(m1[e].x.hi * sr, m1[e].x.lo * sr);
      m1[e].y = dfl(m1[e].y.hi * sr, m1[e].y.lo * sr);
      m2[e].x = dfl(m2[e].x.hi * si, m2[e].x.lo * si);
      m2[e].y = dfl(m2[e].y.hi * si, m2[e].y.lo * si);
    }
    __syncthreads();
    return true;
  } else {
    if (!sm_cholesky<R>(m1, m0, L)) return false;
    sm_tri_inv<R>(m2, m1, L);
    return true;
  }
}

// The L x L steps of a COCG-RQ iteration on shared-memory matrices (the six
// L x L work matrices of SMALL_PROLOGUE); each one-CTA kernel fills the inputs
// (from reduced Gram partials) and calls one of them.
template <typename R> struct SmallWork {
  typename SmallMat<R>::M *m0, *m1, *m2, *m3, *m4, *m5;
  int *piv, *colperm;
};
#define SMALL_WORK SmallWork<R>{m0, m1, m2, m3, m4, m5, piv, colperm}

// QR step 1: R1 = chol(H), R1inv, with H = W^H W in w.m0.  false: breakdown.
template <typename R>
__device__ bool core_chol1(const SmallWork<R>& w, int L, double2* st, SolverCtl* ctl) {
  const int LL = L * L;
  if (!chol_and_inverse<R>(w.m0, w.m1, w.m2, L)) { fail(ctl); return false; }
  sm_store(slot(st, kR1, L), w.m1, LL);
  sm_store(slot(st, kR1Inv, L), w.m2, LL);
  return true;
}

// COCG-RQ, the second CholQR2 step fused with beta, with H2 = W1^H W1 in
// w.m0; load_gt(dst) puts W1^T W1 into a shared matrix.
//   R2 = chol(H2), R2inv, tau = R2 R1, xi = tau xi, err, stopping test;
//   Q' = W1 R2^-1, so Q'^T Q' = R2^-T (W1^T W1) R2^-1 without a pass over Q'
//   (R2 is near the identity: the second CholQR2 factor);
//   beta = (Q^T Q)^-1 (tau^T Q'^T Q') ; Q^T Q <- Q'^T Q'.
// Returns false on breakdown or when the stopping test passed (done).
template <typename R, class LoadGT>
__device__ bool core_chol2_beta(const SmallWork<R>& w, int L, double2* st, SolverCtl* ctl, double* hist, int full,
                                LoadGT load_gt) {
  const int LL = L * L;
  if (!chol_and_inverse<R>(w.m0, w.m1, w.m2, L)) { fail(ctl); return false; }
  sm_store(slot(st, kR2Inv, L), w.m2, LL);
  sm_load(w.m3, slot(st, kR1, L), LL);
  sm_matmul(w.m4, w.m1, w.m3, L, false);  // tau = R2 R1
  sm_store(slot(st, kTau, L), w.m4, LL);
  sm_load(w.m5, slot(st, kXi, L), LL);
  sm_matmul(w.m0, w.m4, w.m5, L, false);  // xi = tau xi
  sm_store(slot(st, kXi, L), w.m0, LL);
  const double nrm = sm_fro<R>(w.m0, LL);
  __shared__ int stop;
  if (threadIdx.x == 0) {
    // the iteration index and the tolerance come from the control block, so
    // the launch is the same at every iteration (captured poll cycles)
    const int k = ctl->iter;
    const double err = nrm / ctl->bnorm;
    ctl->err = err;
    if (hist) hist[k] = err;
    ctl->iter = k + 1;
    stop = 0;
    if (!isfinite(err)) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; stop = 1; }
    else if (err < ctl->tol) { ctl->done = 1; stop = 1; }
  }
  __syncthreads();
  if (stop) return false;
  load_gt(w.m0);                               // W1^T W1
  sm_matmul(w.m3, w.m0, w.m2, L, false);       // (W1^T W1) R2^-1
  sm_matmul(w.m5, w.m2, w.m3, L, true);        // Q'^T Q'
  sm_matmul(w.m0, w.m4, w.m5, L, true);        // tau^T Q'^T Q'
  sm_load(w.m1, slot(st, kQtQ, L), LL);
  if (!sm_lu_solve<R>(w.m1, w.m0, L, L, full != 0, w.colperm, w.piv)) { fail(ctl); return false; }
  sm_store(slot(st, kBeta, L), w.m0, LL);
  sm_store(slot(st, kQtQ, L), w.m5, LL);
  return true;
}

// COCG-RQ alpha with S^T AS in w.m0 and Q^T Q in w.m1 (have_qq; else the kept
// slot): alpha = (S^T AS)^-1 (Q^T Q) ; A_xi = alpha xi ; -alpha.
template <typename R>
__device__ bool core_alpha(const SmallWork<R>& w, int L, double2* st, SolverCtl* ctl, bool have_qq, int full) {
  const int LL = L * L;
  if (have_qq) sm_store(slot(st, kQtQ, L), w.m1, LL);
  else sm_load(w.m1, slot(st, kQtQ, L), LL);
  if (!sm_lu_solve<R>(w.m0, w.m1, L, L, full != 0, w.colperm, w.piv)) { fail(ctl); return false; }
  sm_store(slot(st, kAlpha, L), w.m1, LL);
  sm_store(slot(st, kNAlpha, L), w.m1, LL, true);
  sm_load(w.m2, slot(st, kXi, L), LL);
  sm_matmul(w.m3, w.m1, w.m2, L, false);
  sm_store(slot(st, kAXi, L), w.m3, LL);
  return true;
}

// QR step 1: H = W^H W ; R1 = chol(H) ; R1inv
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_chol1(const double2* __restrict__ part, int nparts, int L, double2* st, SolverCtl* ctl) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  sm_reduce<R>(m0, part, nparts, LL);
  core_chol1<R>(SMALL_WORK, L, st, ctl);
}

// QR step 2: H2 = W1^H W1 ; R2 = chol ; R2inv ; tau = R2 R1.
// mode 0: xi = tau (initial QR of the right-hand side)
// mode 1: xi = tau xi ; err = ||xi|| / bnorm ; stopping test
// mode 2: like mode 0 but R = tau returned in kXi only (qr_reduced)
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_chol2(const double2* __restrict__ part, int nparts, int L, double2* st, SolverCtl* ctl, double tol,
              double* hist, int k, int mode) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  sm_reduce<R>(m0, part, nparts, LL);
  if (!chol_and_inverse<R>(m0, m1, m2, L)) { fail(ctl); return; }
  sm_store(slot(st, kR2Inv, L), m2, LL);
  sm_load(m3, slot(st, kR1, L), LL);
  sm_matmul(m4, m1, m3, L, false);  // tau = R2 R1
  sm_store(slot(st, kTau, L), m4, LL);
  if (mode != 1) {
    sm_store(slot(st, kXi, L), m4, LL);
    return;
  }
  sm_load(m5, slot(st, kXi, L), LL);
  sm_matmul(m0, m4, m5, L, false);  // xi = tau xi
  sm_store(slot(st, kXi, L), m0, LL);
  const double nrm = sm_fro<R>(m0, LL);
  if (threadIdx.x == 0) {
    const double err = nrm / ctl->bnorm;
    ctl->err = err;
    if (hist) hist[k] = err;
    ctl->iter = k + 1;
    if (!isfinite(err)) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; }
    else if (err < tol) ctl->done = 1;
  }
}

// COCG-RQ, the second CholQR2 step fused with beta.  part holds the
// Hermitian and the unconjugated Gram of W1 = W R1^-1 ([2][L*L]).
//   R2 = chol(W1^H W1), R2inv, tau = R2 R1, xi = tau xi, err, stopping test;
//   Q' = W1 R2^-1, so Q'^T Q' = R2^-T (W1^T W1) R2^-1 without a pass over Q'
//   (R2 is near the identity: the second CholQR2 factor);
//   beta = (Q^T Q)^-1 (tau^T Q'^T Q') ; Q^T Q <- Q'^T Q'.
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_chol2_beta(const double2* __restrict__ part, int L, double2* st, SolverCtl* ctl, double* hist, int full) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  sm_reduce<R>(m0, part, 1, LL);
  core_chol2_beta<R>(SMALL_WORK, L, st, ctl, hist, full, [&](M* d) { sm_reduce<R>(d, part + LL, 1, LL); });
}

// COCG-RQ alpha: alpha = (S^T AS)^-1 (Q^T Q) ; A_xi = alpha xi ; -alpha
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_cocg_alpha(const double2* __restrict__ pSAS, const double2* __restrict__ pQQ, int nparts, int L, double2* st,
                   SolverCtl* ctl, int full) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  sm_reduce<R>(m0, pSAS, nparts, LL);
  if (pQQ) sm_reduce<R>(m1, pQQ, nparts, LL);
  core_alpha<R>(SMALL_WORK, L, st, ctl, pQQ != nullptr, full);
}

// COCG-RQ beta: beta = (Q^T Q)^-1 (tau^T Q'^T Q') ; Q^T Q <- Q'^T Q'
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_cocg_beta(const double2* __restrict__ pQQn, int nparts, int L, double2* st, SolverCtl* ctl, int full) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  sm_reduce<R>(m0, pQQn, nparts, LL);        // Q'^T Q'
  sm_load(m1, slot(st, kTau, L), LL);
  sm_matmul(m2, m1, m0, L, true);            // tau^T Q'^T Q'
  sm_load(m3, slot(st, kQtQ, L), LL);
  if (!sm_lu_solve<R>(m3, m2, L, L, full != 0, colperm, piv)) { fail(ctl); return; }
  sm_store(slot(st, kBeta, L), m2, LL);
  sm_store(slot(st, kQtQ, L), m0, LL);
}

// BiCG*: X = M^-1 RHS with M = reduce(pM) (stored in kM), RHS = scale * reduce(pR).
// out slots: x -> so, -x -> sno (optional)
template <typename R>
__global__ void __launch_bounds__(kSmallThreads)
k_small_solve(const double2* __restrict__ pM, const double2* __restrict__ pR, int nparts, int L, double2* st,
              SolverCtl* ctl, int mslot_in, int mslot_store, double rhs_scale, const double2* scal_div, int so, int sno) {
  if (ctl_skip(ctl)) return;
  SMALL_PROLOGUE
  if (pM) sm_reduce<R>(m0, pM, nparts, LL);
  else sm_load(m0, slot(st, mslot_in, L), LL);
  if (mslot_store >= 0) sm_store(slot(st, mslot_store, L), m0, LL);
  sm_reduce<R>(m1, pR, nparts, LL);
  double2 sc = make_double2(rhs_scale, 0.0);
  if (scal_div) sc = cdiv(sc, *scal_div);
  const M scm = m_from_double2<M>(sc);
  for (int e = threadIdx.x; e < LL; e += blockDim.x) m1[e] = cmul(m1[e], scm);
  __syncthreads();
  if (!sm_lu_solve<R>(m0, m1, L, L, false, colperm, piv)) { fail(ctl); return; }
  sm_store(slot(st, so, L), m1, LL);
  if (sno >= 0) sm_store(slot(st, sno, L), m1, LL, true);
}

// zeta = sum(p1) / sum(p2) ; kZetaI = zeta I ; kNZetaI = -zeta I ; scal[0] = zeta, scal[1] = -zeta
__global__ void k_small_zeta(const double2* __restrict__ p1, const double2* __restrict__ p2, int nparts, int L, double2* st,
                             double2* scal, SolverCtl* ctl) {
  if (ctl_skip(ctl)) return;
  __shared__ double2 z;
  if (threadIdx.x == 0) {
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    for (int p = 0; p < nparts; ++p) {
      a.x += p1[p].x; a.y += p1[p].y;
      b.x += p2[p].x; b.y += p2[p].y;
    }
    z = cdiv(a, b);
    if (!cfinite(z)) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; }
    scal[0] = z;
    scal[1] = make_double2(-z.x, -z.y);
  }
  __syncthreads();
  const int LL = L * L;
  for (int e = threadIdx.x; e < LL; e += blockDim.x) {
    const int i = e % L, j = e / L;
    slot(st, kZetaI, L)[e] = i == j ? z : make_double2(0.0, 0.0);
    slot(st, kNZetaI, L)[e] = i == j ? make_double2(-z.x, -z.y) : make_double2(0.0, 0.0);
  }
}

// err = sqrt(sum of column-norm partials) / bnorm ; stopping test.  256 threads.
// The iteration index and tolerance come from the control block (captured cycles).
__global__ void __launch_bounds__(256) k_small_err(const double* __restrict__ vpart, int nparts, int L, SolverCtl* ctl,
                                                   double* hist) {
  if (ctl_skip(ctl)) return;
  const double s = block_sum_256(vpart, nparts * L);
  if (threadIdx.x == 0) {
    const int k = ctl->iter;
    const double err = sqrt(s) / ctl->bnorm;
    ctl->err = err;
    if (hist) hist[k] = err;
    ctl->iter = k + 1;
    if (!isfinite(err)) { ctl->status = BDDA_ERR_BREAKDOWN; ctl->done = 1; }
    else if (err < ctl->tol) ctl->done = 1;
  }
}

// st[s] = reduce(partials)
__global__ void __launch_bounds__(kSmallThreads)
k_small_store_reduce(const double2* __restrict__ part, int nparts, int L, double2* st, SolverCtl* ctl, int s) {
  if (ctl_skip(ctl)) return;
  sm_reduce<double>(slot(st, s, L), part, nparts, L * L);
}

// ---------------------------------------------------------------------------
// host-side runner for one precision
// ---------------------------------------------------------------------------
template <typename T>
struct Krylov {
  using C = typename cplx<T>::type;
  // Arithmetic of the L x L steps of COCG-RQ and CholQR2, whose Gram matrices
  // are of orthonormalised blocks (O(1) entries): FP64 for FP64 solves,
  // double-float for the FP32 inner solves.  The BiCG* steps solve with
  // unnormalised Grams whose entries shrink with the residual (their squares
  // can leave the FP32 exponent range) and stay FP64.
  using SR = typename std::conditional<std::is_same<T, float>::value, dfl, double>::type;
  Op* op;
  SolverWork* w;
  cudaStream_t st;
  int n, L;
  const C* diag;
  const C* jpre;
  int check_every;
  int mvps = 0;

  SolverCtl* ctl() const { return w->ctl.as<SolverCtl>(); }
  double2* small() const { return w->small.as<double2>(); }
  double2* sl(int s) const { return small() + (size_t)s * L * L; }
  C* blk(int i) const { return (std::is_same<T, double>::value ? w->blk64[i] : w->blk32[i]).template as<C>(); }
  int G() const { return gram_grid(n); }

  int mvp(const C* x, C* y) {
    ++mvps;
    return op_block_mvp<T>(op, op->dip, x, n, y, n, L, diag, jpre, st, &ctl()->done);
  }
  // out = op(A)^T B (L x L, FP64): per-CTA partials, then a multi-CTA ordered reduction
  template <bool CONJ> void gram(const C* A, const C* B, double2* out) {
    op->timer.begin(kGram, st);
    using P = typename GramPart<T>::type;
    k_gram<T, CONJ><<<G(), kGramThreads, 0, st>>>(A, n, B, n, n, L, w->gpart.template as<P>(), ctl());
    k_gram_reduce<P><<<(L * L + kRedEntries - 1) / kRedEntries, kRedEntries * kRedGroups, 0, st>>>(
        w->gpart.template as<P>(), G(), L * L, out, ctl());
    op->timer.end(kGram, st);
    op->timer.count(kGram);
  }
  // out[0 .. LL) = A^H A, out[LL .. 2 LL) = A^T A
  void gram2(const C* A, double2* out) {
    op->timer.begin(kGram, st);
    using P = typename GramPart<T>::type;
    k_gram<T, true, true><<<G(), kGramThreads, 0, st>>>(A, n, A, n, n, L, w->gpart.template as<P>(), ctl());
    k_gram_reduce<P><<<(2 * L * L + kRedEntries - 1) / kRedEntries, kRedEntries * kRedGroups, 0, st>>>(
        w->gpart.template as<P>(), G(), 2 * L * L, out, ctl());
    op->timer.end(kGram, st);
    op->timer.count(kGram);
  }
  // Out1 = A Ma ; Out2 = Out1 + B Mb
  void rowmm2(const C* A, const double2* Ma, const C* B, const double2* Mb, C* Out1, C* Out2) {
    op->timer.begin(kUpdate, st);
    k_rowmm2<T><<<(n + kRowRows - 1) / kRowRows, kRowThreads, rowmm_smem<T>(L, true), st>>>(n, L, A, Ma, B, Mb, Out1,
                                                                                         Out2, ctl());
    op->timer.end(kUpdate, st);
  }
  void rowmm(const C* A, const double2* Ma, const C* B, const double2* Mb, const C* Cadd, C* Out) {
    op->timer.begin(kUpdate, st);
    k_rowmm<T><<<(n + kRowRows - 1) / kRowRows, kRowThreads, rowmm_smem<T>(L, B != nullptr), st>>>(
        n, L, A, n, Ma, B, n, Mb, Cadd, n, Out, n, ctl());
    op->timer.end(kUpdate, st);
  }
  void axpby(const double2* a, const C* A, const double2* b, const C* B, C* Out) {
    op->timer.begin(kUpdate, st);
    k_axpby<T><<<vec_grid((size_t)n * L), 256, 0, st>>>(n, L, a, A, n, b, B, n, Out, n, ctl());
    op->timer.end(kUpdate, st);
  }
  void dotc(const C* A, const C* B, double2* part) {
    op->timer.begin(kGram, st);
    k_dotc<T><<<vec_grid((size_t)n * L), 256, 0, st>>>(n, L, A, n, B, n, part, ctl());
    op->timer.end(kGram, st);
  }
  void colnorm(const C* A, double* part) {
    op->timer.begin(kGram, st);
    k_colnorm2<T><<<vec_grid((size_t)n * L), 256, 0, st>>>(A, n, n, L, part);
    op->timer.end(kGram, st);
  }
  template <typename K, typename... Args> void small_launch(K kern, Args... args) {
    op->timer.begin(kSmall, st);
    kern<<<1, kSmallThreads, SmallSmem::bytes(L), st>>>(args...);
    op->timer.end(kSmall, st);
  }

  // poll the control block; returns 1 when the device signalled done
  int poll(bool* done, bool wait = true) {
    BDDA_CUDA(cudaMemcpyAsync(w->ctl_host, ctl(), sizeof(SolverCtl), cudaMemcpyDeviceToHost, st));
    if (wait) BDDA_CUDA(wait_stream(st));
    *done = w->ctl_host->done != 0;
    return BDDA_OK;
  }

  // ||Bp||_F -> ctl->bnorm, identity slots, control reset
  int init(const C* Bp, double tol) {
    double* vp = w->vpart.as<double>();
    const int g = vec_grid((size_t)n * L);
    k_colnorm2<T><<<g, 256, 0, st>>>(Bp, n, n, L, vp);
    k_small_init<<<1, 256, 0, st>>>(vp, g, L, small(), ctl(), tol);
    op->timer.count(kOther, 2);
    return cudaGetLastError() == cudaSuccess ? BDDA_OK : cuda_fail(cudaGetLastError(), "init");
  }

  // [Q, R] = qr(A) by CholQR2 ; R -> kXi (mode 0/2).  W is scratch (may equal Q).
  void cholqr2(const C* A, C* W, C* Q, int mode) {
    double2* p = w->partials.template as<double2>();
    gram<true>(A, A, p);
    small_launch(k_small_chol1<SR>, (const double2*)p, 1, L, small(), ctl());
    rowmm(A, sl(kR1Inv), nullptr, nullptr, nullptr, W);
    gram<true>(W, W, p);
    small_launch(k_small_chol2<SR>, (const double2*)p, 1, L, small(), ctl(), 0.0, (double*)nullptr, 0, mode);
    rowmm(W, sl(kR2Inv), nullptr, nullptr, nullptr, Q);
  }

  // One block COCG-RQ iteration; first adds the Gram Q^T Q of the starting block.
  int cocg_iteration(bool first, C* Q, C* Qn, C* S, C* AS, C* W, C* X, bool full) {
    double2* p = w->partials.template as<double2>();
    double2* p2 = w->partials2.template as<double2>();
    BDDA_TRY(mvp(S, AS));
    gram<false>(S, AS, p);
    if (first) gram<false>(Q, Q, p2);
    small_launch(k_small_cocg_alpha<SR>, (const double2*)p, (const double2*)(first ? p2 : nullptr), 1, L, small(), ctl(),
                 (int)full);
    rowmm(S, sl(kAXi), nullptr, nullptr, X, X);           // X += S alpha xi
    rowmm(AS, sl(kNAlpha), nullptr, nullptr, Q, W);       // W = Q - AS alpha
    gram<true>(W, W, p);
    small_launch(k_small_chol1<SR>, (const double2*)p, 1, L, small(), ctl());
    rowmm(W, sl(kR1Inv), nullptr, nullptr, nullptr, W);   // W1
    gram2(W, p);                                          // W1^H W1, W1^T W1
    small_launch(k_small_chol2_beta<SR>, (const double2*)p, L, small(), ctl(), w->hist.as<double>(), (int)full);
    rowmm2(W, sl(kR2Inv), S, sl(kBeta), Qn, S);           // Q' = W1 R2^-1 ; S = Q' + S beta
    return BDDA_OK;
  }

  // Poll cycles run as graphs with an even cycle length (Q and Qn are back in
  // place after it), on a non-blocking stream: while a blocking stream is
  // captured, work another thread puts on the legacy default stream would
  // fail.  The operators' own streams are non-blocking.  BDDA_NO_GRAPH turns
  // the graphs off (diagnostics).
  bool graphs_allowed() const {
    if (!op->graphs || check_every < 2 || check_every % 2 != 0 || st == nullptr || st == cudaStreamLegacy ||
        st == cudaStreamPerThread || std::getenv("BDDA_NO_GRAPH") != nullptr)
      return false;
    unsigned int flags = 0;
    if (cudaStreamGetFlags(st, &flags) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    return (flags & cudaStreamNonBlocking) != 0;
  }

  // Launches one poll cycle as a graph: `cycle` issues its check_every
  // iterations (none of them the first) and runs only under capture, when the
  // cached graph was captured with other arguments.  *ran = false when the
  // stream could not be captured: nothing was launched then, and the caller
  // runs the cycle launch by launch.
  template <class Cycle>
  int cycle_graph(int solver, const C* X, const C* Bp, const C* first, bool full, Cycle cycle, bool* ran) {
    *ran = false;
    CycleGraph& cg = w->cycle[std::is_same<T, double>::value ? 0 : 1];
    CycleGraph::Key key;
    std::memset(&key, 0, sizeof key);
    key.op = op;
    key.X = X;
    key.Bp = Bp;
    key.Q = first;
    key.diag = diag;
    key.jpre = jpre;
    key.st = st;
    key.dip_epoch = op->dip_epoch;
    key.op_bufs = op->buffer_sig();
    key.work_bufs = w->buffer_sig();
    key.solver = solver;
    key.n = n;
    key.L = L;
    key.full = full ? 1 : 0;
    key.cycle = check_every;
    key.timing = op->timer.state();
    if (!cg.matches(key)) {
      cg.reset();
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        return BDDA_OK;
      }
      op->timer.rec = &cg.rec;
      const int mvps_before = mvps;
      const int rc = cycle();
      const int cycle_mvps = mvps - mvps_before;
      mvps = mvps_before;
      op->timer.rec = nullptr;
      cudaGraph_t graph = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(st, &graph);
      cudaError_t ei = cudaErrorStreamCaptureInvalidated;
      if (rc == BDDA_OK && ec == cudaSuccess && graph) ei = cudaGraphInstantiate(&cg.exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        cg.exec = nullptr;
        cg.reset();
        (void)cudaGetLastError();
        return rc;  // an argument error of the iteration itself, else OK with *ran false
      }
      cg.key = key;
      cg.mvps = cycle_mvps;
    }
    BDDA_CUDA(cudaGraphLaunch(cg.exec, st));
    mvps += cg.mvps;
    *ran = true;
    return BDDA_OK;
  }

  // The iteration loop of the solvers.  iter(first) issues one iteration; the
  // host reads the control block every check_every iterations, and every
  // cycle after the first runs as one captured graph (the buffers an
  // iteration swaps are back in place after an even number of iterations).
  // first_blk names the block the cycle starts from (COCG-RQ's Q), else null.
  template <class Iter>
  int iterate(int solver, const C* X, const C* Bp, const C* const* first_blk, bool full, int itermax, Iter iter) {
    bool done = false;
    bool graphs = graphs_allowed();
    int k = 0;
    while (k < itermax) {
      if (graphs && k >= check_every && k % check_every == 0 && k + check_every <= itermax) {
        bool ran = false;
        auto cycle = [&]() -> int {
          for (int i = 0; i < check_every; ++i) BDDA_TRY(iter(false));
          return BDDA_OK;
        };
        BDDA_TRY(cycle_graph(solver, X, Bp, first_blk ? *first_blk : nullptr, full, cycle, &ran));
        if (ran) {
          k += check_every;
          BDDA_TRY(poll(&done));
          op->timer.replayed(w->cycle[std::is_same<T, double>::value ? 0 : 1].rec);
          if (done) break;
          continue;
        }
        graphs = false;
      }
      BDDA_TRY(iter(k == 0));
      ++k;
      if (k % check_every == 0 || k == itermax) {
        BDDA_TRY(poll(&done));
        if (done) break;
      }
    }
    if (!done) BDDA_TRY(poll(&done));
    return BDDA_OK;
  }

  // Block COCG-RQ (bl_cocg_rq_mvp_fft.cpp:22-71 / bl_cocg_rq_jacobi_mvp_fft.cpp:22-78)
  int cocg_rq(const C* Bp, C* X, bool full, double tol, int itermax, int* iters, double* err, int* status) {
    C* Q = blk(0); C* Qn = blk(1); C* S = blk(2); C* AS = blk(3); C* W = blk(4);
    BDDA_CUDA(cudaMemsetAsync(X, 0, sizeof(C) * (size_t)n * L, st));
    BDDA_TRY(init(Bp, tol));
    cholqr2(Bp, W, Q, 0);
    BDDA_CUDA(cudaMemcpyAsync(S, Q, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_TRY(iterate(0, X, Bp, &Q, full, itermax, [&](bool first) -> int {
      BDDA_TRY(cocg_iteration(first, Q, Qn, S, AS, W, X, full));
      std::swap(Q, Qn);
      return BDDA_OK;
    }));
    *iters = w->ctl_host->iter;
    *err = w->ctl_host->err;
    *status = w->ctl_host->status;
    return cudaGetLastError() == cudaSuccess ? BDDA_OK : cuda_fail(cudaGetLastError(), "cocg_rq");
  }

  // Block BiCGSTAB (bl_bicgstab_mvp_fft.cpp:21-98 / bl_bicgstab_jacobi_mvp_fft.cpp:21-96)
  int bicgstab(const C* Bp, C* X, double tol, int itermax, int* iters, double* err, int* status) {
    C* R = blk(0); C* P = blk(1); C* R0 = blk(2); C* V = blk(3); C* Tm = blk(4); C* Z = blk(5); C* Pt = blk(6);
    double2* p = w->partials.template as<double2>();
    double2* p2 = w->partials2.template as<double2>();
    double2* vp = w->vpart.as<double2>();
    double2* scal = sl(kNumSlots);  // 2 scalars after the matrix slots
    BDDA_CUDA(cudaMemsetAsync(X, 0, sizeof(C) * (size_t)n * L, st));
    BDDA_TRY(init(Bp, tol));
    BDDA_CUDA(cudaMemcpyAsync(R, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_CUDA(cudaMemcpyAsync(P, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_CUDA(cudaMemcpyAsync(R0, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    const int gv = vec_grid((size_t)n * L);
    BDDA_TRY(iterate(1, X, Bp, nullptr, false, itermax, [&](bool) -> int {
      BDDA_TRY(mvp(P, V));                                   // V = A P
      gram<true>(R0, V, p);
      gram<true>(R0, R, p2);
      small_launch(k_small_solve<double>, (const double2*)p, (const double2*)p2, 1, L, small(), ctl(), 0, (int)kM, 1.0,
                   (const double2*)nullptr, (int)kAlpha, (int)kNAlpha);
      rowmm(V, sl(kNAlpha), nullptr, nullptr, R, Tm);        // T = R - V alpha
      BDDA_TRY(mvp(Tm, Z));                                  // Z = A T
      dotc(Z, Tm, vp);
      dotc(Z, Z, vp + gv);
      op->timer.begin(kSmall, st);
      k_small_zeta<<<1, 256, 0, st>>>(vp, vp + gv, gv, L, small(), scal, ctl());
      op->timer.end(kSmall, st);
      rowmm(P, sl(kAlpha), Tm, sl(kZetaI), X, X);            // X = X + P alpha + zeta T
      axpby(nullptr, Tm, scal + 1, Z, R);                    // R = T - zeta Z
      colnorm(R, w->vpart.as<double>());
      op->timer.begin(kSmall, st);
      k_small_err<<<1, 256, 0, st>>>(w->vpart.as<double>(), gv, L, ctl(), w->hist.as<double>());
      op->timer.end(kSmall, st);
      gram<true>(R0, Z, p);
      small_launch(k_small_solve<double>, (const double2*)nullptr, (const double2*)p, 1, L, small(), ctl(), (int)kM, -1, -1.0,
                   (const double2*)nullptr, (int)kBeta, -1);  // beta = M^-1 (-R0^H Z)
      axpby(nullptr, P, scal + 1, V, Pt);                    // Pt = P - zeta V
      rowmm(Pt, sl(kBeta), nullptr, nullptr, R, P);          // P = R + Pt beta
      return BDDA_OK;
    }));
    *iters = w->ctl_host->iter;
    *err = w->ctl_host->err;
    *status = w->ctl_host->status;
    return cudaGetLastError() == cudaSuccess ? BDDA_OK : cuda_fail(cudaGetLastError(), "bicgstab");
  }

  // Block BiCGGR (bl_bicggr_mvp_fft.cpp:18-116 / bl_bicggr_jacobi_mvp_fft.cpp:18-117)
  int bicggr(const C* Bp, C* X, double tol, int itermax, int* iters, double* err, int* status) {
    C* R = blk(0); C* P = blk(1); C* R0 = blk(2); C* V = blk(3); C* Wm = blk(4); C* U = blk(5); C* Y = blk(6); C* Rn = blk(7);
    double2* p = w->partials.template as<double2>();
    double2* p2 = w->partials2.template as<double2>();
    double2* vp = w->vpart.as<double2>();
    double2* scal = sl(kNumSlots);
    BDDA_CUDA(cudaMemsetAsync(X, 0, sizeof(C) * (size_t)n * L, st));
    BDDA_TRY(init(Bp, tol));
    BDDA_CUDA(cudaMemcpyAsync(R, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_CUDA(cudaMemcpyAsync(P, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_CUDA(cudaMemcpyAsync(R0, Bp, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    BDDA_TRY(mvp(R, V));                                     // V = A R
    BDDA_CUDA(cudaMemcpyAsync(Wm, V, sizeof(C) * (size_t)n * L, cudaMemcpyDeviceToDevice, st));
    const int gv = vec_grid((size_t)n * L);
    BDDA_TRY(iterate(2, X, Bp, &R, false, itermax, [&](bool) -> int {
      gram<true>(R0, V, p);
      gram<true>(R0, R, p2);
      small_launch(k_small_solve<double>, (const double2*)p, (const double2*)p2, 1, L, small(), ctl(), 0, -1, 1.0,
                   (const double2*)nullptr, (int)kAlpha, -1);
      // keep R0^H R (old R) for gamma
      small_launch(k_small_store_reduce, (const double2*)p2, 1, L, small(), ctl(), (int)kM2);
      dotc(Wm, R, vp);
      dotc(Wm, Wm, vp + gv);
      op->timer.begin(kSmall, st);
      k_small_zeta<<<1, 256, 0, st>>>(vp, vp + gv, gv, L, small(), scal, ctl());
      op->timer.end(kSmall, st);
      axpby(nullptr, P, scal + 1, V, Rn);                    // S = P - zeta V   (Rn as scratch)
      rowmm(Rn, sl(kAlpha), nullptr, nullptr, nullptr, U);   // U = S alpha
      BDDA_TRY(mvp(U, Y));                                   // Y = A U
      rowmm(R, sl(kZetaI), U, sl(kIdent), X, X);             // X = X + zeta R + U
      rowmm(Wm, sl(kNZetaI), Y, sl(kNIdent), R, Rn);         // Rn = R - zeta W - Y
      colnorm(Rn, w->vpart.as<double>());
      op->timer.begin(kSmall, st);
      k_small_err<<<1, 256, 0, st>>>(w->vpart.as<double>(), gv, L, ctl(), w->hist.as<double>());
      op->timer.end(kSmall, st);
      BDDA_TRY(mvp(Rn, Wm));                                 // W = A Rnew
      gram<true>(R0, Rn, p);
      small_launch(k_small_solve<double>, (const double2*)nullptr, (const double2*)p, 1, L, small(), ctl(), (int)kM2, -1, 1.0,
                   (const double2*)scal, (int)kBeta, -1);    // gamma = (R0^H R)^-1 (R0^H Rnew / zeta)
      std::swap(R, Rn);
      rowmm(U, sl(kBeta), nullptr, nullptr, R, P);           // P = R + U gamma
      rowmm(Y, sl(kBeta), nullptr, nullptr, Wm, V);          // V = W + Y gamma
      return BDDA_OK;
    }));
    // R/Rn swapping above only changes which buffer holds the residual; X is final.
    *iters = w->ctl_host->iter;
    *err = w->ctl_host->err;
    *status = w->ctl_host->status;
    return cudaGetLastError() == cudaSuccess ? BDDA_OK : cuda_fail(cudaGetLastError(), "bicggr");
  }

  int run(int solver, const C* Bp, C* X, bool full, double tol, int itermax, int* iters, double* err, int* status) {
    switch (solver) {
      case BDDA_SOLVER_COCG_RQ: return cocg_rq(Bp, X, full, tol, itermax, iters, err, status);
      case BDDA_SOLVER_BICGSTAB: return bicgstab(Bp, X, tol, itermax, iters, err, status);
      case BDDA_SOLVER_BICGGR: return bicggr(Bp, X, tol, itermax, iters, err, status);
      default: set_error("unknown solver id"); return BDDA_ERR_INVALID;
    }
  }

};

}  // namespace

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
static int ensure_work(Op* op, int n, int L, int itermax, bool need64, bool need32) {
  if (!op->solver) op->solver = std::make_shared<SolverWork>();
  SolverWork* w = op->solver.get();
  const size_t b64 = sizeof(double2) * (size_t)n * L, b32 = sizeof(float2) * (size_t)n * L;
  for (int i = 0; i < 10; ++i) {
    if (need64) BDDA_CUDA(w->blk64[i].ensure(b64, op->stream));
    if (need32) BDDA_CUDA(w->blk32[i].ensure(b32, op->stream));
  }
  BDDA_CUDA(w->X64.ensure(b64, op->stream));
  BDDA_CUDA(w->R64.ensure(b64, op->stream));
  BDDA_CUDA(w->Y64.ensure(b64, op->stream));
  BDDA_CUDA(w->jpre64.ensure(sizeof(double2) * (size_t)n, op->stream));
  if (op->prec & BDDA_PREC_DF64) {
    BDDA_CUDA(w->xdf.ensure(sizeof(dfc) * (size_t)n * L, op->stream));
    BDDA_CUDA(w->ydf.ensure(sizeof(dfc) * (size_t)n * L, op->stream));
    BDDA_CUDA(w->diagdf.ensure(sizeof(dfc) * (size_t)n, op->stream));
  }
  BDDA_CUDA(w->diag32.ensure(sizeof(float2) * (size_t)n, op->stream));
  BDDA_CUDA(w->jpre32.ensure(sizeof(float2) * (size_t)n, op->stream));
  const size_t LL = (size_t)L * L;
  BDDA_CUDA(w->gpart.ensure(sizeof(double2) * 2 * LL * gram_grid(n), op->stream));  // two Grams per CTA (gram2)
  BDDA_CUDA(w->partials.ensure(sizeof(double2) * 2 * LL, op->stream));
  BDDA_CUDA(w->partials2.ensure(sizeof(double2) * 2 * LL, op->stream));
  BDDA_CUDA(w->vpart.ensure(sizeof(double2) * 2 * (size_t)std::max(vec_grid((size_t)n * L) * L, 2 * 608), op->stream));
  BDDA_CUDA(w->small.ensure(sizeof(double2) * (LL * kNumSlots + 8), op->stream));
  BDDA_CUDA(w->ctl.ensure(sizeof(SolverCtl), op->stream));
  BDDA_CUDA(w->colf.ensure(sizeof(double) * 2 * kMaxL, op->stream));
  BDDA_CUDA(w->hist.ensure(sizeof(double) * (size_t)std::max(1, itermax), op->stream));
  w->n = n;
  w->L = L;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    auto set = [](const void* f, int b) {
      const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
      if (e != cudaSuccess) attr_err = e;
    };
    const int mx = (int)SmallSmem::bytes(kMaxL);
    set((const void*)k_small_chol1<double>, mx);
    set((const void*)k_small_chol2<double>, mx);
    set((const void*)k_small_cocg_alpha<double>, mx);
    set((const void*)k_small_cocg_beta<double>, mx);
    set((const void*)k_small_solve<double>, mx);
    set((const void*)k_small_chol1<dfl>, mx);
    set((const void*)k_small_chol2<dfl>, mx);
    set((const void*)k_small_cocg_alpha<dfl>, mx);
    set((const void*)k_small_cocg_beta<dfl>, mx);
    set((const void*)k_small_chol2_beta<double>, mx);
    set((const void*)k_small_chol2_beta<dfl>, mx);
    set((const void*)k_rowmm2<double>, rowmm_smem<double>(kMaxL, true));
    set((const void*)k_rowmm2<float>, rowmm_smem<float>(kMaxL, true));
    set((const void*)k_small_store_reduce, mx);
    set((const void*)k_rowmm<double>, rowmm_smem<double>(kMaxL, true));
    set((const void*)k_rowmm<float>, rowmm_smem<float>(kMaxL, true));
  });
  BDDA_CUDA(attr_err);
  return BDDA_OK;
}

// column norms of an FP64 block -> host (squared)
static int host_colnorm2(Op* op, cudaStream_t st, const double2* A, int n, int L, std::vector<double>* out) {
  SolverWork* w = op->solver.get();
  const int g = vec_grid((size_t)n * L);
  double* vp = w->vpart.as<double>();
  k_colnorm2<double><<<g, 256, 0, st>>>(A, n, n, L, vp);
  op->timer.count(kOther);
  std::vector<double> h((size_t)g * L);
  BDDA_CUDA(cudaMemcpyAsync(h.data(), vp, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  BDDA_CUDA(wait_stream(st));
  out->assign(L, 0.0);
  for (int p = 0; p < g; ++p)
    for (int l = 0; l < L; ++l) (*out)[l] += h[(size_t)p * L + l];
  return BDDA_OK;
}

// R = B - (diag o X + A_off X); returns max_l ||r_l|| / ||b_l||.  The product
// runs in FP64, or in double-float arithmetic when use_df is set (FP64-level
// accuracy on the FP32 pipes); the subtraction and norms are FP64.
static int true_residual(Op* op, cudaStream_t st, const double2* diag, const double2* B, int ldb, const double2* X,
                         int ldx, int n, int L, const std::vector<double>& bn2, double* resmax, int* mvps, bool use_df,
                         std::vector<double>* rn2_out = nullptr) {
  SolverWork* w = op->solver.get();
  const int gv = vec_grid((size_t)n * L);
  if (use_df) {
    k_to_df<<<gv, 256, 0, st>>>(n, L, X, ldx, w->xdf.as<dfc>(), n);
    op->timer.count(kOther);
    BDDA_TRY(op_block_mvp<dfl>(op, op->dip, w->xdf.as<dfc>(), n, w->ydf.as<dfc>(), n, L, w->diagdf.as<dfc>(), nullptr, st));
    k_from_df<<<gv, 256, 0, st>>>(n, L, w->ydf.as<dfc>(), n, w->Y64.as<double2>(), n);
    op->timer.count(kOther);
  } else {
    BDDA_TRY(op_block_mvp<double>(op, op->dip, X, ldx, w->Y64.as<double2>(), n, L, diag, nullptr, st));
  }
  ++*mvps;
  k_residual<<<gv, 256, 0, st>>>(n, L, B, ldb, w->Y64.as<double2>(), n, w->R64.as<double2>(), n);
  op->timer.count(kOther);
  std::vector<double> rn2;
  BDDA_TRY(host_colnorm2(op, st, w->R64.as<double2>(), n, L, &rn2));
  double mx = 0.0;
  for (int l = 0; l < L; ++l) {
    const double r = std::sqrt(rn2[l] / bn2[l]);
    if (!(r <= mx)) mx = r;  // NaN propagates as the maximum
  }
  *resmax = mx;
  if (rn2_out) *rn2_out = rn2;
  return BDDA_OK;
}

static int solve_impl(Op* op, const bdda_solve_opts* o, const double2* diag, const double2* B, int ldb, double2* X,
                      int ldx, int L, bdda_solve_stats* stats, cudaStream_t st) {
  const int n = op->f * op->dip.nocc;
  if (n == 0) { set_error("no dipoles set on the operator"); return BDDA_ERR_INVALID; }
  if (L < 1 || L > kMaxL) { set_error("nrhs must be 1..32"); return BDDA_ERR_INVALID; }
  if (ldb < n || ldx < n) { set_error("leading dimension smaller than f*nocc"); return BDDA_ERR_INVALID; }
  const bool mixed = o->precision == BDDA_SOLVE_MIXED;
  if (mixed && !(op->prec & BDDA_PREC_FP32)) { set_error("mixed precision needs BDDA_PREC_FP32 tables"); return BDDA_ERR_INVALID; }
  // residuals of a mixed refinement run on double-float tables when present
  const bool use_df = mixed && (op->prec & BDDA_PREC_DF64);
  if (!(op->prec & BDDA_PREC_FP64) && (!mixed || (o->true_tol > 0 && !use_df))) {
    set_error("this solve needs BDDA_PREC_FP64 tables (or BDDA_PREC_DF64 for mixed-precision residuals)");
    return BDDA_ERR_INVALID;
  }
  const bool refine = o->true_tol > 0;
  if (o->warm_start && !refine) {
    set_error("warm_start needs true_tol > 0 (refinement from the initial residual)");
    return BDDA_ERR_INVALID;
  }
  const int itermax = o->itermax > 0 ? o->itermax : 300;
  // workspace lives on the operator's stream; order it against a caller's stream
  if (st != op->stream) BDDA_CUDA(order_after(op->stream, st));
  BDDA_TRY(ensure_work(op, n, L, itermax, !mixed, mixed));
  if (st != op->stream) BDDA_CUDA(order_after(st, op->stream));
  SolverWork* w = op->solver.get();
  const int check_every = o->check_every > 0 ? o->check_every : 4;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  k_diag_prep<<<vec_grid(n), 256, 0, st>>>(n, diag, w->jpre64.as<double2>(), w->diag32.as<float2>(), w->jpre32.as<float2>());
  if (use_df) {
    k_to_df<<<vec_grid(n), 256, 0, st>>>(n, 1, diag, n, w->diagdf.as<dfc>(), n);
    op->timer.count(kOther);
  }
  op->timer.count(kOther);
  const double2* jpre64 = o->jacobi ? w->jpre64.as<double2>() : nullptr;
  const float2* jpre32 = o->jacobi ? w->jpre32.as<float2>() : nullptr;
  const bool full = !o->jacobi && o->solver == BDDA_SOLVER_COCG_RQ;  // fullPivLu only in bl_cocg_rq_mvp_fft

  Krylov<double> k64{op, w, st, n, L, diag, jpre64, check_every};
  Krylov<float> k32{op, w, st, n, L, w->diag32.as<float2>(), jpre32, check_every};
  int total_iters = 0, refinements = 0, status = BDDA_OK, mvps = 0, fp64_steps = 0;
  double last_err = 0.0, resmax = -1.0;
  // precision of the inner solves: FP32 for a mixed solve until a refinement
  // step shows that FP32 Krylov cannot make progress on this system (below)
  bool inner64 = !mixed;

  // inner solve on RHS R (FP64, leading dim ldr): the correction D is solved in
  // the inner precision into block 9 (right-hand side in block 8), then added
  // to (accumulate) or written into Dst.  With rn2 (the squared column norms of
  // R, refinement mode) the right-hand side's columns are scaled to unit norm
  // and the correction's scaled back: the block Krylov space is the same, but
  // a residual block whose columns converged to very different sizes keeps a
  // well-conditioned Gram matrix (its CholQR would otherwise break down).
  auto inner = [&](const double2* R, int ldr, double tol, double2* Dst, int ldd, bool accumulate,
                   const std::vector<double>* rn2) -> int {
    int it = 0, stt = 0;
    double er = 0.0;
    const int gv = vec_grid((size_t)n * L);
    const double* cf = nullptr;   // column scaling of the right-hand side
    const double* cfi = nullptr;  // and of the correction
    if (rn2) {
      std::vector<double> h(2 * (size_t)L);
      for (int l = 0; l < L; ++l) {
        const double nr = std::sqrt((*rn2)[l]);
        h[l] = nr > 0.0 ? 1.0 / nr : 1.0;
        h[L + l] = nr > 0.0 ? nr : 1.0;
      }
      BDDA_CUDA(cudaMemcpyAsync(w->colf.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, st));
      BDDA_CUDA(wait_stream(st));  // h is a local
      cf = w->colf.as<double>();
      cfi = cf + L;
    }
    if (inner64) {
      if (mixed) ++fp64_steps;
      double2* Bp = w->blk64[8].as<double2>();
      double2* D = w->blk64[9].as<double2>();
      if (o->jacobi) k_rowscale<double, double><<<gv, 256, 0, st>>>(n, L, w->jpre64.as<double2>(), R, ldr, Bp, n, cf);
      else k_convert<double, double><<<gv, 256, 0, st>>>(n, L, R, ldr, Bp, n, cf);
      op->timer.count(kOther);
      BDDA_TRY(k64.run(o->solver, Bp, D, full, tol, itermax, &it, &er, &stt));
      if (accumulate) k_accumulate<double><<<gv, 256, 0, st>>>(n, L, D, n, Dst, ldd, cfi);
      else k_convert<double, double><<<gv, 256, 0, st>>>(n, L, D, n, Dst, ldd, cfi);
      op->timer.count(kOther);
    } else {
      float2* Bp = w->blk32[8].as<float2>();
      float2* D = w->blk32[9].as<float2>();
      if (o->jacobi) k_rowscale<float, double><<<gv, 256, 0, st>>>(n, L, w->jpre64.as<double2>(), R, ldr, Bp, n, cf);
      else k_convert<float, double><<<gv, 256, 0, st>>>(n, L, R, ldr, Bp, n, cf);
      op->timer.count(kOther);
      // an FP32 inner solve of a refinement that has not met its tolerance after
      // kMixedInnerCap iterations (well-posed systems need tens) ends there, and
      // the refinement decides whether to continue, to switch to FP64 inner
      // solves (FP64 tables) or to report the stall (the request server then
      // solves again with FP64 tables)
      const int imax = refine ? std::min(itermax, kMixedInnerCap) : itermax;
      BDDA_TRY(k32.run(o->solver, Bp, D, full, tol, imax, &it, &er, &stt));
      if (accumulate) k_accumulate<float><<<gv, 256, 0, st>>>(n, L, D, n, Dst, ldd, cfi);
      else k_convert<double, float><<<gv, 256, 0, st>>>(n, L, D, n, Dst, ldd, cfi);
      op->timer.count(kOther);
    }
    total_iters += it;
    last_err = er;
    ++refinements;
    if (stt != 0) status = stt;
    return BDDA_OK;
  };

  if (!refine) {
    BDDA_TRY(inner(B, ldb, o->tol, X, ldx, false, nullptr));
    if (status == BDDA_OK && last_err >= o->tol) status = BDDA_ERR_NOT_CONVERGED;
  } else {
    std::vector<double> bn2;
    BDDA_TRY(host_colnorm2(op, st, B, n, L, &bn2));
    for (int l = 0; l < L; ++l)
      if (!(bn2[l] > 0.0)) { set_error("zero right-hand side column"); return BDDA_ERR_INVALID; }
    const int max_refine = o->max_refine > 0 ? o->max_refine : 8;
    // first-step inner tolerance; later steps go no tighter than ifloor, the
    // reduction one FP32 inner solve reaches before its rounding drift
    const double itol = o->inner_tol > 0 ? o->inner_tol : (mixed ? 5e-5 : 0.3 * o->true_tol);
    const double ifloor = mixed ? std::min(itol, 2e-5) : itol;
    const double2* R = B;
    int ldr = ldb;
    std::vector<double> rn2 = bn2;  // squared column norms of R
    bool converged = false;
    if (o->warm_start) {
      // X holds the initial guess (e.g. the previous wavelength's solution): refine from r = B - A X
      BDDA_TRY(true_residual(op, st, diag, B, ldb, X, ldx, n, L, bn2, &resmax, &mvps, use_df, &rn2));
      R = w->R64.as<double2>();
      ldr = n;
      converged = resmax <= o->true_tol;
      if (!(resmax < 1.0)) {  // the guess is no better than zero: start from zero
        BDDA_CUDA(cudaMemset2DAsync(X, sizeof(double2) * (size_t)ldx, 0, sizeof(double2) * (size_t)n, L, st));
        R = B;
        ldr = ldb;
        rn2 = bn2;
      }
    } else {
      BDDA_CUDA(cudaMemset2DAsync(X, sizeof(double2) * (size_t)ldx, 0, sizeof(double2) * (size_t)n, L, st));
    }
    const bool warm = o->warm_start && R != B;  // refining from a kept initial guess
    for (int r = 0; r < max_refine && !converged; ++r) {
      // Inner tolerance: itol for a cold first step; afterwards (and from a
      // warm guess) the reduction this step needs, 0.3 true_tol / residual,
      // but not tighter than ifloor (or 1e-6 from a warm guess, which lets a
      // close guess converge in one step) and not looser than 0.1.
      double tol_r = itol;
      if (r > 0 || warm) {
        const double need = std::min(0.1, 0.3 * o->true_tol / std::max(resmax, 1e-300));
        tol_r = std::max(need, (r == 0 && o->inner_tol <= 0) ? std::min(ifloor, 1e-6) : ifloor);
      }
      const double before = (r == 0 && !warm) ? 1.0 : resmax;
      BDDA_TRY(inner(R, ldr, tol_r, X, ldx, true, &rn2));
      // A breakdown (a rank-deficient residual block: its FP32 Gram loses
      // positive definiteness) ends the inner solve; its iterate is kept --
      // every kernel after the failed step returned -- and the refinement
      // restarts the Krylov solve from the true residual, as long as that
      // residual still decreases.
      const bool broke = status == BDDA_ERR_BREAKDOWN;
      if (broke) status = BDDA_OK;
      BDDA_TRY(true_residual(op, st, diag, B, ldb, X, ldx, n, L, bn2, &resmax, &mvps, use_df, &rn2));
      R = w->R64.as<double2>();
      ldr = n;
      if (resmax <= o->true_tol) { converged = true; break; }
      // A mixed solve whose FP32 inner step broke down or cut the true
      // residual less than tenfold (a system so ill-conditioned that FP32
      // Krylov stagnates: an FP32 step normally gains three to four digits)
      // runs its remaining steps with FP64 inner solves, when the operator
      // holds FP64 tables.  The FP64 Krylov blocks are allocated then.
      if (!inner64 && (broke || !(resmax < 0.1 * before)) && (op->prec & BDDA_PREC_FP64)) {
        if (st != op->stream) BDDA_CUDA(order_after(op->stream, st));
        BDDA_TRY(ensure_work(op, n, L, itermax, true, true));
        if (st != op->stream) BDDA_CUDA(order_after(st, op->stream));
        inner64 = true;
        continue;
      }
      if (broke && !(resmax < before)) { status = BDDA_ERR_BREAKDOWN; break; }
    }
    if (converged) status = BDDA_OK;  // an inner solve that hit itermax does not matter once the residual is met
    else if (status == BDDA_OK) status = BDDA_ERR_NOT_CONVERGED;
  }
  cudaEventRecord(e1, st);
  BDDA_CUDA(wait_stream(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    const int ks = take_kernel_status(op, st);  // a pipelined z pass whose copy wait gave up
    if (ks != BDDA_OK) {
      if (stats) stats->status = ks;
      return ks;
    }
  }
  if (stats) {
    stats->status = status;
    stats->iterations = total_iters;
    stats->refinements = refinements;
    stats->mvps = mvps + k64.mvps + k32.mvps;
    stats->final_err = last_err;
    stats->true_res_max = resmax;
    stats->ms_solve = ms;
    stats->fp64_inner_steps = fp64_steps;
  }
  BDDA_CUDA(cudaGetLastError());
  if (status == BDDA_ERR_BREAKDOWN) set_error("breakdown: singular L x L system, failed Cholesky or non-finite value");
  if (status == BDDA_ERR_NOT_CONVERGED) set_error("tolerance not reached within itermax / max_refine");
  return status;
}

}  // namespace bdda

using namespace bdda;

extern "C" {

void bdda_solve_opts_default(bdda_solve_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->solver = BDDA_SOLVER_COCG_RQ;
  o->jacobi = 1;
  o->precision = BDDA_SOLVE_FP64;
  o->tol = 1e-2;
  o->itermax = 300;
  o->true_tol = 0.0;
  o->inner_tol = 0.0;
  o->max_refine = 8;
  o->check_every = 4;
}

int bdda_solve_device(bdda_op* op, const bdda_solve_opts* opts, const double* diag, const double* B, int ldb, double* X,
                      int ldx, int L, bdda_solve_stats* stats, void* stream) {
  if (!op || !opts || !diag || !B || !X) { set_error("null argument"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : op->stream;
  return solve_impl(op, opts, (const double2*)diag, (const double2*)B, ldb, (double2*)X, ldx, L, stats, st);
}

int bdda_solve(bdda_op* op, const bdda_solve_opts* opts, const double* diag, const double* B, int ldb, double* X, int ldx,
               int L, bdda_solve_stats* stats) {
  if (!op || !opts || !diag || !B || !X) { set_error("null argument"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  const int n = op->f * op->dip.nocc;
  if (n == 0) { set_error("no dipoles set on the operator"); return BDDA_ERR_INVALID; }
  if (ldb < n || ldx < n || L < 1) { set_error("bad leading dimension or nrhs"); return BDDA_ERR_INVALID; }
  cudaStream_t st = op->stream;
  DevBuf d, b, x;
  BDDA_CUDA(d.ensure(sizeof(double2) * (size_t)n, op->stream));
  BDDA_CUDA(b.ensure(sizeof(double2) * (size_t)n * L, op->stream));
  BDDA_CUDA(x.ensure(sizeof(double2) * (size_t)n * L, op->stream));
  BDDA_CUDA(cudaMemcpyAsync(d.p, diag, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
  BDDA_CUDA(cudaMemcpy2DAsync(b.p, sizeof(double2) * n, B, sizeof(double2) * (size_t)ldb, sizeof(double2) * n, L,
                              cudaMemcpyHostToDevice, st));
  if (opts->warm_start)
    BDDA_CUDA(cudaMemcpy2DAsync(x.p, sizeof(double2) * n, X, sizeof(double2) * (size_t)ldx, sizeof(double2) * n, L,
                                cudaMemcpyHostToDevice, st));
  const int rc = solve_impl(op, opts, d.as<double2>(), b.as<double2>(), n, x.as<double2>(), n, L, stats, st);
  if (rc == BDDA_OK || rc == BDDA_ERR_NOT_CONVERGED) {
    BDDA_CUDA(cudaMemcpy2DAsync(X, sizeof(double2) * (size_t)ldx, x.p, sizeof(double2) * n, sizeof(double2) * n, L,
                                cudaMemcpyDeviceToHost, st));
    BDDA_CUDA(wait_stream(st));
  }
  return rc;
}

int bdda_qr_reduced(const double* A, int m, int nc, int lda, double* Q, int ldq, double* R) {
  if (!A || !Q || !R || m < 1 || nc < 1 || nc > kMaxL || lda < m || ldq < m) {
    set_error("bad qr_reduced arguments");
    return BDDA_ERR_INVALID;
  }
  Op tmp;  // bookkeeping only (stream, timer, workspace); no tables
  BDDA_CUDA(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
  keep_pool_memory();
  const cudaStream_t st = tmp.stream;
  int rc = ensure_work(&tmp, m, nc, 1, true, false);
  if (rc) return rc;
  SolverWork* w = tmp.solver.get();
  Krylov<double> kr{&tmp, w, st, m, nc, nullptr, nullptr, 4};
  double2* a = w->blk64[0].as<double2>();
  double2* q = w->blk64[1].as<double2>();
  double2* s = w->blk64[2].as<double2>();
  BDDA_CUDA(cudaMemcpy2DAsync(a, sizeof(double2) * m, A, sizeof(double2) * (size_t)lda, sizeof(double2) * m, nc,
                              cudaMemcpyHostToDevice, st));
  rc = kr.init(a, 0.0);
  if (rc != BDDA_OK) return rc;
  kr.cholqr2(a, s, q, 2);
  std::vector<double2> hr((size_t)nc * nc);
  BDDA_CUDA(cudaMemcpy2DAsync(Q, sizeof(double2) * (size_t)ldq, q, sizeof(double2) * m, sizeof(double2) * m, nc,
                              cudaMemcpyDeviceToHost, st));
  BDDA_CUDA(cudaMemcpyAsync(hr.data(), kr.sl(kXi), sizeof(double2) * hr.size(), cudaMemcpyDeviceToHost, st));
  bool done = false;
  rc = kr.poll(&done);
  if (rc != BDDA_OK) return rc;
  BDDA_CUDA(wait_stream(st));
  if (w->ctl_host->status != 0) {
    set_error("qr_reduced: rank-deficient block (Cholesky failed)");
    return BDDA_ERR_BREAKDOWN;
  }
  std::memcpy(R, hr.data(), sizeof(double2) * hr.size());
  return BDDA_OK;
}

}  // extern "C"
