// Single-CTA complex L x L algebra for the block Krylov solvers (included by
// solver.cu only).  Matrices are column-major in shared memory, M[i + j*L].
// Every routine is called by all kSmallThreads threads of the CTA and ends
// with a barrier.
//
// Replaces Eigen's partialPivLu / fullPivLu solves
// (bl_krylov_mvp_fft/bl_cocg_rq_mvp_fft.cpp:56,66, bl_cocg_rq_jacobi_mvp_fft.cpp:63,73,
// bl_bicgstab_mvp_fft.cpp:58-59,93, bl_bicggr_mvp_fft.cpp:51,110) and the L x L
// part of qr_reduced (qr_reduced.cpp:9-31, here as the Cholesky factors of
// CholQR2), so a whole Krylov iteration runs without a host round trip.
//
// Two arithmetics, R: double (complex FP64, double2 matrices) for FP64
// solves, and dfl (double-float, dfc matrices, ~48-bit significand) for the
// mixed-precision inner solves, whose block vectors are FP32 -- GB300 issues
// FP32 at 64 times its FP64 rate.  Inputs (Gram partials) and the state slots
// in global memory stay complex FP64 either way.
#pragma once

#include "common.cuh"
#include "krylov_kernels.cuh"

namespace bdda {

constexpr int kSmallThreads = 256;

template <typename R> struct SmallMat;
template <> struct SmallMat<double> { using M = double2; };
template <> struct SmallMat<dfl> { using M = dfc; };

// ---- double-float reciprocal and square root --------------------------------
// The FP32 result refined by Newton steps whose residual is evaluated in
// double-float (Dekker 1971; Hida, Li and Bailey 2001, "Algorithms for
// quad-double precision floating point arithmetic").
__device__ __forceinline__ dfl df_recip(dfl b) {
  const float q1 = 1.0f / b.hi;
  const dfl one(1.0f, 0.0f);
  const dfl q = df_quick_two_sum(q1, (one - b * dfl(q1, 0.0f)).hi * q1);
  return q + dfl((one - b * q).hi * q1, 0.0f);
}
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.hi > 0.0f)) return dfl(sqrtf(a.hi), 0.0f);  // zero, negative or NaN: the FP32 answer
  const float x = sqrtf(a.hi);
  const dfl xx(x, 0.0f);
  return xx + dfl((a - xx * xx).hi * (0.5f / x), 0.0f);
}

// ---- scalar and complex helpers of the two arithmetics ---------------------
__device__ __forceinline__ double r_recip(double a) { return 1.0 / a; }
__device__ __forceinline__ dfl r_recip(dfl a) { return df_recip(a); }
__device__ __forceinline__ double r_sqrt(double a) { return sqrt(a); }
__device__ __forceinline__ dfl r_sqrt(dfl a) { return df_sqrt(a); }
__device__ __forceinline__ bool r_gt(double a, double b) { return a > b; }
__device__ __forceinline__ bool r_gt(dfl a, dfl b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool r_eq(double a, double b) { return a == b; }
__device__ __forceinline__ bool r_eq(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool r_pos_finite(double a) { return a > 0.0 && isfinite(a); }
__device__ __forceinline__ bool r_pos_finite(dfl a) { return a.hi > 0.0f && isfinite(a.hi) && isfinite(a.lo); }
__device__ __forceinline__ double r_to_double(double a) { return a; }
__device__ __forceinline__ double r_to_double(dfl a) { return df_to_double(a); }
__device__ __forceinline__ double r_shfl_xor(double a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
__device__ __forceinline__ dfl r_shfl_xor(dfl a, int o) {
  return dfl(__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o));
}
template <typename R> __device__ __forceinline__ R r_const(float v) { return R(v); }
template <> __device__ __forceinline__ dfl r_const<dfl>(float v) { return dfl(v, 0.0f); }

__device__ __forceinline__ double2 m_to_double2(double2 a) { return a; }
__device__ __forceinline__ double2 m_to_double2(dfc a) { return make_double2(df_to_double(a.x), df_to_double(a.y)); }
template <typename M> __device__ M m_from_double2(double2 a);
template <> __device__ __forceinline__ double2 m_from_double2<double2>(double2 a) { return a; }
template <> __device__ __forceinline__ dfc m_from_double2<dfc>(double2 a) { return cmake(dfl(a.x), dfl(a.y)); }

template <typename M> __device__ __forceinline__ auto m_abs2(M a) { return a.x * a.x + a.y * a.y; }
template <typename M> __device__ __forceinline__ M m_neg(M a) { return cmake(-a.x, -a.y); }
template <typename M> __device__ __forceinline__ bool m_finite(M a) {
  return isfinite(r_to_double(a.x)) && isfinite(r_to_double(a.y));
}
// a / b; operands are O(1) pivots (no scaling against overflow)
__device__ __forceinline__ double2 m_div(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ dfc m_div(dfc a, dfc b) {
  const dfl di = df_recip(b.x * b.x + b.y * b.y);
  return cmake((a.x * b.x + a.y * b.y) * di, (a.y * b.x - a.x * b.y) * di);
}
template <typename R> __device__ __forceinline__ typename SmallMat<R>::M m_one() {
  return cmake(r_const<R>(1.0f), r_const<R>(0.0f));
}

// complex FP64 helpers used outside the templated routines
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) { return m_div(a, b); }
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// dst[e] = sum over p of partials[p*LL + e] (complex FP64 partials).  16
// independent accumulators (partial p goes to accumulator p mod 16), combined
// in a fixed order: the loads of one round are in flight together and the
// result is bitwise reproducible for a given nparts.
template <typename R>
__device__ void sm_reduce(typename SmallMat<R>::M* dst, const double2* __restrict__ partials, int nparts, int LL) {
  constexpr int U = 16;
  if (nparts == 1) {  // an already reduced matrix: convert only (FP64 adds are scarce on GB300)
    for (int e = threadIdx.x; e < LL; e += blockDim.x) dst[e] = m_from_double2<typename SmallMat<R>::M>(__ldg(partials + e));
    __syncthreads();
    return;
  }
  for (int e = threadIdx.x; e < LL; e += blockDim.x) {
    double2 acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = make_double2(0.0, 0.0);
    int p = 0;
    for (; p + U <= nparts; p += U) {
      double2 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = __ldg(partials + (size_t)(p + u) * LL + e);
#pragma unroll
      for (int u = 0; u < U; ++u) { acc[u].x += v[u].x; acc[u].y += v[u].y; }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (p + u < nparts) {
        const double2 v = __ldg(partials + (size_t)(p + u) * LL + e);
        acc[u].x += v.x;
        acc[u].y += v.y;
      }
    double2 s = acc[0];
#pragma unroll
    for (int u = 1; u < U; ++u) { s.x += acc[u].x; s.y += acc[u].y; }
    dst[e] = m_from_double2<typename SmallMat<R>::M>(s);
  }
  __syncthreads();
}

template <typename M> __device__ void sm_copy(M* dst, const M* src, int LL) {
  for (int e = threadIdx.x; e < LL; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
}
// state slot (complex FP64, global) <-> shared matrix
template <typename M> __device__ void sm_load(M* dst, const double2* src, int LL) {
  for (int e = threadIdx.x; e < LL; e += blockDim.x) dst[e] = m_from_double2<M>(src[e]);
  __syncthreads();
}
template <typename M> __device__ void sm_store(double2* dst, const M* src, int LL, bool negate = false) {
  for (int e = threadIdx.x; e < LL; e += blockDim.x) dst[e] = m_to_double2(negate ? m_neg(src[e]) : src[e]);
  __syncthreads();
}

// C = op(A) * B with op = transpose (TA=1) or identity (TA=0); C must not alias.
template <typename M> __device__ void sm_matmul(M* Cm, const M* A, const M* B, int L, bool TA) {
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) {
    const int i = e % L, j = e / L;
    M s = czero<M>();
    for (int k = 0; k < L; ++k) {
      const M a = TA ? A[k + i * L] : A[i + k * L];
      s = cadd(s, cmul(a, B[k + j * L]));
    }
    Cm[e] = s;
  }
  __syncthreads();
}

// ---- teams --------------------------------------------------------------------
// The sequential L x L factorisations run on a team: the whole CTA (step
// phases separated by __syncthreads) or, for L <= kWarpL, warp 0 alone (phases
// separated by __syncwarp; the other warps wait at the routine's final
// barrier).  For small L a step's phase is a few elements per lane, so the
// CTA-wide barriers cost more than the work they separate (L = 2: 10% more
// solves per second at N=1024); at L = 16 one warp's share of the trailing
// updates (about 40 double-float elements per lane) outweighs the barriers.
constexpr int kWarpL = 8;
struct CtaTeam {
  int rank, size;
  __device__ void sync() const { __syncthreads(); }
};
struct WarpTeam {
  int rank, size;
  __device__ void sync() const { __syncwarp(); }
};

// LU solve on a team (see sm_lu_solve); *bad (shared) set on a zero /
// non-finite pivot or result.
template <typename R, class Team>
__device__ void lu_solve_team(const Team tm, typename SmallMat<R>::M* A, typename SmallMat<R>::M* B, int L, int nrhs,
                              bool full, int* colperm, int* piv, int* bad) {
  using M = typename SmallMat<R>::M;
  const int tid = tm.rank, nt = tm.size;
  for (int i = tid; i < L; i += nt) colperm[i] = i;
  tm.sync();
  for (int k = 0; k < L; ++k) {
    // ---- pivot search by the first 32 ranks: lanes scan candidates, shuffle
    // argmax (the largest |a|, first in column-major order on ties); |a|^2
    // orders the candidates as |a| does, without a square root
    if (tid < 32) {
      const int m = L - k;
      const int cnt = full ? m * m : m;
      R best = r_const<R>(-1.0f);
      int bidx = 0x7fffffff;
      for (int t = tid; t < cnt; t += 32) {
        const int ii = k + (t % m);
        const int jj = full ? k + t / m : k;
        const R v = m_abs2(A[ii + jj * L]);
        const int lin = ii + jj * L;  // column-major order
        if (r_gt(v, best) || (r_eq(v, best) && lin < bidx)) { best = v; bidx = lin; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R v2 = r_shfl_xor(best, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (r_gt(v2, best) || (r_eq(v2, best) && i2 < bidx)) { best = v2; bidx = i2; }
      }
      if (tid == 0) {
        piv[0] = bidx % L;
        piv[1] = bidx / L;
        if (!r_pos_finite(best)) *bad = 1;
      }
    }
    tm.sync();
    const int pr = piv[0], pc = piv[1];
    // ---- row swap k <-> pr (A and B)
    if (pr != k) {
      for (int j = tid; j < L + nrhs; j += nt) {
        M* Mt = j < L ? A : B;
        const int jc = j < L ? j : j - L;
        const M t = Mt[k + jc * L];
        Mt[k + jc * L] = Mt[pr + jc * L];
        Mt[pr + jc * L] = t;
      }
    }
    if (full) tm.sync();  // the row and the column swap share elements
    // ---- column swap k <-> pc (A only, record permutation)
    if (full && pc != k) {
      for (int i = tid; i < L; i += nt) {
        const M t = A[i + k * L];
        A[i + k * L] = A[i + pc * L];
        A[i + pc * L] = t;
      }
      if (tid == 0) { const int t = colperm[k]; colperm[k] = colperm[pc]; colperm[pc] = t; }
    }
    tm.sync();
    if (*bad) continue;
    // ---- multipliers (one complex division per row), then the trailing update
    const M pinv = m_div(m_one<R>(), A[k + k * L]);
    for (int i = k + 1 + tid; i < L; i += nt) A[i + k * L] = cmul(A[i + k * L], pinv);
    tm.sync();
    const int rows = L - k - 1;
    for (int t = tid; t < rows * (L - k - 1 + nrhs); t += nt) {
      const int i = k + 1 + t % rows;
      const int jj = t / rows;  // 0..(L-k-2) -> A columns k+1.., then B columns
      const M f = A[i + k * L];
      if (jj < L - k - 1) {
        const int j = k + 1 + jj;
        A[i + j * L] = csub(A[i + j * L], cmul(f, A[k + j * L]));
      } else {
        const int j = jj - (L - k - 1);
        B[i + j * L] = csub(B[i + j * L], cmul(f, B[k + j * L]));
      }
    }
    tm.sync();
  }
  // ---- back substitution, right-looking: row k of X is final once the rows
  // below were eliminated; then every remaining row sheds its row-k term in
  // parallel (the serial chain per row is one product per step, not L)
  for (int k = tid; k < L; k += nt) A[k + k * L] = m_div(m_one<R>(), A[k + k * L]);
  tm.sync();  // the diagonal now holds 1 / pivot
  for (int k = L - 1; k >= 0; --k) {
    for (int j = tid; j < nrhs; j += nt) B[k + j * L] = cmul(B[k + j * L], A[k + k * L]);
    tm.sync();
    for (int t = tid; t < k * nrhs; t += nt) {
      const int r = t % k, j = t / k;
      B[r + j * L] = csub(B[r + j * L], cmul(A[r + k * L], B[k + j * L]));
    }
    tm.sync();
  }
  if (full) {
    // x[colperm[k]] = y[k]; use A as scratch (A no longer needed)
    for (int e = tid; e < L * nrhs; e += nt) A[e] = B[e];
    tm.sync();
    for (int e = tid; e < L * nrhs; e += nt) {
      const int k = e % L, j = e / L;
      B[colperm[k] + j * L] = A[e];
    }
    tm.sync();
  }
  for (int e = tid; e < L * nrhs; e += nt)
    if (!m_finite(B[e])) *bad = 1;
}

// Solve A X = B (L x L, nrhs columns) by LU; A and B are overwritten (B <- X).
// full=false: partial (row) pivoting on the largest |a| in the column (first
// max); full=true: complete pivoting on the largest |a| of the trailing block,
// first max in column-major order.  Returns false on a zero / non-finite pivot.
template <typename R>
__device__ bool sm_lu_solve(typename SmallMat<R>::M* A, typename SmallMat<R>::M* B, int L, int nrhs, bool full,
                            int* colperm /*smem[L]*/, int* piv /*smem[2]*/) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  if (L <= kWarpL) {
    if (threadIdx.x < 32) lu_solve_team<R>(WarpTeam{(int)threadIdx.x, 32}, A, B, L, nrhs, full, colperm, piv, &bad);
  } else {
    lu_solve_team<R>(CtaTeam{(int)threadIdx.x, (int)blockDim.x}, A, B, L, nrhs, full, colperm, piv, &bad);
  }
  __syncthreads();
  const bool ok = !bad;
  __syncthreads();
  return ok;
}

// Right-looking Cholesky on a team (see sm_cholesky), in place on Rm.  Every
// rank takes the square root and reciprocal of the pivot itself (no broadcast
// phase); rank 0 writes the diagonal after all ranks have read it.
template <typename R, class Team>
__device__ void cholesky_team(const Team tm, typename SmallMat<R>::M* Rm, int L, int* bad) {
  using M = typename SmallMat<R>::M;
  const int tid = tm.rank, nt = tm.size;
  for (int k = 0; k < L; ++k) {
    R d = Rm[k + k * L].x;
    if (!r_pos_finite(d)) { if (tid == 0) *bad = 1; d = r_const<R>(1.0f); }
    d = r_sqrt(d);
    const R di = r_recip(d);
    tm.sync();
    if (tid == 0) Rm[k + k * L] = cmake(d, r_const<R>(0.0f));
    for (int j = k + 1 + tid; j < L; j += nt) {
      const M v = Rm[k + j * L];
      Rm[k + j * L] = cmake(v.x * di, v.y * di);
    }
    tm.sync();
    // trailing block (upper part, i <= j): H_ij -= conj(R_ki) R_kj
    const int m = L - k - 1;
    for (int t = tid; t < m * m; t += nt) {
      const int i = k + 1 + t % m, j = k + 1 + t / m;
      if (i <= j) Rm[i + j * L] = csub(Rm[i + j * L], cconjmul(Rm[k + i * L], Rm[k + j * L]));
    }
    tm.sync();
  }
}

// H = R^H R with R upper triangular, real positive diagonal.  R may alias H.
// Right-looking: step k takes the square root of the (already updated)
// diagonal, scales row k and subtracts its outer product from the trailing
// block, every element in parallel.
template <typename R>
__device__ bool sm_cholesky(typename SmallMat<R>::M* Rm, const typename SmallMat<R>::M* H, int L) {
  using M = typename SmallMat<R>::M;
  __shared__ int bad;
  const int tid = threadIdx.x;
  if (tid == 0) bad = 0;
  if (Rm != H) for (int e = tid; e < L * L; e += blockDim.x) Rm[e] = H[e];
  __syncthreads();
  if (L <= kWarpL) {
    if (tid < 32) cholesky_team<R>(WarpTeam{tid, 32}, Rm, L, &bad);
  } else {
    cholesky_team<R>(CtaTeam{tid, (int)blockDim.x}, Rm, L, &bad);
  }
  __syncthreads();
  // zero the strictly lower part
  for (int e = tid; e < L * L; e += blockDim.x) {
    const int i = e % L, j = e / L;
    if (i > j) Rm[e] = czero<M>();
  }
  __syncthreads();
  const bool ok = !bad;
  __syncthreads();
  return ok;
}

// Inverse of an upper triangular matrix with a real positive diagonal (the
// Cholesky factors): R X = I solved bottom-up, right-looking -- row i of X is
// final after scaling by 1 / R_ii, then the rows above shed their row-i term,
// all elements in parallel.
template <typename R>
__device__ void sm_tri_inv(typename SmallMat<R>::M* Ri, const typename SmallMat<R>::M* Rm, int L) {
  using M = typename SmallMat<R>::M;
  __shared__ R dinv[kMaxL];
  for (int i = threadIdx.x; i < L; i += blockDim.x) dinv[i] = r_recip(Rm[i + i * L].x);
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) Ri[e] = (e % L) == (e / L) ? m_one<R>() : czero<M>();
  __syncthreads();
  auto run = [&](auto tm) {
    for (int i = L - 1; i >= 0; --i) {
      for (int j = i + tm.rank; j < L; j += tm.size) {
        const M v = Ri[i + j * L];
        Ri[i + j * L] = cmake(v.x * dinv[i], v.y * dinv[i]);
      }
      tm.sync();
      // rows r < i, columns j >= i: X_rj -= R_ri X_ij
      const int nc = L - i;
      for (int t = tm.rank; t < i * nc; t += tm.size) {
        const int r = t % i, j = i + t / i;
        Ri[r + j * L] = csub(Ri[r + j * L], cmul(Rm[r + i * L], Ri[i + j * L]));
      }
      tm.sync();
    }
  };
  if (L <= kWarpL) {
    if (threadIdx.x < 32) run(WarpTeam{(int)threadIdx.x, 32});
  } else {
    run(CtaTeam{(int)threadIdx.x, (int)blockDim.x});
  }
  __syncthreads();
}

// Frobenius norm in FP64 (any scale): per-thread sums of |m|^2, a warp
// shuffle tree, then the warps' sums in order (deterministic).
template <typename R> __device__ double sm_fro(const typename SmallMat<R>::M* Mm, int LL) {
  __shared__ double wsum[kSmallThreads / 32];
  __shared__ double r;
  double s = 0.0;
  for (int e = threadIdx.x; e < LL; e += blockDim.x) s += cabs2(m_to_double2(Mm[e]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = wsum[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    r = sqrt(t);
  }
  __syncthreads();
  const double v = r;
  __syncthreads();
  return v;
}

}  // namespace bdda
