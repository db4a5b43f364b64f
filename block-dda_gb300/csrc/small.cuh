// Single-CTA complex-FP64 L x L algebra for the block Krylov solvers
// (included by solver.cu only).  Matrices are column-major in shared memory,
// M[i + j*L].  Every routine is called by all kSmallThreads threads of the CTA
// and ends with a barrier.
//
// Replaces Eigen's partialPivLu / fullPivLu solves
// (bl_krylov_mvp_fft/bl_cocg_rq_mvp_fft.cpp:56,66, bl_cocg_rq_jacobi_mvp_fft.cpp:63,73,
// bl_bicgstab_mvp_fft.cpp:58-59,93, bl_bicggr_mvp_fft.cpp:51,110) and the L x L
// part of qr_reduced (qr_reduced.cpp:9-31, here as the Cholesky factors of
// CholQR2), so a whole Krylov iteration runs without a host round trip.
#pragma once

#include "common.cuh"
#include "krylov_kernels.cuh"

namespace bdda {

constexpr int kSmallThreads = 256;

__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith-free plain division; operands are O(1) pivots.
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// dst[e] = sum over p of partials[p*LL + e].  16 independent accumulators
// (partial p goes to accumulator p mod 16), combined in a fixed order: the
// loads of one round are in flight together and the result is bitwise
// reproducible for a given nparts.
__device__ void sm_reduce(double2* dst, const double2* __restrict__ partials, int nparts, int LL) {
  constexpr int U = 16;
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
    dst[e] = s;
  }
  __syncthreads();
}

__device__ void sm_copy(double2* dst, const double2* src, int LL) {
  for (int e = threadIdx.x; e < LL; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
}

// C = op(A) * B with op = transpose (TA=1) or identity (TA=0); C must not alias.
__device__ void sm_matmul(double2* Cm, const double2* A, const double2* B, int L, bool TA, double2 scale = make_double2(1.0, 0.0)) {
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) {
    const int i = e % L, j = e / L;
    double2 s = make_double2(0.0, 0.0);
    for (int k = 0; k < L; ++k) {
      const double2 a = TA ? A[k + i * L] : A[i + k * L];
      s = cadd(s, cmul(a, B[k + j * L]));
    }
    Cm[e] = cmul(s, scale);
  }
  __syncthreads();
}

// Solve A X = B (L x L, nrhs columns) by LU; A and B are overwritten (B <- X).
// full=false: partial (row) pivoting on the largest |a| in the column (first
// max); full=true: complete pivoting on the largest |a| of the trailing block,
// first max in column-major order.  Returns false on a zero / non-finite pivot.
__device__ bool sm_lu_solve(double2* A, double2* B, int L, int nrhs, bool full, int* colperm /*smem[L]*/,
                            int* piv /*smem[2]*/, double* red_v /*smem[kSmallThreads]*/, int* red_i /*smem[kSmallThreads]*/) {
  const int tid = threadIdx.x;
  for (int i = tid; i < L; i += blockDim.x) colperm[i] = i;
  __shared__ int bad;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < L; ++k) {
    // ---- pivot search by warp 0: lanes scan candidates, shuffle argmax (the
    // largest |a|, first in column-major order on ties)
    if (tid < 32) {
      const int m = L - k;
      const int cnt = full ? m * m : m;
      double best = -1.0;
      int bidx = 0x7fffffff;
      for (int t = tid; t < cnt; t += 32) {
        const int ii = k + (t % m);
        const int jj = full ? k + t / m : k;
        const double v = sqrt(cabs2(A[ii + jj * L]));
        const int lin = ii + jj * L;  // column-major order
        if (v > best || (v == best && lin < bidx)) { best = v; bidx = lin; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double v2 = __shfl_xor_sync(0xffffffffu, best, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (v2 > best || (v2 == best && i2 < bidx)) { best = v2; bidx = i2; }
      }
      if (tid == 0) {
        piv[0] = bidx % L;
        piv[1] = bidx / L;
        if (!(best > 0.0) || !isfinite(best)) bad = 1;
      }
    }
    __syncthreads();
    const int pr = piv[0], pc = piv[1];
    // ---- row swap k <-> pr (A and B)
    if (pr != k) {
      for (int j = tid; j < L + nrhs; j += blockDim.x) {
        double2* M = j < L ? A : B;
        const int jc = j < L ? j : j - L;
        const double2 t = M[k + jc * L];
        M[k + jc * L] = M[pr + jc * L];
        M[pr + jc * L] = t;
      }
    }
    __syncthreads();
    // ---- column swap k <-> pc (A only, record permutation)
    if (full && pc != k) {
      for (int i = tid; i < L; i += blockDim.x) {
        const double2 t = A[i + k * L];
        A[i + k * L] = A[i + pc * L];
        A[i + pc * L] = t;
      }
      if (tid == 0) { const int t = colperm[k]; colperm[k] = colperm[pc]; colperm[pc] = t; }
    }
    __syncthreads();
    if (bad) continue;
    // ---- multipliers (one complex division per row), then the trailing update
    const double2 p = A[k + k * L];
    const double2 pinv = cdiv(make_double2(1.0, 0.0), p);
    for (int i = k + 1 + tid; i < L; i += blockDim.x) A[i + k * L] = cmul(A[i + k * L], pinv);
    __syncthreads();
    const int rows = L - k - 1;
    for (int t = tid; t < rows * (L - k - 1 + nrhs); t += blockDim.x) {
      const int i = k + 1 + t % rows;
      const int jj = t / rows;  // 0..(L-k-2) -> A columns k+1.., then B columns
      const double2 f = A[i + k * L];
      if (jj < L - k - 1) {
        const int j = k + 1 + jj;
        A[i + j * L] = csub(A[i + j * L], cmul(f, A[k + j * L]));
      } else {
        const int j = jj - (L - k - 1);
        B[i + j * L] = csub(B[i + j * L], cmul(f, B[k + j * L]));
      }
    }
    __syncthreads();
  }
  // ---- back substitution, right-looking: row k of X is final once the rows
  // below were eliminated; then every remaining row sheds its row-k term in
  // parallel (the serial chain per row is one product per step, not L)
  for (int k = tid; k < L; k += blockDim.x) {
    const double2 inv = cdiv(make_double2(1.0, 0.0), A[k + k * L]);
    A[k + k * L] = inv;  // the diagonal now holds 1 / pivot
  }
  __syncthreads();
  for (int k = L - 1; k >= 0; --k) {
    for (int j = tid; j < nrhs; j += blockDim.x) B[k + j * L] = cmul(B[k + j * L], A[k + k * L]);
    __syncthreads();
    for (int t = tid; t < k * nrhs; t += blockDim.x) {
      const int r = t % k, j = t / k;
      B[r + j * L] = csub(B[r + j * L], cmul(A[r + k * L], B[k + j * L]));
    }
    __syncthreads();
  }
  if (full) {
    // x[colperm[k]] = y[k]; use A's first column block as scratch (A no longer needed)
    for (int e = tid; e < L * nrhs; e += blockDim.x) A[e] = B[e];
    __syncthreads();
    for (int e = tid; e < L * nrhs; e += blockDim.x) {
      const int k = e % L, j = e / L;
      B[colperm[k] + j * L] = A[e];
    }
    __syncthreads();
  }
  bool ok = !bad;
  for (int e = tid; e < L * nrhs; e += blockDim.x)
    if (!cfinite(B[e])) bad = 1;
  __syncthreads();
  ok = !bad;
  __syncthreads();
  return ok;
}

// H = R^H R with R upper triangular, real positive diagonal.  R may alias H.
// Right-looking: step k takes the square root of the (already updated)
// diagonal, scales row k and subtracts its outer product from the trailing
// block, every element in parallel.
__device__ bool sm_cholesky(double2* R, const double2* H, int L) {
  __shared__ int bad;
  __shared__ double dinv;
  const int tid = threadIdx.x;
  if (tid == 0) bad = 0;
  if (R != H) for (int e = tid; e < L * L; e += blockDim.x) R[e] = H[e];
  __syncthreads();
  for (int k = 0; k < L; ++k) {
    if (tid == 0) {
      double d = R[k + k * L].x;
      if (!(d > 0.0) || !isfinite(d)) { bad = 1; d = 1.0; }
      d = sqrt(d);
      R[k + k * L] = make_double2(d, 0.0);
      dinv = 1.0 / d;
    }
    __syncthreads();
    const double di = dinv;
    for (int j = k + 1 + tid; j < L; j += blockDim.x) {
      const double2 v = R[k + j * L];
      R[k + j * L] = make_double2(v.x * di, v.y * di);
    }
    __syncthreads();
    // trailing block (upper part, i <= j): H_ij -= conj(R_ki) R_kj
    const int m = L - k - 1;
    for (int t = tid; t < m * m; t += blockDim.x) {
      const int i = k + 1 + t % m, j = k + 1 + t / m;
      if (i <= j) R[i + j * L] = csub(R[i + j * L], cconjmul(R[k + i * L], R[k + j * L]));
    }
    __syncthreads();
  }
  // zero the strictly lower part
  for (int e = tid; e < L * L; e += blockDim.x) {
    const int i = e % L, j = e / L;
    if (i > j) R[e] = make_double2(0.0, 0.0);
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
__device__ void sm_tri_inv(double2* Ri, const double2* R, int L) {
  __shared__ double dinv[kMaxL];
  for (int i = threadIdx.x; i < L; i += blockDim.x) dinv[i] = 1.0 / R[i + i * L].x;
  for (int e = threadIdx.x; e < L * L; e += blockDim.x)
    Ri[e] = make_double2((e % L) == (e / L) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  for (int i = L - 1; i >= 0; --i) {
    for (int j = i + threadIdx.x; j < L; j += blockDim.x) {
      const double2 v = Ri[i + j * L];
      Ri[i + j * L] = make_double2(v.x * dinv[i], v.y * dinv[i]);
    }
    __syncthreads();
    // rows r < i, columns j >= i: X_rj -= R_ri X_ij
    const int nc = L - i;
    for (int t = threadIdx.x; t < i * nc; t += blockDim.x) {
      const int r = t % i, j = i + t / i;
      Ri[r + j * L] = csub(Ri[r + j * L], cmul(R[r + i * L], Ri[i + j * L]));
    }
    __syncthreads();
  }
}

// Frobenius norm (thread 0 result broadcast through smem)
__device__ double sm_fro(const double2* M, int LL) {
  __shared__ double r;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int e = 0; e < LL; ++e) s += cabs2(M[e]);
    r = sqrt(s);
  }
  __syncthreads();
  const double v = r;
  __syncthreads();
  return v;
}

}  // namespace bdda
