// Tall-skinny block kernels for the block Krylov solvers (included by solver.cu only).
//
// Blocks are n x L column-major (the reference's Eigen layout of B, X, S, AS,
// Q ...; rows 3*m + c).  Coefficient matrices (L x L) are complex FP64,
// column-major, in global memory.  All reductions run in a fixed order (per
// CTA partials, then an ordered sum), so results are bitwise reproducible.
#pragma once

#include "common.cuh"

namespace bdda {

constexpr int kMaxL = 32;          // largest block width (nrhs) supported
constexpr int kGramThreads = 256;
constexpr int kGramRows = 32;      // rows per shared-memory sub-tile
constexpr int kRowRows = 64;       // rows per CTA of the row-transform kernel
constexpr int kRowThreads = 256;   // its threads: kRowRows rows x 4 column groups

// Device-side solver control block (lives in device memory).
struct SolverCtl {
  int done;         // 1 once the stopping test passed (all later kernels return)
  int status;       // 0 ok, 4 breakdown (singular L x L / non-finite / Cholesky)
  int iter;         // iterations completed
  int flags;
  double err;       // last recurrence error (the value the reference prints)
  double bnorm;     // ||B||_F of the (preconditioned) right-hand side
  double tol;       // stopping tolerance of the COCG-RQ recurrence error
};

__device__ __forceinline__ bool ctl_skip(const SolverCtl* ctl) {
  return ctl != nullptr && *(volatile const int*)&ctl->done != 0;
}

// Gram partial sums: complex FP64 for FP64 blocks; double-float (FP32
// instructions only -- GB300 runs FP64 at a small fraction of its FP32 rate)
// for FP32 blocks.
template <typename T> struct GramPart { using type = double2; };
template <> struct GramPart<float> { using type = dfc; };
__device__ __forceinline__ void gp_zero(double2& a) { a = make_double2(0.0, 0.0); }
__device__ __forceinline__ void gp_zero(dfc& a) { a.x = dfl(0.0f, 0.0f); a.y = dfl(0.0f, 0.0f); }
__device__ __forceinline__ void gp_add(double2& a, double2 b) { a.x += b.x; a.y += b.y; }
__device__ __forceinline__ void gp_add(double2& a, float2 b) { a.x += (double)b.x; a.y += (double)b.y; }
__device__ __forceinline__ void gp_add(dfc& a, dfc b) { a.x = a.x + b.x; a.y = a.y + b.y; }
__device__ __forceinline__ void gp_add(dfc& a, float2 b) { a.x = a.x + dfl(b.x, 0.0f); a.y = a.y + dfl(b.y, 0.0f); }
__device__ __forceinline__ double2 gp_d2(double2 a) { return a; }
__device__ __forceinline__ double2 gp_d2(dfc a) { return make_double2(df_to_double(a.x), df_to_double(a.y)); }

// ---------------------------------------------------------------------------
// Gram partials: partials[blk][i + j*L] = sum_{r in chunk} op(A[r,i]) B[r,j]
// Each CTA owns a contiguous row chunk; FP32 data is multiplied in FP32 and
// summed in FP32 over one 32-row sub-tile, then added to double-float
// accumulators (FP64 data: FP64 throughout).
// ---------------------------------------------------------------------------
// BOTH (with A == B): the Hermitian and the unconjugated Gram of A in one
// pass, partials[blk][e] = A^H A and partials[blk][LL + e] = A^T A.
template <typename T, bool CONJ, bool BOTH = false>
__global__ void __launch_bounds__(kGramThreads)
k_gram(const typename cplx<T>::type* __restrict__ A, int lda,
       const typename cplx<T>::type* __restrict__ B, int ldb,
       int n, int L, typename GramPart<T>::type* __restrict__ partials, const SolverCtl* ctl) {
  using C = typename cplx<T>::type;
  using P = typename GramPart<T>::type;
  if (ctl_skip(ctl)) return;
  __shared__ C sa[kMaxL][kGramRows + 1];
  __shared__ C sb[kMaxL][kGramRows + 1];
  const int tid = threadIdx.x;
  const int LL = L * L;
  // entries owned by this thread: e = tid + k*256, k < 4  (L <= 32 -> LL <= 1024)
  P acc[4], acc2[BOTH ? 4 : 1];
#pragma unroll
  for (int k = 0; k < 4; ++k) gp_zero(acc[k]);
#pragma unroll
  for (int k = 0; k < (BOTH ? 4 : 1); ++k) gp_zero(acc2[k]);
  const long long rows_per = ((long long)n + gridDim.x - 1) / gridDim.x;
  const long long r0 = (long long)blockIdx.x * rows_per;
  const long long r1 = min((long long)n, r0 + rows_per);
  for (long long rb = r0; rb < r1; rb += kGramRows) {
    const int nr = (int)min((long long)kGramRows, r1 - rb);
    __syncthreads();
    for (int idx = tid; idx < L * kGramRows; idx += kGramThreads) {
      const int rr = idx % kGramRows, col = idx / kGramRows;
      C va = czero<C>(), vb = czero<C>();
      if (rr < nr) {
        va = A[(size_t)col * lda + rb + rr];
        vb = B[(size_t)col * ldb + rb + rr];
      }
      sa[col][rr] = va;
      sb[col][rr] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int e = tid + k * kGramThreads;
      if (e < LL) {
        const int i = e % L, j = e / L;
        C s = czero<C>(), s2 = czero<C>();
        for (int rr = 0; rr < nr; ++rr) {
          const C a = sa[i][rr], b = sb[j][rr];
          s = CONJ ? cadd(s, cconjmul(a, b)) : cadd(s, cmul(a, b));
          if (BOTH) s2 = cadd(s2, cmul(a, b));
        }
        gp_add(acc[k], s);
        if (BOTH) gp_add(acc2[BOTH ? k : 0], s2);
      }
    }
  }
  const int LLo = BOTH ? 2 * LL : LL;  // partial entries per CTA
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int e = tid + k * kGramThreads;
    if (e < LL) {
      partials[(size_t)blockIdx.x * LLo + e] = acc[k];
      if (BOTH) partials[(size_t)blockIdx.x * LLo + LL + e] = acc2[BOTH ? k : 0];
    }
  }
}

// out[e] = sum over p of part[p*LL + e] (complex FP64 out), spread over
// ceil(LL/16) CTAs: thread group g (of 16) sums p = g, g+16, ... with two
// independent accumulators; the groups are combined in a fixed order
// (deterministic).  Sums in the partials' arithmetic (FP64 or double-float).
constexpr int kRedEntries = 16, kRedGroups = 16;
template <typename P>
__global__ void __launch_bounds__(kRedEntries * kRedGroups)
k_gram_reduce(const P* __restrict__ part, int nparts, int LL, double2* __restrict__ out, const SolverCtl* ctl) {
  if (ctl_skip(ctl)) return;
  __shared__ P red[kRedGroups][kRedEntries];
  const int el = threadIdx.x % kRedEntries, g = threadIdx.x / kRedEntries;
  const int e = blockIdx.x * kRedEntries + el;
  P acc[2];
  gp_zero(acc[0]);
  gp_zero(acc[1]);
  if (e < LL) {
    int p = g;
    for (; p + kRedGroups < nparts; p += 2 * kRedGroups) {
      const P v0 = part[(size_t)p * LL + e], v1 = part[(size_t)(p + kRedGroups) * LL + e];
      gp_add(acc[0], v0);
      gp_add(acc[1], v1);
    }
    if (p < nparts) gp_add(acc[0], part[(size_t)p * LL + e]);
  }
  gp_add(acc[0], acc[1]);
  red[g][el] = acc[0];
  __syncthreads();
  if (g == 0 && e < LL) {
    P s = red[0][el];
#pragma unroll
    for (int k = 1; k < kRedGroups; ++k) gp_add(s, red[k][el]);
    out[e] = gp_d2(s);
  }
}

// Column sums of |A[r,l]|^2 (squared column norms) -> partials[blk][l] (double)
template <typename T>
__global__ void __launch_bounds__(256)
k_colnorm2(const typename cplx<T>::type* __restrict__ A, int lda, int n, int L, double* __restrict__ partials) {
  using C = typename cplx<T>::type;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long rows_per = ((long long)n + gridDim.x - 1) / gridDim.x;
  const long long r0 = (long long)blockIdx.x * rows_per;
  const long long r1 = min((long long)n, r0 + rows_per);
  for (int l = warp; l < L; l += 8) {
    double s = 0.0;
    for (long long r = r0 + lane; r < r1; r += 32) {
      const C v = A[(size_t)l * lda + r];
      s += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) partials[(size_t)blockIdx.x * L + l] = s;
  }
}

// ---------------------------------------------------------------------------
// Row transform: Out = A*Ma [+ B*Mb] [+ Cadd]
// A CTA stages kRowRows rows of A (and B) in shared memory; thread (row,
// group) then forms the columns j = group, group + 4, ... of its row.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kRowThreads)
k_rowmm(int n, int L, const typename cplx<T>::type* A, int lda, const double2* __restrict__ Ma,
        const typename cplx<T>::type* B, int ldb, const double2* __restrict__ Mb,
        const typename cplx<T>::type* Cadd, int ldc,
        typename cplx<T>::type* Out, int ldo, const SolverCtl* ctl) {
  // Out may alias A, B or Cadd: a CTA reads its rows of A and B completely
  // before it writes, each Cadd element is read by the thread that then
  // writes it, and CTAs own disjoint rows.
  using C = typename cplx<T>::type;
  if (ctl_skip(ctl)) return;
  // dynamic smem: ta[L][kRowRows], tb[L][kRowRows], ma[L*L], mb[L*L]
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* ta = reinterpret_cast<C*>(smem_raw);
  C* tb = ta + L * kRowRows;
  C* ma = tb + (B ? L * kRowRows : 0);
  C* mb = ma + L * L;
  const int tid = threadIdx.x;
  const int LL = L * L;
  for (int e = tid; e < LL; e += kRowThreads) {
    const double2 v = Ma[e];
    ma[e] = cmake((T)v.x, (T)v.y);
    if (Mb) { const double2 w = Mb[e]; mb[e] = cmake((T)w.x, (T)w.y); }
  }
  const long long row0 = (long long)blockIdx.x * kRowRows;
  for (int e = tid; e < L * kRowRows; e += kRowThreads) {
    const int l = e / kRowRows;
    const long long r = row0 + (e - l * kRowRows);
    ta[e] = r < n ? A[(size_t)l * lda + r] : czero<C>();
    if (B) tb[e] = r < n ? B[(size_t)l * ldb + r] : czero<C>();
  }
  __syncthreads();
  const int rr = tid % kRowRows, grp = tid / kRowRows;
  const long long r = row0 + rr;
  if (r >= n) return;
  for (int j = grp; j < L; j += kRowThreads / kRowRows) {
    C acc = Cadd ? Cadd[(size_t)j * ldc + r] : czero<C>();
    for (int l = 0; l < L; ++l) acc = cadd(acc, cmul(ta[l * kRowRows + rr], ma[l + j * L]));
    if (B)
      for (int l = 0; l < L; ++l) acc = cadd(acc, cmul(tb[l * kRowRows + rr], mb[l + j * L]));
    Out[(size_t)j * ldo + r] = acc;
  }
}

// Out1 = A*Ma and Out2 = Out1 + B*Mb in one pass (Out2 may alias B).
template <typename T>
__global__ void __launch_bounds__(kRowThreads)
k_rowmm2(int n, int L, const typename cplx<T>::type* A, const double2* __restrict__ Ma,
         const typename cplx<T>::type* B, const double2* __restrict__ Mb,
         typename cplx<T>::type* Out1, typename cplx<T>::type* Out2, const SolverCtl* ctl) {
  using C = typename cplx<T>::type;
  if (ctl_skip(ctl)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* ta = reinterpret_cast<C*>(smem_raw);
  C* tb = ta + L * kRowRows;
  C* ma = tb + L * kRowRows;
  C* mb = ma + L * L;
  const int tid = threadIdx.x;
  for (int e = tid; e < L * L; e += kRowThreads) {
    const double2 v = Ma[e], w = Mb[e];
    ma[e] = cmake((T)v.x, (T)v.y);
    mb[e] = cmake((T)w.x, (T)w.y);
  }
  const long long row0 = (long long)blockIdx.x * kRowRows;
  for (int e = tid; e < L * kRowRows; e += kRowThreads) {
    const int l = e / kRowRows;
    const long long r = row0 + (e - l * kRowRows);
    ta[e] = r < n ? A[(size_t)l * n + r] : czero<C>();
    tb[e] = r < n ? B[(size_t)l * n + r] : czero<C>();
  }
  __syncthreads();
  const int rr = tid % kRowRows, grp = tid / kRowRows;
  const long long r = row0 + rr;
  if (r >= n) return;
  for (int j = grp; j < L; j += kRowThreads / kRowRows) {
    C a1 = czero<C>();
    for (int l = 0; l < L; ++l) a1 = cadd(a1, cmul(ta[l * kRowRows + rr], ma[l + j * L]));
    C a2 = a1;
    for (int l = 0; l < L; ++l) a2 = cadd(a2, cmul(tb[l * kRowRows + rr], mb[l + j * L]));
    Out1[(size_t)j * n + r] = a1;
    Out2[(size_t)j * n + r] = a2;
  }
}

template <typename T>
inline int rowmm_smem(int L, bool two) {
  return (int)sizeof(typename cplx<T>::type) * ((two ? 2 : 1) * L * kRowRows + 2 * L * L);
}

// Out = a*A + b*B (a, b complex FP64 scalars in device memory; null a -> 1; null B -> no term)
template <typename T>
__global__ void k_axpby(int n, int L, const double2* __restrict__ a, const typename cplx<T>::type* A, int lda,
                        const double2* __restrict__ b, const typename cplx<T>::type* B, int ldb,
                        typename cplx<T>::type* Out, int ldo, const SolverCtl* ctl) {
  using C = typename cplx<T>::type;
  if (ctl_skip(ctl)) return;
  const C ca = a ? cmake((T)a->x, (T)a->y) : cmake((T)1, (T)0);
  const C cb = b ? cmake((T)b->x, (T)b->y) : cmake((T)1, (T)0);
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    C v = cmul(ca, A[l * lda + r]);
    if (B) v = cadd(v, cmul(cb, B[l * ldb + r]));
    Out[l * ldo + r] = v;
  }
}

// Complex dot partials over a whole block: partials[blk] = sum conj(A) * B  (FP64)
template <typename T>
__global__ void __launch_bounds__(256)
k_dotc(int n, int L, const typename cplx<T>::type* __restrict__ A, int lda,
       const typename cplx<T>::type* __restrict__ B, int ldb, double2* __restrict__ partials, const SolverCtl* ctl) {
  using C = typename cplx<T>::type;
  if (ctl_skip(ctl)) return;
  __shared__ double2 red[8];
  const size_t total = (size_t)n * L;
  double2 s = make_double2(0.0, 0.0);
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const C a = A[l * lda + r], b = B[l * ldb + r];
    s.x += (double)a.x * (double)b.x + (double)a.y * (double)b.y;
    s.y += (double)a.x * (double)b.y - (double)a.y * (double)b.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, o);
    s.y += __shfl_down_sync(0xffffffffu, s.y, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t.x += red[w].x; t.y += red[w].y; }
    partials[blockIdx.x] = t;
  }
}

// Precision conversion / copy of an n x L block; colf (optional, FP64 [L])
// scales column l by colf[l].
template <typename TO, typename TI>
__global__ void k_convert(int n, int L, const typename cplx<TI>::type* __restrict__ in, int ldi,
                          typename cplx<TO>::type* __restrict__ out, int ldo, const double* __restrict__ colf = nullptr) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const auto v = in[l * ldi + r];
    const double f = colf ? colf[l] : 1.0;
    out[l * ldo + r] = cmake((TO)(f * (double)v.x), (TO)(f * (double)v.y));
  }
}

// complex FP64 <-> complex double-float blocks
__global__ void k_to_df(int n, int L, const double2* __restrict__ in, int ldi, dfc* __restrict__ out, int ldo) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const double2 v = in[l * ldi + r];
    out[l * ldo + r] = cmake(dfl(v.x), dfl(v.y));
  }
}
__global__ void k_from_df(int n, int L, const dfc* __restrict__ in, int ldi, double2* __restrict__ out, int ldo) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const dfc v = in[l * ldi + r];
    out[l * ldo + r] = make_double2(df_to_double(v.x), df_to_double(v.y));
  }
}

// X64 += D (D in T precision); colf (optional, FP64 [L]) scales column l of D
template <typename T>
__global__ void k_accumulate(int n, int L, const typename cplx<T>::type* __restrict__ D, int ldd,
                             double2* __restrict__ X, int ldx, const double* __restrict__ colf = nullptr) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const auto d = D[l * ldd + r];
    const double f = colf ? colf[l] : 1.0;
    double2 x = X[l * ldx + r];
    x.x += f * (double)d.x;
    x.y += f * (double)d.y;
    X[l * ldx + r] = x;
  }
}

// R = B - Y (FP64)
__global__ void k_residual(int n, int L, const double2* __restrict__ B, int ldb, const double2* __restrict__ Y, int ldy,
                           double2* __restrict__ R, int ldr) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    R[l * ldr + r] = csub(B[l * ldb + r], Y[l * ldy + r]);
  }
}

// Out = v o In   (per-row complex scaling, e.g. B_pre = jpre o B)
// (colf, optional, FP64 [L]: column l also scaled by colf[l])
template <typename TO, typename TI>
__global__ void k_rowscale(int n, int L, const double2* __restrict__ v, const typename cplx<TI>::type* __restrict__ In, int ldi,
                           typename cplx<TO>::type* __restrict__ Out, int ldo, const double* __restrict__ colf = nullptr) {
  const size_t total = (size_t)n * L;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t l = idx / n, r = idx - l * n;
    const auto a = In[l * ldi + r];
    const double f = colf ? colf[l] : 1.0;
    const double2 s = make_double2(f * v[r].x, f * v[r].y);
    const double2 p = cmul(make_double2((double)a.x, (double)a.y), s);
    Out[l * ldo + r] = cmake((TO)p.x, (TO)p.y);
  }
}

// d -> 1/d (FP64) and its FP32 copies
__global__ void k_diag_prep(int n, const double2* __restrict__ diag, double2* __restrict__ jpre64,
                            float2* __restrict__ diag32, float2* __restrict__ jpre32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 d = diag[i];
    const double den = d.x * d.x + d.y * d.y;
    const double2 j = make_double2(d.x / den, -d.y / den);
    if (jpre64) jpre64[i] = j;
    if (diag32) diag32[i] = make_float2((float)d.x, (float)d.y);
    if (jpre32) jpre32[i] = make_float2((float)j.x, (float)j.y);
  }
}

}  // namespace bdda
