// Internal interfaces of the block-MVP kernels (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "common.cuh"

namespace bdda {

// z-tile width of the strided passes (8 lines per CTA, one warp each):
// rows of 8 x c64 = 64 B or 8 x c128 = 128 B.
constexpr int kTZ = 8;
constexpr int kTileThreads = kTZ * 32;
// Warps per CTA of the fused z pass (one (x, y, rhs) task each), at most.
constexpr int kZWarps = 8;
// The fused z pass (f = 3) runs its last forward stage, the Green product and
// its first inverse stage in one sweep (sfft::middle3 / pk::middle3) when the
// z plan has two or more stages and a last radix Rl <= kFusedMaxRadix (fused_z); a
// thread then takes the Rl adjacent frequencies b Rl .. b Rl + Rl - 1 of a
// butterfly b, so the complex FP32 Green spectrum of such operators is stored
// last-radix-major (frequency b Rl + i at i (Pz / Rl) + b): the lanes' loads
// of one component are then adjacent (coalesced).  With the complex FP32 z
// table's first-stage radices up to 32, most lengths are two stages with a
// fused last radix (250 = 25 x 10, 243 = 27 x 9, 270 = 27 x 10): the first
// stage reads T2 and writes shared memory, the fused step reads and writes it
// once, the last inverse stage reads it and writes T2.  Shorter lines (below
// kFusedWideMinN points, the packed-pair kernel's range) keep plans of radices
// <= 16 and fuse only up to radix 5, the packed kernel's limit
// (zpacked::supported).
constexpr int kFusedMaxRadix = 10;
constexpr int kFusedMaxRadixShort = 5;
constexpr int kFusedWideMinN = 181;
BDDA_HD constexpr bool fused_z(int N, int nst, int rl) {
  return nst >= 2 && (rl <= kFusedMaxRadixShort || (rl <= kFusedMaxRadix && N >= kFusedWideMinN));
}
// (complex FP32 only: the double-float fused step needs 168 registers and ran
// slower than the separate stages, 54.9 vs 41.6 ms per N=65536, L=32 pass.)
inline int green_perm_radix(int f, const AxisPlan& pz) {
  return (f == 3 && fused_z(pz.N, pz.nst, pz.radix[pz.nst - 1])) ? pz.radix[pz.nst - 1] : 0;
}
BDDA_HD int green_pos(int p, int N, int rl) { return rl ? (p % rl) * (N / rl) + p / rl : p; }

// Dynamic shared memory one CTA may take (227 KB).
constexpr int kZSmemMax = 227 * 1024;
// Warps per CTA of the z pass when each warp needs per_warp bytes of lines.
inline int z_warps_per_cta(int per_warp) {
  const int w = kZSmemMax / (per_warp > 0 ? per_warp : 1);
  return w < 1 ? 1 : (w > kZWarps ? kZWarps : w);
}

// Launch schedule of a block MVP's tile passes, chosen per operator and nrhs
// by the autotuner (op.cu: candidates timed with CUDA events on the operator's
// own buffers) or left at the defaults.
struct MvpTune {
  // pass C kernel: -1 the default rule (pipelined where the plan and shared memory allow, else packed where
  // three 8-warp CTAs fit, else scalar), 0 scalar, 1 packed, 2 pipelined (zpass_pipe.cuh)
  int zkern = -1;
  int ywaves = 4;    // passes B, D: grid of this many waves of the CTAs resident per SM
  int ybuf = 2;      // passes B, D: tile buffers per CTA (2: prefetch the next task; 1: twice the CTAs)
  int ybufd = 0;     // pass D's own buffers and waves when > 0 (the autotuner times it separately)
  int ywavesd = 0;
  int xcta = 10;     // passes A, E: aim at this many CTAs per SM (fields split into groups)
};

// Geometry shared by both precisions (device pointers).
struct MvpGeom {
  int f;                       // components per dipole: 3 (E) or 6 (E, M)
  int nx, ny, nz;
  int nzp;                     // row pitch of T1 / T2 along z: nz rounded up to a multiple of 4
  int Px, Py, Pz;
  AxisPlan px, py, pz;
  int nzt;                     // ceil(nz / kTZ)
  int gperm;                   // Green spectrum layout along z: 0 natural (ghat[.][c][p]); else the z plan's
                               // last radix Rl, ghat[.][c][(p % Rl) (Pz / Rl) + p / Rl] (see fused_z)
  MvpTune tune;                // launch schedule of the tile passes
  unsigned passes = 0x1fu;     // passes launched (bit 0 = A .. bit 4 = E); the autotuner times them one by one
  int ntiles;                  // (y, z-tile) pairs holding >= 1 dipole
  long long tile_rows;         // sum over those tiles of their valid z count
  int* kstat = nullptr;        // status word of the pipelined z pass (1: a bounded copy wait gave up)
  int zstall = 0;              // test hook: the pipelined z pass gives up one wait (bdda_op_test_z_stall)
  const int* occ;              // [nx*ny*nz] dipole index or -1
  const int* tiles;            // [ntiles]  y*nzt + zt
  const unsigned char* tmask;  // [ny*nzt]  1 for those tiles
};

// Precision-specific tables (device pointers).
template <typename T> struct MvpPrec {
  using C = typename cplx<T>::type;
  const C* twx;
  const C* twy;
  const C* twz;
  const C* ghat;  // [Px][Py][6 or 9][Pz] (digit-reversed frequencies), divided by Px*Py*Pz
  const float4* twzp = nullptr;  // complex FP32: z twiddle pairs {wx, wx, wy, wy} (packed z pass)
  // staged tables (stage_twiddles) of the compile-time-plan kernels: x, y, z
  // (complex FP32), z pairs (packed z pass), z (double-float z pass)
  const C* twxs = nullptr;
  const C* twys = nullptr;
  const C* twzs = nullptr;
  const float4* twzps = nullptr;
};

// Timed kernel classes: the five MVP passes per precision (FP32 first), then
// the Krylov block kernels.
enum KernelId {
  kPassA = 0, kPassB, kPassC, kPassD, kPassE,            // complex FP32 MVP
  kPassA64, kPassB64, kPassC64, kPassD64, kPassE64,       // complex FP64 MVP
  kGram, kUpdate, kSmall, kOther,
  kNumKernelIds
};

// Optional per-kernel CUDA-event timing (accumulated when resolved).
// Launch counts and timed event pairs of kernels launched while a stream was
// captured into a graph: the graph's event-record nodes re-record the same
// events at every replay, and the timer adds the record once per replay.
struct TimerRec {
  struct Pair { int id; cudaEvent_t a, b; };
  long long counts[kNumKernelIds] = {0};
  std::vector<Pair> pairs;
  std::vector<cudaEvent_t> owned;
  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    owned.push_back(e);
    return e;
  }
  void clear() {
    for (auto e : owned) cudaEventDestroy(e);
    owned.clear();
    pairs.clear();
    for (auto& c : counts) c = 0;
  }
  TimerRec() = default;
  TimerRec(const TimerRec&) = delete;
  TimerRec& operator=(const TimerRec&) = delete;
  ~TimerRec() { clear(); }
};

struct KernelTimer {
  struct Pending { int id; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  double ms[kNumKernelIds] = {0};
  long long launches[kNumKernelIds] = {0};
  cudaEvent_t cur_a[kNumKernelIds] = {};
  bool enabled = false;
  unsigned mask = ~0u;      // kernel classes timed while enabled (bit per KernelId)
  TimerRec* rec = nullptr;  // set while the launching stream is captured into a graph

  cudaEvent_t get() {
    if (rec) return rec->event();
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  }
  void record(cudaEvent_t e, cudaStream_t st) {
    if (rec) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);  // an event-record node of the graph
    else cudaEventRecord(e, st);
  }
  void count(int id, int k = 1) { (rec ? rec->counts[id] : launches[id]) += k; }
  bool on(int id) const { return enabled && ((mask >> id) & 1u); }
  unsigned state() const { return enabled ? mask : 0u; }
  void begin(int id, cudaStream_t st) {
    count(id);
    if (!on(id)) return;
    cur_a[id] = get();
    record(cur_a[id], st);
  }
  void end(int id, cudaStream_t st) {
    if (!on(id)) return;
    cudaEvent_t b = get();
    record(b, st);
    if (rec) rec->pairs.push_back({id, cur_a[id], b});
    else pending.push_back({id, cur_a[id], b});
  }
  // Call after the stream was synchronised.
  void resolve() {
    for (auto& p : pending) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ms[p.id] += t;
      pool.push_back(p.a); pool.push_back(p.b);
    }
    pending.clear();
  }
  // One replay of a graph recorded into r has completed (stream synchronised).
  void replayed(const TimerRec& r) {
    for (int i = 0; i < kNumKernelIds; ++i) launches[i] += r.counts[i];
    for (auto& p : r.pairs) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ms[p.id] += t;
    }
  }
  void reset() {
    resolve();
    for (int i = 0; i < kNumKernelIds; ++i) { ms[i] = 0; launches[i] = 0; }
  }
  ~KernelTimer() {
    for (auto& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Workspace elements (complex T) the MVP needs for L right-hand sides.
inline size_t mvp_t1_elems(const MvpGeom& g, int L) { return (size_t)g.f * L * g.Px * g.ny * g.nzp; }
inline size_t mvp_t2_elems(const MvpGeom& g, int L) { return (size_t)g.f * L * g.Px * g.Py * g.nzp; }

template <typename T>
cudaError_t launch_block_mvp(const MvpGeom& g, const MvpPrec<T>& p, const typename cplx<T>::type* x, int ldx,
                             typename cplx<T>::type* y, int ldy, int L,
                             const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre,
                             typename cplx<T>::type* t1, typename cplx<T>::type* t2,
                             cudaStream_t st, KernelTimer* timer, const int* done = nullptr);

template <typename T> cudaError_t configure_mvp_kernels();

// Arguments of the strided passes of one complex FP32 block MVP.
struct TileArgs {
  const MvpGeom* g;
  const float2* x;
  int ldx;
  float2* y;
  int ldy;
  int nfield;
  const float2* diag;
  const float2* jpre;
  float2* t1;
  float2* t2;
  const float2* twx;
  const float2* twy;
  int sms;              // multiprocessors of the device
  cudaStream_t st;
  const int* done;
};
enum TilePass { kTileA = 0, kTileB, kTileD, kTileE };

// Grid of the y passes (B, D), whose CTAs take tasks (field, x, z tile) in a
// fixed stride: by default four waves of the CTAs resident per SM
// (MvpTune::ywaves).  Measured on the
// column-pair passes (N=16384 / 8192, tasks of uneven cost: empty rows are
// skipped): one exact wave 0.244 / 0.146 ms (forward), two 0.239 / 0.138,
// four 0.233 / 0.135; the earlier fixed 8 CTAs per SM (1.1-1.6 waves) 0.239 /
// 0.159.
constexpr int kYWaves = 4;

// Fields per CTA of the x passes (A, E), an even number: a tile's fields are
// split over groups of CTAs so that a launch has about xcta CTAs per
// multiprocessor (default 10: two waves of five; one CTA per tile left most
// of the GPU idle: 301 tiles at N=8192).  Returns the number of groups.
inline int x_field_groups(int nfield, int ntiles, int sms, int* fpg, int xcta = 10) {
  const int pairs = (nfield + 1) / 2;
  const int want = (xcta * sms + ntiles - 1) / ntiles;
  const int groups = want < 1 ? 1 : (want < pairs ? want : pairs);
  *fpg = 2 * ((pairs + groups - 1) / groups);
  return (nfield + *fpg - 1) / *fpg;
}

// Strided pass `pass` for complex FP32 with the compile-time plan of its axis
// (tplans.inc: Px for A / E; yplans.inc: Py for B / D); false (nothing launched) when the
// length has none.  *err: launch status.
bool launch_tile_static(int pass, const TileArgs& a, cudaError_t* err);

// Pass C for complex FP32 with the compile-time z plan of g.Pz (zplans.inc);
// returns false (nothing launched) when g.Pz has none.  With twzp (the z
// twiddle pair table {wx, wx, wy, wy}) and f = 3 the packed-pair kernel runs.
// *err: launch status.
bool launch_pass_c_static(const MvpGeom& g, float2* t2, int L, const float2* twz, const float4* twzp, const float2* ghat,
                          cudaStream_t st, const int* done, cudaError_t* err);

// Whether the packed-pair pass C can run for z length Pz and f (an autotuner
// candidate besides the scalar kernel).
bool packed_z_available(int Pz, int f);
// Whether the pipelined z pass (zpass_pipe.cuh) can run this geometry at nrhs
// L (an autotuner candidate; the default rule also wants two CTAs per SM).
bool pipe_z_available(int Pz, int f, int nzp, int L);

// Pass C of a double-float block MVP (f = 3) with the compile-time z plan of
// g.Pz; false (nothing launched) when g.Pz has none or f = 6.
bool launch_pass_c_static_df(const MvpGeom& g, dfzc* t2, int L, const dfzc* twz, const dfzc* ghat, cudaStream_t st,
                             const int* done, cudaError_t* err);

// Green tensor: build Ghat (FP64 evaluation + FP64 3-D FFT), layout
// [Px][Py][nc][Pz] with nc = 6 (g.f = 3) or 9 (g.f = 6), for any of the
// precisions (null pointers skipped); the complex FP32 output in the z layout
// gperm (green_pos), the others natural.  work: c128 [nc*Px*Py*Pz].
cudaError_t build_green_hat(const MvpGeom& g, double lf, double k_re, double k_im,
                            const double2* twx, const double2* twy, const double2* twz,
                            double2* work, double2* ghat_d, float2* ghat_f, dfc* ghat_df, int gperm, cudaStream_t st);

// Radix schedule and shared-memory layout for a 5-smooth 2 <= N <= kMaxLine.
// three: the fused z pass (three lines per warp), else the single-line tile
// passes.  wide = false (complex FP32): the radix sequence of the compile-time
// plan tables (zplans.inc / tplans.inc); wide = true (16-byte FP64 and
// double-float): the z table's sequence, and for the tile passes the radices
// 2, 3, 4, 5, 8 with the fewest stages in the order a shared-memory bank model
// prefers.  The skew shift and line pitch of both element widths come from the
// same bank model (cached per plan).
bool make_axis_plan(int N, AxisPlan* p, bool three, bool wide);
// FP64 twiddle table exp(-2 pi i t / N), t < N.
void make_twiddles(int N, std::vector<double2>* out);
// Staged twiddle table of a plan, for the compile-time-plan kernels: stage s
// (butterfly span M_s, radix R_s, table stride N / (M_s R_s)) holds
// w^(k n1 N / (M_s R_s)) at offset_s + (k - 1) M_s + n1 for k = 1 .. R_s - 1,
// n1 < M_s, offset_s = sum over t < s of (R_t - 1) M_t (sfft::Plan::TWO).
// k-major, so adjacent butterflies of a stage read adjacent entries.
void stage_twiddles(const AxisPlan& p, std::vector<double2>* out);

}  // namespace bdda
