// Operator lifecycle and MVP entry points of the C ABI.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bdda.h"
#include "op.hpp"

#include <mutex>

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

#define BDDA_TRY_CUDA(call) BDDA_CUDA(call)

// Make stream 'later' wait for everything enqueued so far on 'earlier'.
cudaError_t order_after(cudaStream_t later, cudaStream_t earlier) {
  cudaEvent_t ev;
  cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  e = cudaEventRecord(ev, earlier);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(later, ev, 0);
  cudaEventDestroy(ev);
  return e;
}

cudaError_t wait_stream(cudaStream_t st) {
  thread_local cudaEvent_t ev = nullptr;
  if (ev == nullptr) {
    const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming);
    if (e != cudaSuccess) { ev = nullptr; return e; }
  }
  cudaError_t e = cudaEventRecord(ev, st);
  if (e != cudaSuccess) return e;
  return cudaEventSynchronize(ev);
}

static int smooth235(int v) {
  for (;; ++v) {
    int t = v;
    for (int p : {2, 3, 5})
      while (t % p == 0) t /= p;
    if (t == 1) return v;
  }
}

void keep_pool_memory() {
  static bool done[64] = {};
  static std::mutex mu;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = true;
}

Op::~Op() {
  // release every stream-ordered buffer on the operator's stream before it goes away
  solver.reset();
  for (auto* o : {&dip, &cub}) { o->occ.release(); o->tiles.release(); o->tmask.release(); }
  for (int i = 0; i < 3; ++i) {
    tw64[i].release(); tw32[i].release(); twdf[i].release(); tw32p[i].release(); tws32[i].release();
  }
  tws32p.release(); twsdf.release();
  ghat64.release(); ghat32.release(); ghatdf.release();
  kstat.release();
  for (int i = 0; i < 3; ++i) { t1[i].release(); t2[i].release(); }
  if (stream) {
    wait_stream(stream);
    cudaStreamDestroy(stream);
  }
}

int take_kernel_status(Op* op, cudaStream_t st) {
  if (!op->kstat.p) return BDDA_OK;
  int h = 0;
  BDDA_CUDA(cudaMemcpyAsync(&h, op->kstat.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  BDDA_CUDA(wait_stream(st));
  if (h == 0) return BDDA_OK;
  BDDA_CUDA(cudaMemsetAsync(op->kstat.p, 0, sizeof(int), st));
  BDDA_CUDA(wait_stream(st));
  set_error("z pass: a wait on a bulk copy to shared memory gave up after 2 s (results invalid)");
  return BDDA_ERR_CUDA;
}

int build_occupancy(Op* op, const int* address, int nocc, Occupancy* o) {
  const int nx = op->n[0], ny = op->n[1], nz = op->n[2];
  const int nzt = (nz + kTZ - 1) / kTZ;
  const size_t nc = (size_t)nx * ny * nz;
  std::vector<int> occ(nc, -1);
  std::vector<unsigned char> tmask((size_t)ny * nzt, 0);
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
    const long long iy = (a / nz) % ny, iz = a % nz;
    tmask[iy * nzt + iz / kTZ] = 1;
  }
  std::vector<int> tiles;
  long long rows = 0;
  for (int t = 0; t < ny * nzt; ++t)
    if (tmask[t]) {
      tiles.push_back(t);
      const int z0 = (t % nzt) * kTZ;
      rows += std::min(kTZ, nz - z0);
    }
  o->nocc = nocc;
  o->ntiles = (int)tiles.size();
  o->tile_rows = rows;
  BDDA_CUDA(o->occ.ensure(nc * sizeof(int), op->stream));
  BDDA_CUDA(o->tmask.ensure(tmask.size(), op->stream));
  BDDA_CUDA(o->tiles.ensure(std::max<size_t>(1, tiles.size()) * sizeof(int), op->stream));
  BDDA_CUDA(cudaMemcpyAsync(o->occ.p, occ.data(), nc * sizeof(int), cudaMemcpyHostToDevice, op->stream));
  BDDA_CUDA(cudaMemcpyAsync(o->tmask.p, tmask.data(), tmask.size(), cudaMemcpyHostToDevice, op->stream));
  if (!tiles.empty())
    BDDA_CUDA(cudaMemcpyAsync(o->tiles.p, tiles.data(), tiles.size() * sizeof(int), cudaMemcpyHostToDevice, op->stream));
  BDDA_CUDA(wait_stream(op->stream));  // host vectors die on return
  return BDDA_OK;
}

// Measured choice of the tile passes' launch schedule for a complex FP32 block
// MVP of L columns (the FFT schedules: y-pass grid waves, scalar or packed z
// pass, x-pass CTAs per SM).  Each candidate is launched alone on the
// operator's own workspace -- pass A reads x and writes T1, B reads T1 and
// writes T2, C works in place on T2, so re-running them is harmless -- three
// times with CUDA events, and the fastest is kept.  Runs once per operator and
// nrhs, outside stream capture, for workspaces of at least kTuneMinBytes (below
// that the MVP is bound by launch latency and the defaults are kept); a
// process-wide table keyed by the geometry lets later operators of the same
// box, occupancy and nrhs skip the measurement.
constexpr size_t kTuneMinBytes = 64ull << 20;

static std::mutex g_tune_mu;
static std::map<std::string, Op::TuneRec> g_tune_cache;

static std::string tune_key(const MvpGeom& g, int L) {
  return std::to_string(g.f) + ":" + std::to_string(g.nx) + "," + std::to_string(g.ny) + "," + std::to_string(g.nz) +
         ":" + std::to_string(g.ntiles) + ":" + std::to_string(g.tile_rows) + ":" + std::to_string(L);
}

static cudaError_t autotune_f32(MvpGeom g, const MvpPrec<float>& p, const float2* x, int ldx, int L, float2* t1,
                                float2* t2, cudaStream_t st, Op::TuneRec* out) {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  auto timed = [&](unsigned passes, const MvpTune& t, float* ms) -> cudaError_t {
    g.tune = t;
    g.passes = passes;
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaError_t r = cudaEventRecord(a, st);
      if (r == cudaSuccess) r = launch_block_mvp<float>(g, p, x, ldx, nullptr, ldx, L, nullptr, nullptr, t1, t2, st,
                                                        nullptr, nullptr);
      if (r == cudaSuccess) r = cudaEventRecord(b, st);
      if (r == cudaSuccess) r = cudaEventSynchronize(b);
      float t_ms = 0.f;
      if (r == cudaSuccess) r = cudaEventElapsedTime(&t_ms, a, b);
      if (r != cudaSuccess) return r;
      best = std::min(best, t_ms);
    }
    *ms = best;
    return cudaSuccess;
  };
  Op::TuneRec rec{};
  for (float& v : rec.ms) v = -1.f;
  MvpTune t;  // defaults
  float dummy = 0.f;
  if (e == cudaSuccess) e = timed(1u, t, &dummy);  // pass A fills T1
  const int yw[4] = {2, 4, 8, 16};
  int best = -1;
  for (int i = 0; i < 8 && e == cudaSuccess; ++i) {  // y pass: buffers 1, 2 x waves 2, 4, 8, 16
    MvpTune c = t;
    c.ybuf = 1 + i / 4;
    c.ywaves = yw[i % 4];
    e = timed(2u, c, &rec.ms[i]);
    if (e == cudaSuccess && (best < 0 || rec.ms[i] < rec.ms[best])) best = i;
  }
  if (e == cudaSuccess) {
    t.ybuf = 1 + best / 4;
    t.ywaves = yw[best % 4];
  }
  {  // pass C: scalar, packed and pipelined kernels where they run this geometry
    const bool packed = packed_z_available(g.Pz, g.f) && p.twzps;
    const bool pipe = pipe_z_available(g.Pz, g.f, g.nzp, L);
    if (e == cudaSuccess && (packed || pipe)) {
      MvpTune c = t;
      c.zkern = 0;
      e = timed(4u, c, &rec.ms[8]);
      int kbest = 0;
      float mbest = rec.ms[8];
      if (e == cudaSuccess && packed) {
        c.zkern = 1;
        e = timed(4u, c, &rec.ms[9]);
        if (e == cudaSuccess && rec.ms[9] < mbest) { kbest = 1; mbest = rec.ms[9]; }
      }
      if (e == cudaSuccess && pipe) {
        c.zkern = 2;
        e = timed(4u, c, &rec.ms[13]);
        if (e == cudaSuccess && rec.ms[13] < mbest) { kbest = 2; mbest = rec.ms[13]; }
      }
      if (e == cudaSuccess) t.zkern = kbest;
    }
  }
  best = -1;
  for (int i = 0; i < 8 && e == cudaSuccess; ++i) {  // inverse y pass (D, reads T2): its own buffers and waves
    MvpTune c = t;
    c.ybufd = 1 + i / 4;
    c.ywavesd = yw[i % 4];
    e = timed(8u, c, &rec.ms[14 + i]);
    if (e == cudaSuccess && (best < 0 || rec.ms[14 + i] < rec.ms[14 + best])) best = i;
  }
  if (e == cudaSuccess) {
    t.ybufd = 1 + best / 4;
    t.ywavesd = yw[best % 4];
  }
  const int xc[3] = {5, 10, 20};
  best = -1;
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
    MvpTune c = t;
    c.xcta = xc[i];
    e = timed(1u, c, &rec.ms[10 + i]);
    if (e == cudaSuccess && (best < 0 || rec.ms[10 + i] < rec.ms[10 + best])) best = i;
  }
  if (e == cudaSuccess) t.xcta = xc[best];
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  rec.tune = t;
  rec.measured = e == cudaSuccess;
  *out = rec;
  return e;
}

template <typename T>
int op_block_mvp(Op* op, const Occupancy& o, const typename cplx<T>::type* x, int ldx, typename cplx<T>::type* y, int ldy,
                 int L, const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre, cudaStream_t st,
                 const int* done) {
  using C = typename cplx<T>::type;
  const int pi = PrecInfo<T>::slot;
  const int need = PrecInfo<T>::bit;
  if (!(op->prec & need)) {
    set_error("operator was created without the tables of this precision");
    return BDDA_ERR_INVALID;
  }
  if (L < 1 || ldx < op->f * o.nocc || ldy < op->f * o.nocc) {
    set_error("bad L or leading dimension");
    return BDDA_ERR_INVALID;
  }
  MvpGeom g = op->geom<T>(o);
  const bool grow = op->t1[pi].bytes < mvp_t1_elems(g, L) * sizeof(C) || op->t2[pi].bytes < mvp_t2_elems(g, L) * sizeof(C);
  if (grow && st != op->stream) BDDA_TRY_CUDA(order_after(op->stream, st));  // old buffers may be in use on st
  BDDA_CUDA(op->t1[pi].ensure(mvp_t1_elems(g, L) * sizeof(C), op->stream));
  BDDA_CUDA(op->t2[pi].ensure(mvp_t2_elems(g, L) * sizeof(C), op->stream));
  if (grow && st != op->stream) BDDA_TRY_CUDA(order_after(st, op->stream));  // new buffers exist before st uses them
  // the kernels' arithmetic: dfz (unrenormalised) for the double-float tables
  using A = typename MvpArith<T>::type;
  using CA = typename cplx<A>::type;
  static_assert(sizeof(CA) == sizeof(C), "storage layouts agree");
  const MvpPrec<T> tb = op->tables<T>();
  MvpPrec<A> ta{(const CA*)tb.twx, (const CA*)tb.twy, (const CA*)tb.twz, (const CA*)tb.ghat, tb.twzp,
                (const CA*)tb.twxs, (const CA*)tb.twys, (const CA*)tb.twzs, tb.twzps};
  if constexpr (std::is_same<T, float>::value) {
    auto it = op->tuned.find(L);
    if (it != op->tuned.end()) {
      g.tune = it->second.tune;
    } else if (op->autotune && &o == &op->dip && mvp_t2_elems(g, L) * sizeof(C) >= kTuneMinBytes) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      BDDA_CUDA(cudaStreamIsCapturing(st, &cs));
      if (cs == cudaStreamCaptureStatusNone) {
        const std::string key = tune_key(g, L);
        Op::TuneRec rec{};
        bool have = false;
        {
          std::lock_guard<std::mutex> lk(g_tune_mu);
          auto c = g_tune_cache.find(key);
          if (c != g_tune_cache.end()) { rec = c->second; have = true; }
        }
        if (!have) {
          BDDA_CUDA(autotune_f32(g, ta, x, ldx, L, op->t1[pi].as<float2>(), op->t2[pi].as<float2>(), st, &rec));
          std::lock_guard<std::mutex> lk(g_tune_mu);
          g_tune_cache[key] = rec;
        }
        op->tuned[L] = rec;
        g.tune = rec.tune;
      }
    }
    if (op->zkern_force >= 0) g.tune.zkern = op->zkern_force;
  }
  cudaError_t e = launch_block_mvp<A>(g, ta, (const CA*)x, ldx, (CA*)y, ldy, L, (const CA*)diag, (const CA*)jpre,
                                      op->t1[pi].as<CA>(), op->t2[pi].as<CA>(), st, &op->timer, done);
  if (e != cudaSuccess) return cuda_fail(e, "block MVP launch");
  return BDDA_OK;
}

template int op_block_mvp<double>(Op*, const Occupancy&, const double2*, int, double2*, int, int, const double2*,
                                  const double2*, cudaStream_t, const int*);
template int op_block_mvp<float>(Op*, const Occupancy&, const float2*, int, float2*, int, int, const float2*,
                                 const float2*, cudaStream_t, const int*);
template int op_block_mvp<dfl>(Op*, const Occupancy&, const dfc*, int, dfc*, int, int, const dfc*, const dfc*,
                               cudaStream_t, const int*);

}  // namespace bdda

using namespace bdda;

// Green spectra of the operator's box, spacing and f at wavenumber k (FP64
// evaluation and transform; packed for every precision the operator holds).
static int build_spectrum(Op* op, double k_re, double k_im) {
  const int f = op->f, prec = op->prec;
  const double lf = op->lf;
  const int Px = op->P[0], Py = op->P[1], Pz = op->P[2];
  const size_t ng = (size_t)Px * Py * Pz;
  DevBuf work;
  const size_t nc = f == 6 ? 9 : 6;  // Green components (symmetric A; f = 6 adds antisymmetric B)
  BDDA_CUDA(work.ensure(nc * ng * sizeof(double2), op->stream));
  if (prec & BDDA_PREC_FP64) BDDA_CUDA(op->ghat64.ensure(nc * ng * sizeof(double2), op->stream));
  if (prec & BDDA_PREC_FP32) BDDA_CUDA(op->ghat32.ensure(nc * ng * sizeof(float2), op->stream));
  if (prec & BDDA_PREC_DF64) BDDA_CUDA(op->ghatdf.ensure(nc * ng * sizeof(dfc), op->stream));
  // one spectrum per distinct digit order (radix sequences) of the plan sets
  bool same = true;
  for (int i = 0; i < 3; ++i) {
    const AxisPlan &a = op->plan[0][i], &b = op->plan[1][i];
    same = same && a.nst == b.nst && std::equal(a.radix, a.radix + a.nst, b.radix);
  }
  const double2 *tx = op->tw64[0].as<double2>(), *ty = op->tw64[1].as<double2>(), *tz = op->tw64[2].as<double2>();
  const int gperm = green_perm_radix(f, op->plan[0][2]);  // FP32 / double-float spectra for the fused z pass
  BDDA_CUDA(build_green_hat(op->geom(op->dip, 1), lf, k_re, k_im, tx, ty, tz, work.as<double2>(),
                            op->ghat64.as<double2>(), same ? op->ghat32.as<float2>() : nullptr,
                            op->ghatdf.as<dfc>(), gperm, op->stream));
  if (!same && op->ghat32.p)
    BDDA_CUDA(build_green_hat(op->geom(op->dip, 0), lf, k_re, k_im, tx, ty, tz, work.as<double2>(), nullptr,
                              op->ghat32.as<float2>(), nullptr, gperm, op->stream));
  BDDA_CUDA(wait_stream(op->stream));
  op->kr = k_re;
  op->ki = k_im;
  return BDDA_OK;
}

extern "C" {

const char* bdda_last_error(void) { return bdda::last_error(); }

int bdda_op_create(bdda_op** out, const int n[3], int f, double lf, double k_re, double k_im, int prec) {
  if (!out || !n) { set_error("null argument"); return BDDA_ERR_INVALID; }
  *out = nullptr;
  if (f != 3 && f != 6) { set_error("unknown f value (3 or 6)"); return BDDA_ERR_INVALID; }
  if ((prec & (BDDA_PREC_FP64 | BDDA_PREC_FP32 | BDDA_PREC_DF64)) == 0) {
    set_error("no precision requested");
    return BDDA_ERR_INVALID;
  }
  for (int i = 0; i < 3; ++i)
    if (n[i] < 1 || n[i] > kMaxLine / 2) {
      set_error("lattice box dimension outside 1.." + std::to_string(kMaxLine / 2));
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
    // z lines: the fused pass (three lines per warp); x / y: the tile passes
    if (!make_axis_plan(op->P[i], &op->plan[0][i], i == 2, false) ||
        !make_axis_plan(op->P[i], &op->plan[1][i], i == 2, true)) {
      set_error("no FFT plan for the padded grid");
      return BDDA_ERR_INVALID;
    }
  }
  BDDA_CUDA(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  BDDA_CUDA(op->kstat.ensure(sizeof(int), op->stream));
  BDDA_CUDA(cudaMemsetAsync(op->kstat.p, 0, sizeof(int), op->stream));
  keep_pool_memory();
  // twiddles
  for (int i = 0; i < 3; ++i) {
    std::vector<double2> tw;
    make_twiddles(op->P[i], &tw);
    BDDA_CUDA(op->tw64[i].ensure(tw.size() * sizeof(double2), op->stream));
    BDDA_CUDA(cudaMemcpyAsync(op->tw64[i].p, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice, op->stream));
    std::vector<float2> tf(tw.size());
    for (size_t t = 0; t < tw.size(); ++t) tf[t] = make_float2((float)tw[t].x, (float)tw[t].y);
    BDDA_CUDA(op->tw32[i].ensure(tf.size() * sizeof(float2), op->stream));
    BDDA_CUDA(cudaMemcpyAsync(op->tw32[i].p, tf.data(), tf.size() * sizeof(float2), cudaMemcpyHostToDevice, op->stream));
    std::vector<float4> tp(tw.size());
    for (size_t t = 0; t < tw.size(); ++t) tp[t] = make_float4(tf[t].x, tf[t].x, tf[t].y, tf[t].y);
    if (i == 2 && !std::getenv("BDDA_NO_PACK")) {
      BDDA_CUDA(op->tw32p[i].ensure(tp.size() * sizeof(float4), op->stream));
      BDDA_CUDA(cudaMemcpyAsync(op->tw32p[i].p, tp.data(), tp.size() * sizeof(float4), cudaMemcpyHostToDevice, op->stream));
    }
    std::vector<dfc> td(tw.size());
    for (size_t t = 0; t < tw.size(); ++t) td[t] = cmake(dfl(tw[t].x), dfl(tw[t].y));
    BDDA_CUDA(op->twdf[i].ensure(td.size() * sizeof(dfc), op->stream));
    BDDA_CUDA(cudaMemcpyAsync(op->twdf[i].p, td.data(), td.size() * sizeof(dfc), cudaMemcpyHostToDevice, op->stream));
    // staged tables of the complex FP32 compile-time-plan kernels (plan set 0)
    std::vector<double2> ts;
    stage_twiddles(op->plan[0][i], &ts);
    const size_t nts = std::max<size_t>(ts.size(), 1);
    std::vector<float2> tsf(nts, make_float2(1.f, 0.f));
    std::vector<float4> tsp(nts, make_float4(1.f, 1.f, 0.f, 0.f));
    for (size_t t = 0; t < ts.size(); ++t) {
      tsf[t] = make_float2((float)ts[t].x, (float)ts[t].y);
      tsp[t] = make_float4(tsf[t].x, tsf[t].x, tsf[t].y, tsf[t].y);
    }
    // the double-float z pass runs the 16-byte z table's plan (plan set 1)
    std::vector<double2> tsw;
    stage_twiddles(op->plan[1][i], &tsw);
    const size_t ntw = std::max<size_t>(tsw.size(), 1);
    std::vector<dfc> tsd(ntw, cmake(dfl(1.0), dfl(0.0)));
    for (size_t t = 0; t < tsw.size(); ++t) tsd[t] = cmake(dfl(tsw[t].x), dfl(tsw[t].y));
    BDDA_CUDA(op->tws32[i].ensure(nts * sizeof(float2), op->stream));
    BDDA_CUDA(cudaMemcpyAsync(op->tws32[i].p, tsf.data(), nts * sizeof(float2), cudaMemcpyHostToDevice, op->stream));
    if (i == 2) {
      BDDA_CUDA(op->tws32p.ensure(nts * sizeof(float4), op->stream));
      BDDA_CUDA(cudaMemcpyAsync(op->tws32p.p, tsp.data(), nts * sizeof(float4), cudaMemcpyHostToDevice, op->stream));
      BDDA_CUDA(op->twsdf.ensure(ntw * sizeof(dfc), op->stream));
      BDDA_CUDA(cudaMemcpyAsync(op->twsdf.p, tsd.data(), ntw * sizeof(dfc), cudaMemcpyHostToDevice, op->stream));
    }
    BDDA_CUDA(wait_stream(op->stream));  // tw / tf / ts die at the end of this iteration
  }
  {
    // kernel attributes sized for the largest line, so every live operator fits; once per process
    static std::once_flag once;
    static cudaError_t cfg = cudaSuccess;
    std::call_once(once, [] {
      cfg = configure_mvp_kernels<double>();
      if (cfg == cudaSuccess) cfg = configure_mvp_kernels<float>();
      if (cfg == cudaSuccess) cfg = configure_mvp_kernels<dfz>();
    });
    BDDA_CUDA(cfg);
  }
  {
    const int rc = build_spectrum(op.get(), k_re, k_im);
    if (rc != BDDA_OK) return rc;
  }
  BDDA_CUDA(wait_stream(op->stream));
  *out = op.release();
  return BDDA_OK;
}

int bdda_op_set_wavenumber(bdda_op* op, double k_re, double k_im) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  BDDA_CUDA(cudaStreamSynchronize(op->stream));  // no MVP of the old spectrum may still be running
  return build_spectrum(op, k_re, k_im);
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
  ++op->dip_epoch;
  return build_occupancy(op, address, nocc, &op->dip);
}

int bdda_op_info(const bdda_op* op, int P[3], int* nocc, int* ntiles) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  if (P) for (int i = 0; i < 3; ++i) P[i] = op->P[i];
  if (nocc) *nocc = op->dip.nocc;
  if (ntiles) *ntiles = op->dip.ntiles;
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
  const size_t nrow = (size_t)op->f * op->cub.nocc;
  DevBuf x, y;
  BDDA_CUDA(x.ensure(nrow * sizeof(double2), op->stream));
  BDDA_CUDA(y.ensure(nrow * sizeof(double2), op->stream));
  BDDA_CUDA(cudaMemcpyAsync(x.p, p_hat, nrow * sizeof(double2), cudaMemcpyHostToDevice, op->stream));
  int rc = op_block_mvp<double>(op, op->cub, x.as<double2>(), (int)nrow, y.as<double2>(), (int)nrow, 1, nullptr, nullptr,
                                op->stream);
  if (rc) return rc;
  BDDA_CUDA(cudaMemcpyAsync(q_hat, y.p, nrow * sizeof(double2), cudaMemcpyDeviceToHost, op->stream));
  BDDA_CUDA(wait_stream(op->stream));
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
  if (prec == BDDA_PREC_DF64)
    return op_block_mvp<dfl>(op, op->dip, (const dfc*)x, ldx, (dfc*)y, ldy, L, (const dfc*)diag, (const dfc*)jpre, st);
  set_error("prec must be BDDA_PREC_FP64, BDDA_PREC_FP32 or BDDA_PREC_DF64");
  return BDDA_ERR_INVALID;
}

int bdda_op_mvp_bytes(const bdda_op* op, int prec, int L, int with_diag, int with_jpre, double bytes[5]) {
  if (!op || !bytes || L < 1 || (prec != BDDA_PREC_FP64 && prec != BDDA_PREC_FP32)) {
    set_error("bad mvp_bytes arguments");
    return BDDA_ERR_INVALID;
  }
  const double s = prec == BDDA_PREC_FP64 ? 16.0 : 8.0;
  const double F = (double)op->f * L;                     // fields
  const double nc = op->f == 6 ? 9.0 : 6.0;               // Green components
  const double nocc = op->dip.nocc;
  const double nx = op->n[0], nz = op->n[2], Px = op->P[0], Py = op->P[1], Pz = op->P[2];
  const double rows = (double)op->dip.tile_rows;          // (y, z) columns of occupied tiles
  const double t1 = F * Px * rows * s;                    // x-transformed rows of those tiles
  const double t2 = F * Px * Py * nz * s;                 // y-transformed planes
  const double vec = F * nocc * s;                        // one compact block
  const double occ = nx * rows * 4.0;                     // occupancy of the tiles
  const double ghat = nc * Px * Py * Pz * s;
  bytes[0] = vec + occ + t1;
  bytes[1] = t1 + t2;
  bytes[2] = 2.0 * t2 + ghat;
  bytes[3] = t2 + t1;
  bytes[4] = t1 + occ + vec + (with_diag ? vec + op->f * nocc * s : 0.0) + (with_jpre ? op->f * nocc * s : 0.0);
  return BDDA_OK;
}

int bdda_op_set_graphs(bdda_op* op, int on) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->graphs = on != 0;
  return BDDA_OK;
}

int bdda_op_set_autotune(bdda_op* op, int on) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->autotune = on != 0;
  op->tuned.clear();
  return BDDA_OK;
}

int bdda_op_get_tuning(bdda_op* op, int L, int schedule[6], float candidate_ms[22]) {
  if (!op || !schedule) { set_error("null argument"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  const MvpTune def;
  auto it = op->tuned.find(L);
  const MvpTune& t = it != op->tuned.end() ? it->second.tune : def;
  schedule[0] = t.ywaves;
  schedule[1] = t.ybuf;
  schedule[2] = t.zkern;
  schedule[3] = t.xcta;
  schedule[4] = t.ywavesd > 0 ? t.ywavesd : t.ywaves;
  schedule[5] = t.ybufd > 0 ? t.ybufd : t.ybuf;
  if (candidate_ms)
    for (int i = 0; i < 22; ++i) candidate_ms[i] = it != op->tuned.end() ? it->second.ms[i] : -1.f;
  return it != op->tuned.end() && it->second.measured ? BDDA_OK : BDDA_ERR_NOT_CONVERGED;
}

int bdda_op_set_timing(bdda_op* op, int enable) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->timer.enabled = enable != 0;
  op->timer.mask = enable == 2 ? (1u << kPassC) | (1u << kPassC64) : ~0u;
  return BDDA_OK;
}

int bdda_op_set_z_kernel(bdda_op* op, int kind) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  if (kind < -1 || kind > 2) { set_error("z kernel must be -1 (default), 0 scalar, 1 packed or 2 pipelined"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->zkern_force = kind;
  return BDDA_OK;
}

int bdda_op_test_z_stall(bdda_op* op, int on) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  op->zstall = on != 0;
  return BDDA_OK;
}

int bdda_op_check_status(bdda_op* op) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  return take_kernel_status(op, op->stream);
}

int bdda_op_kernel_stats(bdda_op* op, double* ms, long long* launches, int n, int reset) {
  if (!op) { set_error("null operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  wait_stream(op->stream);
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
