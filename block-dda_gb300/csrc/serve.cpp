// Request server and batched solves: many targets of uneven size and nrhs on
// one GPU, admitted by device-memory footprint and run concurrently.
//
// Replaces the reference's sequential wavelength x target loop
// (block_DDA_main.cpp:138-163: one target at a time, full re-initialisation
// per target, no overlap).  Each admitted request gets its own operator
// (Green spectrum of its box and wavenumber), its own stream and its own
// Krylov workspace, all resident in HBM until the request completes; worker
// slots run requests concurrently so that small targets fill the GPU together.
//
// Admission: requests are considered in arrival order; the head of the queue
// is admitted as soon as its footprint fits in the memory budget.  A later
// request that fits may start before a head that does not, but at most
// kMaxBypass times per head request, so large requests cannot starve.  A
// request whose footprint exceeds the whole budget is rejected at submission.
//
// Results do not depend on the mix: every solve uses only its own buffers and
// fixed-order reductions, so a request computes bitwise the same X alone or
// among others.
//
// Spectrum cache: a finished request's operator -- its Green spectra, plans and
// workspaces, resident in HBM -- is kept idle, keyed by (box, f, lattice
// spacing, wavenumber, precision), and the next request with the same key
// takes it instead of rebuilding the spectrum (only its dipoles are set
// again).  Idle operators count against the memory budget and against a
// cache limit (a quarter of the budget unless set); the least recently used
// are destroyed when an admission needs their memory.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bdda.h"

namespace bdda {
void set_error(const std::string& msg);
}

namespace {

constexpr int kMaxBypass = 8;
constexpr int kMaxBoxSide = 600;  // bdda_op_create's limit: half the longest FFT line (kMaxLine)

int smooth235(int v) {
  for (;; ++v) {
    int t = v;
    for (int p : {2, 3, 5})
      while (t % p == 0) t /= p;
    if (t == 1) return v;
  }
}

// Device bytes of one request of f components per dipole: Green spectra (6
// or 9 components; FP64 or FP32 + double-float), the initialisation's FP64
// work grid, occupancy, MVP workspace of both precisions, Krylov blocks.
double footprint_bytes(const int n[3], int nocc, int L, int precision, int f) {
  const double Px = smooth235(2 * n[0]), Py = smooth235(2 * n[1]), Pz = smooth235(2 * n[2]);
  const double Ng = Px * Py * Pz;
  const double nc = (double)n[0] * n[1] * n[2];
  const bool mixed = precision == BDDA_SOLVE_MIXED;
  const double ncomp = f == 6 ? 9.0 : 6.0;
  const double tables = ncomp * Ng * (16.0 + (mixed ? 8.0 : 0.0));
  const double init_work = ncomp * Ng * 16.0;
  const double occ = nc * 4.0 + (double)n[1] * ((n[2] + 7) / 8) * 5.0;
  const double nzp = (double)((n[2] + 3) & ~3);
  const double t1 = (double)f * L * Px * n[1] * nzp, t2 = (double)f * L * Px * Py * nzp;
  const double mvp = (t1 + t2) * (16.0 + (mixed ? 8.0 : 0.0));
  const double nu = (double)f * nocc, LL = (double)L * L;
  const double blocks = 10.0 * nu * L * (mixed ? 8.0 : 16.0) + 3.0 * nu * L * 16.0 + nu * 32.0;
  const double small = 2.0 * LL * 152.0 * 16.0 + 2.0 * std::max(608.0 * L, 1216.0) * 16.0 + LL * 16.0 * 20.0 + 8.0 * 4096;
  const double io = nu * 16.0 + 2.0 * nu * L * 16.0;
  const double peak = std::max(tables + init_work + occ, tables + occ + mvp + blocks + small + io);
  return peak * 1.05 + 8.0 * (1 << 20);
}

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct bdda_server {
  // Operator kept idle after its request, with the device bytes it holds.
  struct OpKey {
    int n[3], f, prec;
    double lf, kr, ki;
    bool operator==(const OpKey& o) const {
      return n[0] == o.n[0] && n[1] == o.n[1] && n[2] == o.n[2] && f == o.f && prec == o.prec && lf == o.lf &&
             kr == o.kr && ki == o.ki;
    }
  };
  struct Cached {
    OpKey key;
    bdda_op* op;
    double bytes;
    unsigned long long tick;
  };
  struct Item {
    bdda_request req;
    long long ticket;
    double footprint;
    double t_submit;
    int bypassed = 0;
    bool exclusive = false;  // ran out of device memory once: runs again with nothing else on the GPU
  };

  int slots;
  double budget;
  bdda_solve_opts opts;
  bool dry;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Item> pending;
  std::unordered_map<long long, bdda_request_result> done;
  double in_use = 0, peak_in_use = 0;
  int running = 0, peak_running = 0;
  long long completed = 0, next_ticket = 1;
  bool stopping = false;
  std::vector<std::thread> threads;
  std::vector<Cached> idle;            // idle operators (spectrum cache)
  double cache_limit = 0, cache_bytes = 0;
  unsigned long long tick = 0;
  long long spectra_reused = 0, spectra_built = 0;
  bool solo = false;  // an exclusive request is running: nothing else is admitted

  // Take an idle operator with this key out of the cache (caller holds mu).
  bool take_cached(const OpKey& k, Cached* out) {
    for (size_t i = 0; i < idle.size(); ++i)
      if (idle[i].key == k) {
        *out = idle[i];
        idle.erase(idle.begin() + i);
        cache_bytes -= out->bytes;
        in_use -= out->bytes;
        return true;
      }
    return false;
  }
  // Remove the least recently used idle operator (caller holds mu; the caller
  // destroys it after releasing mu).
  bdda_op* evict_lru() {
    size_t j = 0;
    for (size_t i = 1; i < idle.size(); ++i)
      if (idle[i].tick < idle[j].tick) j = i;
    bdda_op* op = idle[j].op;
    cache_bytes -= idle[j].bytes;
    in_use -= idle[j].bytes;
    idle.erase(idle.begin() + j);
    return op;
  }
  // pick(), destroying idle operators (into *ev) while the head of the queue
  // does not fit (caller holds mu).
  int pick_evicting(std::vector<bdda_op*>* ev) {
    if (!pending.empty() && pending.front().exclusive && running == 0)
      while (!idle.empty()) ev->push_back(evict_lru());  // all of the device for it
    for (;;) {
      const int i = pick();
      if (i >= 0 || idle.empty() || pending.empty()) return i;
      ev->push_back(evict_lru());
    }
  }

  // Express slots: extra workers that take only small requests (footprint up
  // to kExpressBytes), so that a queue held up by long solves of large
  // targets still serves the many small ones.
  static constexpr double kExpressBytes = 2e9;
  // index of the first small request that fits, or -1 (caller holds mu)
  int pick_express() const {
    if (solo || (!pending.empty() && pending.front().exclusive)) return -1;
    for (size_t i = 0; i < pending.size(); ++i)
      if (pending[i].footprint <= kExpressBytes && in_use + pending[i].footprint <= budget) {
        // passing a head that waits for memory counts as a bypass, and is limited likewise
        const bool head_waits = i > 0 && in_use + pending.front().footprint > budget;
        return (head_waits && pending.front().bypassed >= kMaxBypass) ? -1 : (int)i;
      }
    return -1;
  }

  // index of the request to admit now, or -1 (caller holds mu)
  int pick() const {
    if (pending.empty() || solo) return -1;
    if (pending.front().exclusive)  // waits for every running request to finish, then runs alone
      return (running == 0 && in_use + pending.front().footprint <= budget) ? 0 : -1;
    if (in_use + pending.front().footprint <= budget) return 0;
    if (pending.front().bypassed >= kMaxBypass) return -1;
    for (size_t i = 1; i < pending.size(); ++i)
      if (in_use + pending[i].footprint <= budget) return (int)i;
    return -1;
  }

  // Runs one admitted request; *reserved is the memory it holds while it runs
  // (its footprint, or more when it takes a cached operator grown by an
  // earlier, larger request).  Returns the operator to keep idle, or null.
  bdda_op* execute(const Item& it, bdda_request_result* res, const OpKey& key, double* reserved) {
    const bdda_request& r = it.req;
    if (dry) {
      // no device work: hold the slot for a time proportional to the footprint
      std::this_thread::sleep_for(std::chrono::microseconds((long long)(it.footprint / 1e6 * 200.0) + 200));
      res->status = BDDA_OK;
      return nullptr;
    }
    bdda_op* op = nullptr;
    Cached c{};
    bool reused = false;
    if (it.exclusive) {
      // return the stream-ordered pool's cached free memory to the device, so
      // that the request's large buffers are not refused for fragmentation
      int dev = 0;
      cudaMemPool_t pool;
      if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        cudaDeviceSynchronize();  // nothing else runs: an exclusive request waits for the others
        cudaMemPoolTrimTo(pool, 0);
      }
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      if (take_cached(key, &c)) {
        reused = true;
        op = c.op;
        const double extra = std::max(0.0, c.bytes - *reserved);  // the operator may hold more than this request needs
        in_use += extra;
        peak_in_use = std::max(peak_in_use, in_use);
        *reserved += extra;
        ++spectra_reused;
      } else {
        ++spectra_built;
      }
    }
    const int f = key.f;
    int rc = BDDA_OK;
    if (!reused) {
      rc = bdda_op_create(&op, r.n, f, r.lf, r.k_re, r.k_im, key.prec);
      // concurrent requests keep the GPU busy between one stream's launches, so
      // captured poll cycles save nothing here and cost their capture (batched
      // workload: 245 vs 251 RHS-solves/s with and without them)
      if (rc == BDDA_OK) rc = bdda_op_set_graphs(op, 0);
      // one solve per operator: measuring its FFT schedule would cost more than it saves
      if (rc == BDDA_OK) rc = bdda_op_set_autotune(op, 0);
    }
    if (rc == BDDA_OK) rc = bdda_op_set_dipoles(op, r.address, r.nocc);
    bdda_solve_stats st{};
    if (rc == BDDA_OK) rc = bdda_solve(op, &opts, r.diag, r.B, f * r.nocc, r.X, f * r.nocc, r.L, &st);
    if ((rc == BDDA_ERR_BREAKDOWN || rc == BDDA_ERR_NOT_CONVERGED) && opts.precision == BDDA_SOLVE_MIXED &&
        !(key.prec & BDDA_PREC_FP64)) {
      // A mixed solve that broke down or stagnated on FP32 Krylov: solve again
      // in FP64 on an operator with FP64 tables, starting from the mixed
      // solve's iterate (the solver restarts from zero if that is no better;
      // the operator is not cached: its key would not match later requests')
      bdda_op_destroy(op);
      op = nullptr;
      rc = bdda_op_create(&op, r.n, f, r.lf, r.k_re, r.k_im, BDDA_PREC_FP64);
      if (rc == BDDA_OK) rc = bdda_op_set_graphs(op, 0);
      if (rc == BDDA_OK) rc = bdda_op_set_autotune(op, 0);
      if (rc == BDDA_OK) rc = bdda_op_set_dipoles(op, r.address, r.nocc);
      bdda_solve_opts o64 = opts;
      o64.precision = BDDA_SOLVE_FP64;
      o64.warm_start = 1;
      bdda_solve_stats st2{};
      if (rc == BDDA_OK) rc = bdda_solve(op, &o64, r.diag, r.B, f * r.nocc, r.X, f * r.nocc, r.L, &st2);
      st2.iterations += st.iterations;
      st2.refinements += st.refinements;
      st = st2;
      res->retried_fp64 = 1;
      if (op) bdda_op_destroy(op);
      op = nullptr;
    }
    res->status = rc;
    res->iterations = st.iterations;
    res->refinements = st.refinements;
    res->true_res_max = st.true_res_max;
    if (op && !res->retried_fp64 && (rc == BDDA_OK || rc == BDDA_ERR_NOT_CONVERGED) && *reserved <= cache_limit)
      return op;
    if (op) bdda_op_destroy(op);
    return nullptr;
  }

  void worker(bool express) {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      std::vector<bdda_op*> evicted;
      cv_work.wait(lk, [&] {
        return (stopping && pending.empty()) || (express ? pick_express() >= 0 : pick_evicting(&evicted) >= 0);
      });
      if (!evicted.empty()) {
        lk.unlock();
        for (bdda_op* op : evicted) bdda_op_destroy(op);
        lk.lock();
      }
      if (stopping && pending.empty()) return;
      const int i = express ? pick_express() : pick();
      if (i < 0) continue;
      if (i > 0 && (!express || in_use + pending.front().footprint > budget)) pending.front().bypassed++;
      Item it = pending[i];
      pending.erase(pending.begin() + i);
      if (it.exclusive) solo = true;
      in_use += it.footprint;
      peak_in_use = std::max(peak_in_use, in_use);
      peak_running = std::max(peak_running, ++running);
      bdda_request_result res{};
      res.t_submit = it.t_submit;
      res.t_start = now_s(t0);
      res.footprint_bytes = it.footprint;
      lk.unlock();
      OpKey key{};
      for (int d = 0; d < 3; ++d) key.n[d] = it.req.n[d];
      key.f = it.req.f == 6 ? 6 : 3;
      // mixed: FP32 inner solves + double-float residuals; otherwise plain FP64
      key.prec = opts.precision == BDDA_SOLVE_MIXED ? (BDDA_PREC_FP32 | BDDA_PREC_DF64) : BDDA_PREC_FP64;
      key.lf = it.req.lf;
      key.kr = it.req.k_re;
      key.ki = it.req.k_im;
      double reserved = it.footprint;
      bdda_op* keep = execute(it, &res, key, &reserved);
      res.t_done = now_s(t0);
      lk.lock();
      in_use -= reserved;
      if (it.exclusive) solo = false;
      if (res.status == BDDA_ERR_NOMEM && !it.exclusive && !dry) {
        // the device refused memory that the footprint allowed (other requests'
        // buffers, pool fragmentation): queue the request again at the head,
        // to run alone once the running ones are done
        if (keep) {
          lk.unlock();
          bdda_op_destroy(keep);
          lk.lock();
        }
        Item again = it;
        again.exclusive = true;
        pending.push_front(again);
        --running;
        cv_work.notify_all();
        continue;
      }
      if (keep) {
        // keep the operator idle, within the cache limit (oldest first out)
        std::vector<bdda_op*> out;
        while (!idle.empty() && cache_bytes + reserved > cache_limit) out.push_back(evict_lru());
        idle.push_back({key, keep, reserved, ++tick});
        cache_bytes += reserved;
        in_use += reserved;
        if (!out.empty()) {
          lk.unlock();
          for (bdda_op* op : out) bdda_op_destroy(op);
          lk.lock();
        }
      }
      --running;
      ++completed;
      done[it.ticket] = res;
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" {

double bdda_request_footprint(const int n[3], int nocc, int L, int precision) {
  return bdda_request_footprint_f(n, nocc, L, precision, 3);
}

double bdda_request_footprint_f(const int n[3], int nocc, int L, int precision, int f) {
  if (!n || nocc < 1 || L < 1 || (f != 3 && f != 6)) return -1.0;
  return footprint_bytes(n, nocc, L, precision, f);
}

int bdda_server_create(bdda_server** out, int slots, double mem_budget_bytes, const bdda_solve_opts* opts, int dry_run) {
  if (!out || slots < 1 || slots > 256 || !(mem_budget_bytes > 0) || !opts) {
    bdda::set_error("bad server arguments");
    return BDDA_ERR_INVALID;
  }
  if (opts->true_tol <= 0) {
    bdda::set_error("the server solves to a true residual: set opts.true_tol > 0");
    return BDDA_ERR_INVALID;
  }
  bdda_server* s = new bdda_server();
  s->slots = slots;
  s->budget = mem_budget_bytes;
  s->cache_limit = 0.25 * mem_budget_bytes;
  s->opts = *opts;
  s->dry = dry_run != 0;
  for (int i = 0; i < slots; ++i) s->threads.emplace_back([s] { s->worker(false); });
  // express slots for small requests: a quarter of the slots, at least one
  const int express = dry_run ? 0 : std::max(1, slots / 4);
  for (int i = 0; i < express; ++i) s->threads.emplace_back([s] { s->worker(true); });
  *out = s;
  return BDDA_OK;
}

int bdda_server_submit(bdda_server* s, const bdda_request* r, long long* ticket) {
  if (!s || !r || !ticket || r->nocc < 1 || r->L < 1 || r->L > 32 || !r->address || !r->diag || !r->B || !r->X ||
      (r->f != 0 && r->f != 3 && r->f != 6)) {
    bdda::set_error("bad request");
    return BDDA_ERR_INVALID;
  }
  for (int i = 0; i < 3; ++i)
    if (r->n[i] < 1 || r->n[i] > kMaxBoxSide) {
      bdda::set_error("lattice box dimension outside 1.." + std::to_string(kMaxBoxSide) +
                      " (padded FFT lines are limited to " + std::to_string(2 * kMaxBoxSide) + " points)");
      return BDDA_ERR_INVALID;
    }
  const double fp = footprint_bytes(r->n, r->nocc, r->L, s->opts.precision, r->f == 6 ? 6 : 3);
  if (fp > s->budget) {
    bdda::set_error("request footprint " + std::to_string((long long)fp) + " bytes exceeds the server memory budget");
    return BDDA_ERR_NOMEM;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stopping) {
    bdda::set_error("server is shutting down");
    return BDDA_ERR_INVALID;
  }
  bdda_server::Item it;
  it.req = *r;
  it.ticket = s->next_ticket++;
  it.footprint = fp;
  it.t_submit = now_s(s->t0);
  s->pending.push_back(it);
  *ticket = it.ticket;
  s->cv_work.notify_all();
  return BDDA_OK;
}

int bdda_server_wait(bdda_server* s, long long ticket, bdda_request_result* res) {
  if (!s || !res) {
    bdda::set_error("bad wait arguments");
    return BDDA_ERR_INVALID;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket < 1 || ticket >= s->next_ticket) {
    bdda::set_error("unknown ticket");
    return BDDA_ERR_INVALID;
  }
  s->cv_done.wait(lk, [&] { return s->done.count(ticket) != 0; });
  *res = s->done[ticket];
  s->done.erase(ticket);
  if (res->status != BDDA_OK) bdda::set_error("request failed with status " + std::to_string(res->status));
  return res->status;
}

int bdda_server_stats(bdda_server* s, double* peak_inflight_bytes, int* peak_running, long long* completed) {
  if (!s) {
    bdda::set_error("null server");
    return BDDA_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (peak_inflight_bytes) *peak_inflight_bytes = s->peak_in_use;
  if (peak_running) *peak_running = s->peak_running;
  if (completed) *completed = s->completed;
  return BDDA_OK;
}

int bdda_server_set_spectrum_cache(bdda_server* s, double max_bytes) {
  if (!s || max_bytes < 0) {
    bdda::set_error("bad spectrum-cache arguments");
    return BDDA_ERR_INVALID;
  }
  std::vector<bdda_op*> out;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->cache_limit = std::min(max_bytes, s->budget);
    while (!s->idle.empty() && s->cache_bytes > s->cache_limit) out.push_back(s->evict_lru());
    s->cv_work.notify_all();
  }
  for (bdda_op* op : out) bdda_op_destroy(op);
  return BDDA_OK;
}

int bdda_server_cache_stats(bdda_server* s, long long* spectra_reused, long long* spectra_built, double* cached_bytes) {
  if (!s) {
    bdda::set_error("null server");
    return BDDA_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (spectra_reused) *spectra_reused = s->spectra_reused;
  if (spectra_built) *spectra_built = s->spectra_built;
  if (cached_bytes) *cached_bytes = s->cache_bytes;
  return BDDA_OK;
}

int bdda_server_destroy(bdda_server* s) {
  if (!s) return BDDA_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
  }
  for (auto& t : s->threads) t.join();
  for (auto& c : s->idle) bdda_op_destroy(c.op);
  s->idle.clear();
  delete s;
  return BDDA_OK;
}

int bdda_batch_solve(const bdda_request* reqs, int count, int slots, double mem_budget_bytes, const bdda_solve_opts* opts,
                     bdda_request_result* results) {
  if (!reqs || count < 1 || !results) {
    bdda::set_error("bad batch arguments");
    return BDDA_ERR_INVALID;
  }
  bdda_server* s = nullptr;
  int rc = bdda_server_create(&s, slots, mem_budget_bytes, opts, 0);
  if (rc) return rc;
  std::vector<long long> tickets(count, 0);
  int first_err = BDDA_OK;
  for (int i = 0; i < count; ++i) {
    rc = bdda_server_submit(s, &reqs[i], &tickets[i]);
    if (rc != BDDA_OK) {
      std::memset(&results[i], 0, sizeof(results[i]));
      results[i].status = rc;
      if (!first_err) first_err = rc;
    }
  }
  for (int i = 0; i < count; ++i) {
    if (!tickets[i]) continue;
    rc = bdda_server_wait(s, tickets[i], &results[i]);
    if (rc != BDDA_OK && !first_err) first_err = rc;
  }
  bdda_server_destroy(s);
  return first_err;
}

}  // extern "C"
