// Serving loop: continuous batching of factor+solve and solve-only requests
// over factorizations kept resident in HBM.
//
// A request either brings a new matrix for a key (factor, then solve) or only
// a right-hand side for a key whose factors are resident (solve).  Worker
// threads, each with its own context and CUDA stream, take the oldest
// runnable request: its key must not be in use by another worker and, when it
// needs a new factorization object, the HBM budget must admit it (least
// recently used idle factorizations are evicted first).  Requests on one key
// run in submission order; consecutive solve-only requests on the same key are
// merged into one multi-right-hand-side solve.  Work from different workers
// overlaps on the device.  Each solve's arithmetic depends only on its own
// inputs (fixed launch shapes per n, fixed-order reductions), so a result is
// the same whether the request runs alone or in a mix.
//
// No counterpart in the reference: LinearSolve.jl solves one LinearProblem per
// call; this is the request loop around repeated solve!(cache) calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gblu_internal.h"
#include "objects.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
  gblu_request req;
  Clock::time_point t_submit;
  uint64_t seq;
  bool waited = false;  // counted once in admission_waits
};

struct Resident {
  gblu_factor* f = nullptr;
  gblu_ctx* owner = nullptr;
  int64_t n = 0;
  uint64_t bytes = 0;
  bool busy = false;
  bool valid = false;  // holds a successful factorization
  uint64_t last_use = 0;
  std::vector<double> a_small;  // small-lane key: its current matrix (host)
};

}  // namespace

struct gblu_server {
  gblu_ctx* parent = nullptr;
  gblu_serve_config cfg{};
  std::vector<gblu_ctx*> wctx;
  std::vector<std::thread> threads;
  gblu_ctx* small_ctx = nullptr;  // the small-system lane's context and buffers
  gblu::BatchLane* lane = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::deque<gblu_completion> done;
  std::unordered_map<uint64_t, Resident> cache;
  uint64_t bytes_resident = 0;
  uint64_t seq = 0, use_clock = 0;
  bool stopping = false;
  int64_t in_flight = 0;
  int large_running = 0;  // factorizations of n >= cfg.large_n on the workers
  gblu_serve_stats stats{};
};

namespace gblu {
namespace {

uint64_t factor_bytes_estimate(gblu_server* s, gblu_ctx* c, int64_t n) {
  // what gblu_factor_create will allocate, plus the inverses of an FP64
  // factor switched to the fast solve
  uint64_t b = factor_arena_bytes(n, n, s->cfg.precision, c->device);
  if (s->cfg.precision == GBLU_FP64 && s->cfg.solve_mode == GBLU_SOLVE_FAST)
    b += getrs_inverse_bytes(n, sizeof(double));
  return b;
}

// Evict least recently used idle factorizations until `need` more bytes fit.
// The evicted objects are handed back in `victims` and destroyed by the
// caller after it released s->mu (destroying synchronises the owner's stream).
bool admit(gblu_server* s, uint64_t need, std::vector<std::pair<gblu_ctx*, gblu_factor*>>& victims) {
  const uint64_t budget = s->cfg.hbm_budget_bytes;
  if (budget == 0) return true;
  // would evicting every idle object be enough?  Otherwise evict nothing.
  uint64_t idle = 0;
  for (auto& kv : s->cache)
    if (!kv.second.busy) idle += kv.second.bytes;
  if (s->bytes_resident - std::min(s->bytes_resident, idle) + need > budget) return false;
  while (s->bytes_resident + need > budget) {
    auto victim = s->cache.end();
    for (auto it = s->cache.begin(); it != s->cache.end(); ++it)
      if (!it->second.busy && it->second.bytes > 0 &&  // small-lane keys hold no HBM
          (victim == s->cache.end() || it->second.last_use < victim->second.last_use))
        victim = it;
    if (victim == s->cache.end()) return false;  // everything resident is in use: wait
    if (victim->second.f) victims.emplace_back(victim->second.owner, victim->second.f);
    s->bytes_resident -= std::min(s->bytes_resident, victim->second.bytes);
    s->cache.erase(victim);
    s->stats.evictions++;
  }
  return true;
}

void complete(gblu_server* s, const Pending& p, int32_t status, int64_t info, int32_t refactored,
              const gblu_refine_stats& rs, Clock::time_point t_start) {
  gblu_completion c{};
  c.tag = p.req.tag;
  c.status = status;
  c.info = info;
  c.refactored = refactored;
  c.fell_back = rs.fell_back;
  c.iterations = rs.iterations;
  c.backward_error = rs.backward_error;
  const auto now = Clock::now();
  c.latency_us = std::chrono::duration<double, std::micro>(now - p.t_submit).count();
  c.queue_us = std::chrono::duration<double, std::micro>(t_start - p.t_submit).count();
  s->done.push_back(c);
  if (status == GBLU_OK) s->stats.completed++;
  else s->stats.failed++;
}

void worker(gblu_server* s, int wi) {
  gblu_ctx* ctx = s->wctx[wi];
  std::vector<double> packed;
  for (;;) {
    std::vector<Pending> batch;
    Resident* res = nullptr;
    bool need_new = false;
    bool took_large = false;  // holds one of the max_large slots
    uint64_t need_bytes = 0;
    std::vector<std::pair<gblu_ctx*, gblu_factor*>> victims;  // destroyed outside the lock
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        if (s->stopping && s->queue.empty()) return;
        // oldest runnable request: key idle, and memory admitted if it needs a new object
        auto pick = s->queue.end();
        for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
          bool key_busy = false, earlier_same_key = false;
          for (auto jt = s->queue.begin(); jt != it; ++jt)
            if (jt->req.key == it->req.key) { earlier_same_key = true; break; }
          if (earlier_same_key) continue;  // keep per-key order
          if (s->cfg.small_n > 0 && it->req.n <= s->cfg.small_n) continue;  // the small lane's
          const bool large = it->req.A && s->cfg.max_large > 0 && it->req.n >= s->cfg.large_n;
          if (large && s->large_running >= s->cfg.max_large) continue;  // waits for a large slot
          auto c = s->cache.find(it->req.key);
          if (c != s->cache.end()) key_busy = c->second.busy;
          if (key_busy) continue;
          const bool has_obj = c != s->cache.end() && c->second.f && c->second.n == it->req.n;
          if (it->req.A && !has_obj) {
            uint64_t nb = factor_bytes_estimate(s, ctx, it->req.n);
            if (c != s->cache.end() && !c->second.busy) {  // resize: free the old object first
              if (c->second.f) victims.emplace_back(c->second.owner, c->second.f);
              s->bytes_resident -= std::min(s->bytes_resident, c->second.bytes);
              s->cache.erase(c);
            }
            if (!admit(s, nb, victims)) {
              if (!it->waited) {
                it->waited = true;
                s->stats.admission_waits++;
              }
              continue;
            }
            need_new = true;
            need_bytes = nb;
          } else {
            need_new = false;
          }
          pick = it;
          break;
        }
        if (pick != s->queue.end()) {
          took_large = pick->req.A && s->cfg.max_large > 0 && pick->req.n >= s->cfg.large_n;
          if (took_large) s->large_running++;
          batch.push_back(*pick);
          const uint64_t key = pick->req.key;
          auto next = s->queue.erase(pick);
          // merge the following solve-only requests on the same key, up to the
          // next refactor of it (a factoring head request is merged with the
          // solves queued behind it: they use the matrix it factors)
          for (auto it = next; it != s->queue.end() && (int)batch.size() < std::max(1, s->cfg.max_rhs_batch);) {
            if (it->req.key != key) { ++it; continue; }
            if (it->req.A || it->req.n != batch[0].req.n) break;
            batch.push_back(*it);
            it = s->queue.erase(it);
          }
          if (need_new) {
            Resident r;
            r.n = batch[0].req.n;
            r.bytes = need_bytes;
            r.owner = ctx;
            s->cache[key] = r;
            s->bytes_resident += need_bytes;
          }
          res = &s->cache[key];
          res->busy = true;
          res->last_use = ++s->use_clock;
          s->in_flight += (int64_t)batch.size();
          break;
        }
        if (s->stopping && s->queue.empty()) return;
        if (!victims.empty()) break;  // release evicted objects before waiting
        s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
      }
    }
    for (auto& v : victims) gblu_factor_destroy(v.first, v.second);
    if (batch.empty()) continue;
    const auto t_start = Clock::now();
    const Pending& head = batch[0];
    const int64_t n = head.req.n;
    int32_t st = GBLU_OK;
    int64_t info = 0;
    int32_t refactored = 0;
    gblu_refine_stats rs{};
    if (need_new) {
      gblu_factor* f = nullptr;
      st = gblu_factor_create(ctx, n, n, s->cfg.precision, &f);
      if (st == GBLU_OK) st = gblu_factor_set_solve(ctx, f, s->cfg.solve_mode);
      if (st == GBLU_OK && s->cfg.precision != GBLU_FP64 && s->cfg.pivoting != GBLU_PIVOT_PARTIAL &&
          !(s->cfg.pivoting == GBLU_PIVOT_RBT && n < 4))
        st = gblu_factor_set_pivoting(ctx, f, s->cfg.pivoting);
      res->f = f;
      if (f) res->owner = ctx;
    }
    if (st == GBLU_OK && head.req.A) {
      st = gblu_getrf(ctx, res->f, head.req.A, n, GBLU_HOST, &info);
      refactored = 1;
      res->valid = (st == GBLU_OK && info == 0);
    } else if (st == GBLU_OK && (!res->f || !res->valid)) {
      st = GBLU_ENOTFACTORED;
    }
    if (st == GBLU_OK && info == 0) {
      const int64_t k = (int64_t)batch.size();
      packed.resize((size_t)n * k);
      for (int64_t j = 0; j < k; ++j)
        std::copy(batch[j].req.b, batch[j].req.b + n, packed.begin() + j * n);
      if (s->cfg.precision == GBLU_FP64) {
        st = gblu_getrs(ctx, res->f, 'N', k, packed.data(), n, GBLU_HOST);
        rs.converged = 1;
        rs.backward_error = -1;
      } else {
        gblu_refine_opts o;
        gblu_refine_opts_default(&o);
        o.mode = s->cfg.refine_mode;
        st = gblu_solve_refined(ctx, res->f, 'N', k, packed.data(), n, GBLU_HOST, &o, &rs);
      }
      if (st == GBLU_OK)
        for (int64_t j = 0; j < k; ++j)
          std::copy(packed.begin() + j * n, packed.begin() + (j + 1) * n, batch[j].req.x);
    }
    if (st == GBLU_OK && info != 0) st = GBLU_EINVAL;  // singular matrix for this key
    {
      std::lock_guard<std::mutex> lk(s->mu);
      res->busy = false;
      res->last_use = ++s->use_clock;
      if (!res->f) {  // creation failed: drop the reservation
        auto c = s->cache.find(head.req.key);
        if (c != s->cache.end()) {
          s->bytes_resident -= std::min(s->bytes_resident, c->second.bytes);
          s->cache.erase(c);
        }
      }
      for (size_t j = 0; j < batch.size(); ++j)
        complete(s, batch[j], st, info, j == 0 ? refactored : 0, rs, t_start);
      s->in_flight -= (int64_t)batch.size();
      if (took_large) s->large_running--;
      if (batch.size() > 1) s->stats.merged_solves += batch.size() - 1;
      if (refactored) s->stats.factorizations++;
      s->stats.solves += batch.size();
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

// The small-system lane: takes every queued request with n <= small_n whose
// key is idle (per key, the requests up to its first one it cannot take, so a
// key's requests keep their order), and factors + solves all of them in one
// launch of the batched kernels.  A request bringing a matrix uses it (and it
// becomes the key's matrix, copied to host memory); a solve-only request uses
// the key's matrix.  Each system's arithmetic is its own (the batched kernels
// give every system the same result whatever else is in the launch).
void small_worker(gblu_server* s) {
  gblu_ctx* ctx = s->small_ctx;
  const int maxb = std::max(1, s->cfg.max_small_batch);
  std::vector<Pending> batch;
  std::vector<const double*> Ap, bp;
  std::vector<double*> xp;
  std::vector<int32_t> sizes, iters, sys_of;  // sys_of[j]: system of request j (-1: none)
  std::vector<int64_t> info;
  std::vector<std::pair<gblu_ctx*, gblu_factor*>> victims;
  for (;;) {
    batch.clear();
    victims.clear();
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        if (s->stopping && s->queue.empty()) return;
        std::vector<uint64_t> blocked;  // keys with an earlier request left in the queue
        auto is_blocked = [&](uint64_t k) { return std::find(blocked.begin(), blocked.end(), k) != blocked.end(); };
        for (auto it = s->queue.begin(); it != s->queue.end() && (int)batch.size() < maxb;) {
          const uint64_t key = it->req.key;
          if (is_blocked(key)) { ++it; continue; }
          auto c = s->cache.find(key);
          const bool small = it->req.n <= s->cfg.small_n;
          const bool taken_before = std::any_of(batch.begin(), batch.end(),
                                                [&](const Pending& p) { return p.req.key == key; });
          if (!small || (c != s->cache.end() && c->second.busy && !taken_before)) {
            blocked.push_back(key);
            ++it;
            continue;
          }
          if (!taken_before) {
            if (c == s->cache.end()) {
              c = s->cache.emplace(key, Resident{}).first;
            } else if (c->second.f) {  // the key held a large factorization: release it
              victims.emplace_back(c->second.owner, c->second.f);
              s->bytes_resident -= std::min(s->bytes_resident, c->second.bytes);
              c->second.f = nullptr;
              c->second.bytes = 0;
              c->second.valid = false;
              c->second.n = 0;
            }
            c->second.busy = true;
            c->second.last_use = ++s->use_clock;
          }
          batch.push_back(*it);
          it = s->queue.erase(it);
        }
        if (!batch.empty()) {
          s->in_flight += (int64_t)batch.size();
          break;
        }
        if (!victims.empty()) break;
        s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
      }
    }
    for (auto& v : victims) gblu_factor_destroy(v.first, v.second);
    if (batch.empty()) continue;
    const auto t_start = Clock::now();
    // systems: each request's matrix is its own, or its key's latest one
    const size_t k = batch.size();
    Ap.clear(); bp.clear(); xp.clear(); sizes.clear();
    sys_of.assign(k, -1);
    {
      std::lock_guard<std::mutex> lk(s->mu);  // the keys' host matrices
      for (size_t j = 0; j < k; ++j) {
        const gblu_request& r = batch[j].req;
        const double* A = r.A;
        if (!A) {
          for (size_t i = j; i-- > 0;)  // an earlier request of this launch brought one
            if (batch[i].req.key == r.key && batch[i].req.A) {
              A = batch[i].req.n == r.n ? batch[i].req.A : nullptr;
              goto found;
            }
          {
            const Resident& res = s->cache[r.key];
            if (res.valid && res.n == r.n && !res.a_small.empty()) A = res.a_small.data();
          }
        found:;
        }
        if (!A) continue;  // no matrix for this key: not factored
        sys_of[j] = (int32_t)sizes.size();
        sizes.push_back((int32_t)r.n);
        Ap.push_back(A);
        bp.push_back(r.b);
        xp.push_back(r.x);
      }
    }
    info.assign(sizes.size(), 0);
    iters.assign(sizes.size(), 0);
    int32_t st = sizes.empty() ? GBLU_OK
                               : batch_lane_solve(ctx, s->lane, s->cfg.precision, (int)sizes.size(), sizes.data(),
                                                  Ap.data(), bp.data(), xp.data(), info.data(), iters.data());
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t j = 0; j < k; ++j) {
        const gblu_request& r = batch[j].req;
        Resident& res = s->cache[r.key];
        const int sy = sys_of[j];
        if (r.A && st == GBLU_OK && sy >= 0) {  // the key's matrix from now on
          res.a_small.assign(r.A, r.A + (size_t)r.n * r.n);
          res.n = r.n;
          res.valid = info[sy] == 0;
        }
        gblu_refine_stats rs{};
        rs.backward_error = -1;
        rs.converged = 1;
        int32_t rst = st;
        int64_t rinfo = 0;
        if (sy < 0) {
          rst = GBLU_ENOTFACTORED;
        } else if (st == GBLU_OK) {
          rinfo = info[sy];
          rs.iterations = std::max(0, iters[sy]);
          rs.fell_back = iters[sy] < 0 ? 1 : 0;
          if (rinfo != 0) rst = GBLU_EINVAL;  // singular matrix for this key
        }
        complete(s, batch[j], rst, rinfo, r.A ? 1 : 0, rs, t_start);
        if (r.A && rst == GBLU_OK) s->stats.factorizations++;
      }
      for (size_t j = 0; j < k; ++j) {
        Resident& res = s->cache[batch[j].req.key];
        res.busy = false;
        res.last_use = ++s->use_clock;
      }
      s->in_flight -= (int64_t)k;
      s->stats.solves += (int64_t)k;
      s->stats.small_launches += sizes.empty() ? 0 : 1;
      s->stats.small_systems += (int64_t)sizes.size();
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace
}  // namespace gblu

using namespace gblu;

extern "C" {

int32_t gblu_serve_config_default(gblu_serve_config* cfg) {
  if (!cfg) return GBLU_EINVAL;
  cfg->workers = 4;
  cfg->precision = GBLU_FP32;
  cfg->refine_mode = GBLU_REFINE_IR;
  cfg->hbm_budget_bytes = 120ull << 30;
  cfg->max_rhs_batch = 8;
  cfg->small_n = 256;
  cfg->solve_mode = GBLU_SOLVE_FAST;
  cfg->max_small_batch = 1024;
  cfg->large_n = 2048;
  cfg->max_large = 1;
  cfg->pivoting = GBLU_PIVOT_PARTIAL;
  return GBLU_OK;
}

int32_t gblu_serve_create(gblu_ctx* ctx, const gblu_serve_config* cfg, gblu_server** out) {
  if (!ctx || !out) return fail(ctx, GBLU_EINVAL, "gblu_serve_create: NULL argument");
  *out = nullptr;
  gblu_serve_config c;
  gblu_serve_config_default(&c);
  if (cfg) c = *cfg;
  if (c.workers < 1 || c.workers > 32) return fail(ctx, GBLU_EINVAL, "gblu_serve_create: 1..32 workers");
  if (c.precision < GBLU_FP64 || c.precision > GBLU_FP16)
    return fail(ctx, GBLU_EINVAL, "gblu_serve_create: bad precision");
  if (c.refine_mode != GBLU_REFINE_IR && c.refine_mode != GBLU_REFINE_GMRES)
    return fail(ctx, GBLU_EINVAL, "gblu_serve_create: bad refine mode");
  if (c.small_n < 0 || c.small_n > 256) return fail(ctx, GBLU_EINVAL, "gblu_serve_create: small_n in 0..256");
  if (c.solve_mode != GBLU_SOLVE_EXACT && c.solve_mode != GBLU_SOLVE_FAST)
    return fail(ctx, GBLU_EINVAL, "gblu_serve_create: bad solve mode");
  if (c.small_n > 0 && c.max_small_batch < 1)
    return fail(ctx, GBLU_EINVAL, "gblu_serve_create: max_small_batch < 1");
  if (c.pivoting != GBLU_PIVOT_PARTIAL && c.pivoting != GBLU_PIVOT_TOURNAMENT && c.pivoting != GBLU_PIVOT_RBT)
    return fail(ctx, GBLU_EINVAL, "gblu_serve_create: bad pivoting mode");
  gblu_server* s = new gblu_server();
  s->parent = ctx;
  s->cfg = c;
  auto undo = [&]() {
    for (auto* x : s->wctx) gblu_destroy(x);
    if (s->small_ctx) gblu_destroy(s->small_ctx);
    delete s;
  };
  for (int i = 0; i < c.workers; ++i) {
    gblu_ctx* w = nullptr;
    int32_t st = gblu_create(&w, ctx->device, 0);
    if (st) {
      undo();
      return fail(ctx, st, "gblu_serve_create: worker context: %s", gblu_last_error(nullptr));
    }
    s->wctx.push_back(w);
  }
  if (c.small_n > 0) {
    int32_t st = gblu_create(&s->small_ctx, ctx->device, 0);
    if (st == GBLU_OK && !(s->lane = batch_lane_create())) st = GBLU_ENOMEM;
    if (st) {
      undo();
      return fail(ctx, st, "gblu_serve_create: small-system lane: %s", gblu_last_error(nullptr));
    }
  }
  for (int i = 0; i < c.workers; ++i) s->threads.emplace_back(worker, s, i);
  if (c.small_n > 0) s->threads.emplace_back(small_worker, s);
  *out = s;
  return GBLU_OK;
}

int32_t gblu_serve_submit(gblu_server* s, const gblu_request* r) {
  if (!s || !r) return GBLU_EINVAL;
  if (r->n < 1 || !r->b || !r->x) return GBLU_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return GBLU_EINVAL;
    Pending p;
    p.req = *r;
    p.t_submit = std::chrono::steady_clock::now();
    p.seq = ++s->seq;
    s->queue.push_back(p);
    s->stats.submitted++;
  }
  s->cv_work.notify_all();  // the small lane and the workers wait on the same condition
  return GBLU_OK;
}

int32_t gblu_serve_poll(gblu_server* s, gblu_completion* out, int32_t max, int32_t* n_out,
                        int32_t wait_ms) {
  if (!s || !n_out || (max > 0 && !out)) return GBLU_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
  int32_t k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n_out = k;
  return GBLU_OK;
}

int32_t gblu_serve_get_stats(gblu_server* s, gblu_serve_stats* out) {
  if (!s || !out) return GBLU_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->resident_factors = (int64_t)s->cache.size();
  out->resident_bytes = s->bytes_resident;
  out->queued = (int64_t)s->queue.size();
  out->in_flight = s->in_flight;
  return GBLU_OK;
}

int32_t gblu_serve_destroy(gblu_server* s) {
  if (!s) return GBLU_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->threads) t.join();
  for (auto& kv : s->cache)
    if (kv.second.f) gblu_factor_destroy(kv.second.owner, kv.second.f);
  s->cache.clear();
  for (auto* w : s->wctx) gblu_destroy(w);
  if (s->small_ctx) {
    batch_lane_destroy(s->small_ctx, s->lane);
    gblu_destroy(s->small_ctx);
  }
  delete s;
  return GBLU_OK;
}

}  // extern "C"
