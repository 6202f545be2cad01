// Serving loop over the C ABI: a request queue drained by worker threads on
// the context's GPU (each with its own context and stream), batching of
// requests that share an operator, and caches of assembled operators with
// admission by device memory against one budget shared by all workers.
//
// The reference has no serving layer (its examples assemble once and solve
// once); this file is the runtime around the operator for a stream of solves
// on different geometries, refinement levels, degrees and wavenumbers.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <system_error>
#include <thread>
#include <tuple>
#include <vector>

#include "bg_operator.hpp"

namespace {

struct OpKey {
  int geo, kind, M, P;
  double kre, kim;
  bool operator<(const OpKey& o) const {
    return std::tie(geo, kind, M, P, kre, kim) < std::tie(o.geo, o.kind, o.M, o.P, o.kre, o.kim);
  }
  bool operator==(const OpKey& o) const {
    return geo == o.geo && kind == o.kind && M == o.M && P == o.P && kre == o.kre && kim == o.kim;
  }
};

struct CacheEntry {
  OpKey key;
  bg_operator* op;
  size_t bytes;       // admitted footprint (estimate at admission, raised to the measured one after use)
  long last_use = 0;  // server-wide use stamp (least recently used across workers is evicted first)
  bool busy = false;  // its worker is solving with it
};

struct Job {
  long ticket;
  bg_request req;
  std::vector<double> data;  // copy of the data parameters
  double t_submit;
};

OpKey key_of(const bg_request& r) {
  const bool wave = r.op_kind != BG_LAPLACE_SL;
  return OpKey{r.geometry, r.op_kind, r.M, r.P, wave ? r.kre : 0.0, wave ? r.kim : 0.0};
}

// requests that can share one batched solve
bool batchable(const bg_request& a, const bg_request& b) {
  return key_of(a) == key_of(b) && a.data_kind == b.data_kind && a.tol == b.tol &&
         a.inner_precision == b.inner_precision;
}

}  // namespace

// One worker: its own context (stream, pinned staging) on the server's GPU
// and the operators it created. An operator only ever runs on the stream of
// the context that created it, so requests for a cached operator go to its
// worker (owner); requests for an operator that no worker holds go to the
// first worker that is free, which then owns it. The memory budget is one for
// all workers: admission evicts the least recently used idle operator of any
// worker.
struct Worker {
  int id = 0;
  bg_context* ctx = nullptr;
  std::list<CacheEntry> cache;  // front: most recently used by this worker
  DevBuf b_dev, x_dev;
  std::thread th;
};

struct bg_server {
  bg_context* ctx = nullptr;
  size_t budget = 0;
  std::vector<const bg_geometry*> geos;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job> queue;
  std::set<long> pending;                  // submitted, result not yet posted
  std::map<long, bg_request_result> done;  // posted, not yet collected by bg_server_wait
  long next_ticket = 1;
  bool stop = false;
  bg_server_stats st{};
  std::chrono::steady_clock::time_point t0;
  std::vector<Worker*> workers;
  std::map<OpKey, int> owner;       // worker holding (or assembling) the operator of a key
  size_t in_use = 0;                // admitted bytes of all workers, reservations included
  long use_stamp = 0;
  int reserving = 0;                // admissions between reservation and cache entry
  std::condition_variable cv_idle;  // an operator stopped being busy, or a reservation ended
  std::mutex ops_mu;                // operator creation and destruction (context reference counts)

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

  void update_usage() {  // caller holds mu
    int n = 0;
    for (const Worker* w : workers) n += (int)w->cache.size();
    st.bytes_in_use = in_use;
    st.cached_operators = n;
  }

  void destroy_op(bg_operator* op) {
    std::lock_guard<std::mutex> lk(ops_mu);
    bg_operator_destroy(op);
  }

  // Reserve est bytes of the shared budget (caller holds lk on mu): evict
  // idle operators of any worker, least recently used first, and wait for
  // busy ones or other admissions when nothing idle is left. False if est
  // cannot fit even with every other operator gone.
  bool reserve(std::unique_lock<std::mutex>& lk, size_t est) {
    if (est > budget) return false;
    for (;;) {
      if (in_use + est <= budget) {
        in_use += est;
        ++reserving;
        update_usage();
        return true;
      }
      Worker* vw = nullptr;
      std::list<CacheEntry>::iterator victim;
      bool any_busy = reserving > 0;
      for (Worker* o : workers)
        for (auto it = o->cache.begin(); it != o->cache.end(); ++it) {
          if (it->busy) {
            any_busy = true;
            continue;
          }
          if (!vw || it->last_use < victim->last_use) {
            vw = o;
            victim = it;
          }
        }
      if (vw) {
        bg_operator* op = victim->op;
        in_use -= victim->bytes;
        owner.erase(victim->key);
        vw->cache.erase(victim);
        ++st.evictions;
        update_usage();
        lk.unlock();
        destroy_op(op);
        lk.lock();
        continue;
      }
      if (!any_busy) return false;  // nothing to evict and nothing will be freed
      cv_idle.wait(lk);
    }
  }

  // operator of key k, assembled and marked busy; nullptr and *status on failure
  bg_operator* acquire(Worker& w, const OpKey& k, bool* hit, bg_status* status) {
    {
      std::lock_guard<std::mutex> lk(mu);
      for (auto it = w.cache.begin(); it != w.cache.end(); ++it)
        if (it->key == k) {
          w.cache.splice(w.cache.begin(), w.cache, it);
          w.cache.front().busy = true;
          w.cache.front().last_use = ++use_stamp;
          *hit = true;
          return w.cache.front().op;
        }
    }
    *hit = false;
    {
      // another worker may have evicted this key since it was routed here
      std::lock_guard<std::mutex> lk(mu);
      owner[k] = w.id;
    }
    auto give_up = [&](bg_status s) {
      std::lock_guard<std::mutex> lk(mu);
      owner.erase(k);
      *status = s;
      return nullptr;
    };
    if (k.geo < 0 || k.geo >= (int)geos.size()) return give_up(BG_INVALID_ARG);
    bg_h2_params prm;
    bg_h2_params_default(&prm);
    prm.keep_fp64_blocks = 0;  // the cache holds only what the products read
    bg_operator* op = nullptr;
    bg_status s;
    {
      std::lock_guard<std::mutex> lk(ops_mu);
      s = bg_operator_create(w.ctx, geos[k.geo], k.M, k.P, k.kind, &prm, &op);
    }
    if (s == BG_OK && k.kind != BG_LAPLACE_SL) s = bg_operator_set_wavenumber(op, k.kre, k.kim);
    size_t alloc = 0, est = 0;
    if (s == BG_OK) s = bg_operator_memory(op, &alloc, &est);
    if (s == BG_OK) {
      std::unique_lock<std::mutex> lk(mu);
      if (!reserve(lk, est)) s = BG_OOM;
    }
    if (s != BG_OK) {
      if (op) destroy_op(op);
      return give_up(s);
    }
    const double t = now();
    s = bg_operator_assemble(op);
    std::unique_lock<std::mutex> lk(mu);
    st.assembly_s += now() - t;
    --reserving;
    if (s != BG_OK) {
      in_use -= est;
      update_usage();
      owner.erase(k);
      lk.unlock();
      cv_idle.notify_all();
      destroy_op(op);
      *status = s;
      return nullptr;
    }
    CacheEntry e{k, op, est};
    e.busy = true;
    e.last_use = ++use_stamp;
    w.cache.push_front(e);
    update_usage();
    lk.unlock();
    cv_idle.notify_all();
    return op;
  }

  // the worker is done with its front operator
  void release_op(Worker& w) {
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!w.cache.empty()) w.cache.front().busy = false;
    }
    cv_idle.notify_all();
  }

  void finish(Worker& w, std::vector<Job>& batch, bg_status status, int N, double t_start, bool hit, int tot,
              const bg_solve_stats& stats) {
    const double t_done = now();
    std::string msg;
    if (status != BG_OK && status != BG_NOT_CONVERGED) {
      const char* m = bg_last_error_string(w.ctx);
      msg = m ? m : "";
      if (msg.empty()) msg = "status " + std::to_string((int)status);
    }
    std::lock_guard<std::mutex> lk(mu);
    for (const Job& j : batch) {
      bg_request_result r{};
      r.status = status;
      r.N = N;
      r.t_submit = j.t_submit;
      r.t_start = t_start;
      r.t_done = t_done;
      r.cache_hit = hit ? 1 : 0;
      r.batch_nrhs = tot;
      r.stats = stats;
      std::strncpy(r.error, msg.c_str(), sizeof(r.error) - 1);
      done[j.ticket] = r;
      pending.erase(j.ticket);
      ++(status == BG_OK || status == BG_NOT_CONVERGED ? st.completed : st.failed);
    }
    ++st.batches;
    if (status == BG_OK || status == BG_NOT_CONVERGED) (hit ? st.cache_hits : st.cache_misses)++;
    update_usage();
    cv_done.notify_all();
  }

  void process(Worker& w, std::vector<Job>& batch) {
    const double t_start = now();
    bool hit = false;
    bg_status status = BG_OK;
    bg_solve_stats stats{};
    bg_operator* op = acquire(w, key_of(batch[0].req), &hit, &status);
    if (!op) {
      finish(w, batch, status, 0, t_start, hit, 0, stats);
      return;
    }
    struct Release {  // the operator stops being busy however process returns
      bg_server* s;
      Worker& w;
      ~Release() { s->release_op(w); }
    } release{this, w};
    const int N = op->N;
    const size_t usz = op->cplx ? 16 : 8;
    int tot = 0;
    for (const Job& j : batch) tot += j.req.nrhs;
    cudaError_t e = w.b_dev.alloc((size_t)N * tot * usz);
    if (e == cudaSuccess) e = w.x_dev.alloc((size_t)N * tot * usz);
    if (e != cudaSuccess) {
      finish(w, batch, BG_OOM, N, t_start, hit, tot, stats);
      return;
    }
    for (const Job& j : batch)
      if (j.req.x_capacity < (long)N * j.req.nrhs) status = BG_INVALID_ARG;
    long off = 0;
    for (size_t i = 0; i < batch.size() && status == BG_OK; ++i) {
      status = bg_load_vector(op, batch[i].req.data_kind, batch[i].data.data(), batch[i].req.nrhs,
                              static_cast<char*>(w.b_dev.p) + off * N * usz, 1);
      off += batch[i].req.nrhs;
    }
    const double ts = now();
    if (status == BG_OK) {
      bg_solve_params sp;
      bg_solve_params_default(&sp);
      sp.tol = batch[0].req.tol;
      sp.inner_precision = batch[0].req.inner_precision;
      status = bg_solve(op, w.b_dev.p, w.x_dev.p, tot, &sp, &stats, 1);
    }
    off = 0;
    for (size_t i = 0; i < batch.size() && (status == BG_OK || status == BG_NOT_CONVERGED); ++i) {
      e = cudaMemcpyAsync(batch[i].req.x, static_cast<char*>(w.x_dev.p) + off * N * usz,
                          (size_t)N * batch[i].req.nrhs * usz, cudaMemcpyDeviceToHost, w.ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(w.ctx->stream);
      if (e != cudaSuccess) status = BG_DEVICE_ERROR;
      off += batch[i].req.nrhs;
    }
    // raise the admitted footprint to what the operator holds after a solve
    size_t alloc = 0, est = 0;
    const bool measured = bg_operator_memory(op, &alloc, &est) == BG_OK;
    {
      std::lock_guard<std::mutex> lk(mu);
      st.solve_s += now() - ts;
      if (measured && alloc > w.cache.front().bytes) {
        in_use += alloc - w.cache.front().bytes;
        w.cache.front().bytes = alloc;
        update_usage();
      }
    }
    finish(w, batch, status, N, t_start, hit, tot, stats);
  }

  void run(Worker& w) {
    cudaSetDevice(w.ctx->device);
    for (;;) {
      std::vector<Job> batch;
      {
        std::unique_lock<std::mutex> lk(mu);
        // the oldest request whose operator this worker holds or no worker holds
        auto mine = [&] {
          for (auto it = queue.begin(); it != queue.end(); ++it) {
            auto o = owner.find(key_of(it->req));
            if (o == owner.end() || o->second == w.id) return it;
          }
          return queue.end();
        };
        cv_work.wait(lk, [&] { return stop || mine() != queue.end(); });
        auto first = mine();
        if (first == queue.end()) break;  // stopping and nothing left for this worker
        owner[key_of(first->req)] = w.id;
        batch.push_back(std::move(*first));
        queue.erase(first);
        int tot = batch[0].req.nrhs;
        for (auto it = queue.begin(); it != queue.end();) {
          if (batchable(it->req, batch[0].req) && tot + it->req.nrhs <= 32) {
            tot += it->req.nrhs;
            batch.push_back(std::move(*it));
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
      }
      process(w, batch);
      cv_work.notify_all();  // requests for operators this worker gave up may be anyone's now
    }
    std::unique_lock<std::mutex> lk(mu);
    while (!w.cache.empty()) {
      bg_operator* op = w.cache.back().op;
      in_use -= w.cache.back().bytes;
      owner.erase(w.cache.back().key);
      w.cache.pop_back();
      ++st.evictions;
      update_usage();
      lk.unlock();
      destroy_op(op);
      lk.lock();
    }
  }
};

extern "C" {

bg_status bg_server_create(bg_context* ctx, size_t hbm_budget_bytes, int workers, bg_server** out) {
  if (!ctx || !out || hbm_budget_bytes == 0 || workers < 1 || workers > 16) return BG_INVALID_ARG;
  if (ctx->device < 0) return set_error(ctx, BG_UNSUPPORTED, "host-only context: the server needs a GPU");
  bg_server* s = new (std::nothrow) bg_server();
  if (!s) return BG_OOM;
  s->ctx = ctx;
  s->budget = hbm_budget_bytes;
  s->st.bytes_budget = hbm_budget_bytes;
  s->t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < workers; ++i) {
    Worker* w = new (std::nothrow) Worker();
    if (!w) {
      bg_server_destroy(s);
      return BG_OOM;
    }
    w->id = i;
    bg_status st = bg_context_create(ctx->device, &w->ctx);
    if (st != BG_OK) {
      delete w;
      bg_server_destroy(s);
      return set_error(ctx, st, "server worker context");
    }
    s->workers.push_back(w);
  }
  try {
    for (Worker* w : s->workers) w->th = std::thread([s, w] { s->run(*w); });
  } catch (const std::system_error&) {
    bg_server_destroy(s);  // joins the workers already started
    return set_error(ctx, BG_OOM, "server worker threads could not be started");
  }
  *out = s;
  return BG_OK;
}

bg_status bg_server_destroy(bg_server* srv) {
  if (!srv) return BG_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (Worker* w : srv->workers) {
    if (w->th.joinable()) w->th.join();
    w->b_dev.release();
    w->x_dev.release();
    if (w->ctx) bg_context_destroy(w->ctx);
    delete w;
  }
  delete srv;
  return BG_OK;
}

bg_status bg_server_add_geometry(bg_server* srv, const bg_geometry* g, int* index) {
  if (!srv || !g || !index) return BG_INVALID_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->geos.push_back(g);
  *index = (int)srv->geos.size() - 1;
  return BG_OK;
}

bg_status bg_server_submit(bg_server* srv, const bg_request* req, long* ticket) {
  if (!srv || !req || !ticket || !req->data || !req->x || req->nrhs < 1 || req->nrhs > 32 || !(req->tol > 0.0))
    return BG_INVALID_ARG;
  const int npr = req->data_kind == 3 ? 6 : 3;
  try {
    Job j;
    j.req = *req;
    j.data.assign(req->data, req->data + (size_t)npr * req->nrhs);
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stop) return BG_CANCELLED;
    if (req->geometry < 0 || req->geometry >= (int)srv->geos.size()) return BG_INVALID_ARG;
    j.ticket = srv->next_ticket++;
    j.t_submit = srv->now();
    srv->pending.insert(j.ticket);
    srv->queue.push_back(std::move(j));
    *ticket = srv->next_ticket - 1;
    ++srv->st.submitted;
  } catch (const std::bad_alloc&) {
    return BG_OOM;
  }
  srv->cv_work.notify_all();  // the worker of this request's shard may be any of them
  return BG_OK;
}

bg_status bg_server_wait(bg_server* srv, long ticket, double timeout_s, bg_request_result* out) {
  if (!srv || !out) return BG_INVALID_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  // a ticket never issued, or already collected, would never complete
  if (!srv->pending.count(ticket) && !srv->done.count(ticket)) return BG_INVALID_ARG;
  auto ready = [&] { return srv->done.count(ticket) != 0; };
  if (timeout_s < 0) {
    srv->cv_done.wait(lk, ready);
  } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    return BG_TIMEOUT;
  }
  *out = srv->done[ticket];
  srv->done.erase(ticket);
  return BG_OK;
}

bg_status bg_server_stats_get(bg_server* srv, bg_server_stats* out) {
  if (!srv || !out) return BG_INVALID_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  *out = srv->st;
  return BG_OK;
}

}  // extern "C"
