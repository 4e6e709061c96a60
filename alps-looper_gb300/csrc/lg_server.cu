// Request server: continuous batching of simulation requests over one device arena.
//
// A server thread owns one Engine holding every active request as a chain.  It runs the arena in
// ticks of `sweeps_per_tick` sweeps (one CUDA graph launch per sweep).  Between ticks:
//   * chains that reached THERMALIZATION + SWEEPS are retired: their observables become a
//     result and the chain is masked (it inserts no operators) until the next rebuild;
//   * queued requests are admitted in arrival order while their estimated device memory fits the
//     budget (estimate from the expected operator count, beta * W * N_bonds);
//   * when requests were admitted (at most once per `rebuild_interval_s`, or at once when the
//     arena is idle), the arena is rebuilt with the continuing and the admitted chains, and the
//     continuing chains' state (spins, off-diagonal lists, sweep counters, accumulators) moves
//     device to device (Engine::adopt).
// A chain's trajectory does not depend on the other chains in the arena, so every result equals
// the result of the same request run alone, bit for bit.
//
// This translation unit is included at the end of lg_engine.cu (it uses Engine).
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

namespace {

double server_now(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Device bytes a chain needs: per-sweep buffers for its expected operators and segments, static
// tables and persistent state (the figures follow Engine::build / alloc_dynamic).
double chain_bytes(const ChainSpec& s) {
  const double nv = 1.3 * s.expected_vertices() + 64;
  const double per_vertex = 17.0 + 2 * (19.0 + 48.0 + 16.0);  // vertex + its 2 segments
  const double per_site = 64.0;
  return nv * per_vertex + (double)s.N * per_site + (double)s.NB * 24.0;
}

}  // namespace

struct lg_server {
  lg_server_config cfg;
  int device = 0;
  std::chrono::steady_clock::time_point t0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  struct Req {
    uint64_t id;
    ChainSpec spec;
    double t_submit, t_start;
    double bytes;
  };
  std::deque<Req> pending;
  std::vector<lg_result> done;
  uint64_t next_id = 1;
  // server-thread state
  std::unique_ptr<Engine> eng;
  std::vector<Req> active;          // chain c of eng
  std::vector<bool> retired;
  double active_bytes = 0;
  double last_rebuild = -1e30;
  lg_server_stats stats{};
  int fatal = LG_OK;
  std::string fatal_msg;

  void finish(const Req& r, int status, const lg_obs* obs, double t_now) {
    lg_result res{};
    res.id = r.id;
    res.status = status;
    res.t_submit = r.t_submit;
    res.t_start = r.t_start;
    res.t_finish = t_now;
    res.sites = r.spec.volume;
    res.sweeps = (uint64_t)(r.spec.therm + r.spec.sweeps);
    if (obs) res.obs = *obs;
    std::lock_guard<std::mutex> lk(mu);
    done.push_back(res);
    if (status == LG_OK) stats.completed++; else stats.rejected++;
    cv.notify_all();
  }

  int rebuild(std::vector<Req>& admit, double t_now) {
    std::vector<ChainSpec> specs;
    std::vector<int> from;
    std::vector<Req> nact;
    for (size_t c = 0; c < active.size(); ++c) {
      if (retired[c]) continue;
      specs.push_back(eng->spec[c]);
      from.push_back((int)c);
      nact.push_back(active[c]);
    }
    for (auto& r : admit) {
      r.t_start = t_now;
      specs.push_back(r.spec);
      from.push_back(-1);
      nact.push_back(r);
    }
    std::unique_ptr<Engine> ne;
    if (!specs.empty()) {
      ne.reset(new Engine());
      int rc = ne->build(specs);
      if (rc) return rc;
      if (eng) {
        rc = ne->adopt(*eng, from);
        if (rc) return rc;
      }
    }
    eng = std::move(ne);
    active = std::move(nact);
    retired.assign(active.size(), false);
    stats.rebuilds++;
    last_rebuild = t_now;
    return LG_OK;
  }

  void loop() {
    cudaSetDevice(device);
    while (true) {
      std::vector<Req> admit;
      {
        std::unique_lock<std::mutex> lk(mu);
        const bool idle = !eng || active.empty();
        if (idle && pending.empty())
          cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop || !pending.empty(); });
        if (stop) break;
        const double t = server_now(t0);
        const bool may_rebuild = idle || t - last_rebuild >= cfg.rebuild_interval_s;
        while (may_rebuild && !pending.empty()) {
          Req& r = pending.front();
          const int n_act = (int)active.size() + (int)admit.size();
          if (r.bytes > cfg.budget_bytes) {  // can never fit
            Req bad = r;
            pending.pop_front();
            lk.unlock();
            finish(bad, LG_EBUDGET, nullptr, server_now(t0));
            lk.lock();
            continue;
          }
          if (active_bytes + r.bytes > cfg.budget_bytes || n_act >= cfg.max_active) break;
          active_bytes += r.bytes;
          admit.push_back(r);
          pending.pop_front();
        }
      }
      const double t = server_now(t0);
      if (!admit.empty()) {
        int rc = rebuild(admit, t);
        if (rc) {
          std::lock_guard<std::mutex> lk(mu);
          fatal = rc;
          fatal_msg = g_err;
          cv.notify_all();
          break;
        }
      }
      if (!eng) continue;
      bool any = false;
      for (size_t c = 0; c < active.size(); ++c) any = any || !retired[c];
      if (!any) {
        std::lock_guard<std::mutex> lk(mu);
        eng.reset();
        active.clear();
        retired.clear();
        continue;
      }
      int rc = eng->run(cfg.sweeps_per_tick);
      if (rc) {
        std::lock_guard<std::mutex> lk(mu);
        fatal = rc;
        fatal_msg = g_err;
        cv.notify_all();
        break;
      }
      long long ss = 0;
      for (size_t c = 0; c < active.size(); ++c)
        if (!retired[c]) ss += (long long)eng->spec[c].volume * cfg.sweeps_per_tick;
      {
        std::lock_guard<std::mutex> lk(mu);
        stats.site_sweeps += ss;
      }
      const double tn = server_now(t0);
      for (size_t c = 0; c < active.size(); ++c) {
        if (retired[c]) continue;
        const ChainSpec& s = eng->spec[c];
        if (s.mcs < (uint64_t)(s.therm + s.sweeps)) continue;
        lg_obs o;
        eng->acc[c].report(s, &o);
        retired[c] = true;
        eng->set_active((int)c, false);
        {
          std::lock_guard<std::mutex> lk(mu);
          active_bytes -= active[c].bytes;
        }
        finish(active[c], LG_OK, &o, tn);
      }
    }
  }
};

extern "C" {

void lg_server_config_default(lg_server_config* c) {
  c->budget_bytes = 150e9;
  c->sweeps_per_tick = 16;
  c->rebuild_interval_s = 0.02;
  c->max_active = 4096;
}

double lg_request_bytes(const lg_params* p) {
  ChainSpec s;
  if (s.init(*p)) return -1.0;
  return chain_bytes(s);
}

int lg_server_create(const lg_server_config* cfg, lg_server** out) {
  if (!cfg || !out || cfg->sweeps_per_tick < 1 || !(cfg->budget_bytes > 0))
    return lg_fail(LG_EINVAL, "bad server configuration");
  lg_server* s = new lg_server();
  s->cfg = *cfg;
  s->t0 = std::chrono::steady_clock::now();
  cudaGetDevice(&s->device);
  s->th = std::thread([s] { s->loop(); });
  *out = s;
  return LG_OK;
}

int lg_server_submit(lg_server* s, const lg_params* p, uint64_t* id) {
  if (!s || !p) return lg_fail(LG_EINVAL, "null argument");
  lg_server::Req r;
  int rc = r.spec.init(*p);
  if (rc) return rc;
  r.bytes = chain_bytes(r.spec);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
  r.id = s->next_id++;
  r.t_submit = server_now(s->t0);
  r.t_start = -1;
  s->pending.push_back(r);
  s->stats.submitted++;
  if (id) *id = r.id;
  s->cv.notify_all();
  return LG_OK;
}

int lg_server_poll(lg_server* s, lg_result* out, int cap, int* n) {
  std::lock_guard<std::mutex> lk(s->mu);
  int m = std::min<int>(cap, (int)s->done.size());
  for (int i = 0; i < m; ++i) out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + m);
  if (n) *n = m;
  if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
  return LG_OK;
}

int lg_server_wait(lg_server* s, double timeout_s) {
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    return s->fatal || s->stats.completed + s->stats.rejected >= s->stats.submitted;
  });
  if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
  return ok ? LG_OK : lg_fail(LG_ENOTREADY, "requests still running");
}

int lg_server_get_stats(lg_server* s, lg_server_stats* out) {
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->active_bytes = s->active_bytes;
  out->queued = (int64_t)s->pending.size();
  out->elapsed_s = server_now(s->t0);
  return LG_OK;
}

int lg_server_destroy(lg_server* s) {
  if (!s) return LG_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  delete s;
  return LG_OK;
}

}  // extern "C"
