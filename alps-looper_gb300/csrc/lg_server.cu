// Request server: continuous batching of simulation requests over device arenas.
//
// Requests go to one of `lanes` size classes by their expected operators per sweep.  Each lane
// has a thread and one Engine holding every active request of its class as a chain, on its own
// CUDA stream, so the lanes' sweeps run side by side on the GPU and small requests do not wait
// for the sweeps of large ones.  A lane runs its arena in ticks of `sweeps_per_tick` sweeps (one
// CUDA graph launch per sweep).  Between ticks:
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
  static constexpr int MAX_LANES = 4;
  lg_server_config cfg;
  int device = 0;
  int nlanes = 1;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  struct Req {
    uint64_t id;
    ChainSpec spec;
    double t_submit, t_start;
    double bytes;
  };
  std::deque<Req> pending[MAX_LANES];   // per lane, in arrival order
  std::vector<lg_result> done;
  uint64_t next_id = 1;
  double active_bytes = 0;              // over all lanes (the admission budget)
  lg_server_stats stats{};
  int fatal = LG_OK;
  std::string fatal_msg;
  // One lane: an arena of requests of one size class, driven by its own thread on its own CUDA
  // stream (the Engine's), so lanes run side by side on the GPU and a small request never waits
  // for the sweeps of a large one.
  struct Lane {
    std::unique_ptr<Engine> eng;
    std::vector<Req> active;          // chain c of eng
    std::vector<bool> retired;
    double last_rebuild = -1e30;
    int priority = 0;                 // CUDA stream priority: smaller size classes go first
    std::thread th;
  };
  Lane lanes[MAX_LANES];

  // Size class of a request: its expected operators per sweep against fixed cut points
  // (2 lanes: 2^15; 3 lanes: 2^13, 2^17; 4 lanes: 2^12, 2^15, 2^18).
  int lane_of(const ChainSpec& s) const {
    if (nlanes <= 1) return 0;
    const double ev = s.expected_vertices();
    static const double cut[MAX_LANES - 1][MAX_LANES - 1] = {
        {32768.0, 0, 0}, {8192.0, 131072.0, 0}, {4096.0, 32768.0, 262144.0}};
    for (int k = 0; k < nlanes - 1; ++k)
      if (ev < cut[nlanes - 2][k]) return k;
    return nlanes - 1;
  }

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

  void fail(int rc) {
    std::lock_guard<std::mutex> lk(mu);
    if (!fatal) { fatal = rc; fatal_msg = g_err; }
    cv.notify_all();
  }

  int rebuild(Lane& ln, std::vector<Req>& admit, double t_now) {
    std::vector<ChainSpec> specs;
    std::vector<int> from;
    std::vector<Req> nact;
    for (size_t c = 0; c < ln.active.size(); ++c) {
      if (ln.retired[c]) continue;
      specs.push_back(ln.eng->spec[c]);
      from.push_back((int)c);
      nact.push_back(ln.active[c]);
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
      ne->stream_priority = ln.priority;
      // the smallest size class runs chain-resident where its chains fit a CTA
      int rc = ne->build(specs, &ln == &lanes[0]);
      if (rc) return rc;
      if (ln.eng) {
        rc = ne->adopt(*ln.eng, from);
        if (rc) return rc;
      }
    }
    ln.eng = std::move(ne);
    ln.active = std::move(nact);
    ln.retired.assign(ln.active.size(), false);
    {
      std::lock_guard<std::mutex> lk(mu);
      stats.rebuilds++;
    }
    ln.last_rebuild = t_now;
    return LG_OK;
  }

  void loop(int k) {
    cudaSetDevice(device);
    Lane& ln = lanes[k];
    std::deque<Req>& queue = pending[k];
    while (true) {
      std::vector<Req> admit;
      {
        std::unique_lock<std::mutex> lk(mu);
        const bool idle = !ln.eng || ln.active.empty();
        if (idle && queue.empty())
          cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop || fatal || !queue.empty(); });
        if (stop || fatal) break;
        const double t = server_now(t0);
        const bool may_rebuild = idle || t - ln.last_rebuild >= cfg.rebuild_interval_s;
        while (may_rebuild && !queue.empty()) {
          Req& r = queue.front();
          const int n_act = (int)ln.active.size() + (int)admit.size();
          if (r.bytes > cfg.budget_bytes) {  // can never fit
            Req bad = r;
            queue.pop_front();
            lk.unlock();
            finish(bad, LG_EBUDGET, nullptr, server_now(t0));
            lk.lock();
            continue;
          }
          if (active_bytes + r.bytes > cfg.budget_bytes || n_act >= cfg.max_active) break;
          active_bytes += r.bytes;
          admit.push_back(r);
          queue.pop_front();
        }
      }
      const double t = server_now(t0);
      if (!admit.empty()) {
        int rc = rebuild(ln, admit, t);
        if (rc) { fail(rc); break; }
      }
      if (!ln.eng) continue;
      bool any = false;
      for (size_t c = 0; c < ln.active.size(); ++c) any = any || !ln.retired[c];
      if (!any) {
        ln.eng.reset();
        ln.active.clear();
        ln.retired.clear();
        continue;
      }
      int rc = ln.eng->run(cfg.sweeps_per_tick);
      if (rc) { fail(rc); break; }
      long long ss = 0;
      for (size_t c = 0; c < ln.active.size(); ++c)
        if (!ln.retired[c]) ss += (long long)ln.eng->spec[c].volume * cfg.sweeps_per_tick;
      {
        std::lock_guard<std::mutex> lk(mu);
        stats.site_sweeps += ss;
      }
      const double tn = server_now(t0);
      for (size_t c = 0; c < ln.active.size(); ++c) {
        if (ln.retired[c]) continue;
        const ChainSpec& sp = ln.eng->spec[c];
        if (sp.mcs < (uint64_t)(sp.therm + sp.sweeps)) continue;
        lg_obs o;
        ln.eng->acc[c].report(sp, &o);
        ln.retired[c] = true;
        ln.eng->set_active((int)c, false);
        {
          std::lock_guard<std::mutex> lk(mu);
          active_bytes -= ln.active[c].bytes;
        }
        finish(ln.active[c], LG_OK, &o, tn);
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
  c->lanes = 2;
}

double lg_request_bytes(const lg_params* p) {
  if (!p) return -1.0;
  try {  // no exception crosses the ABI (an invalid or unsupported request: -1)
    ChainSpec s;
    if (s.init(*p)) return -1.0;
    return chain_bytes(s);
  } catch (...) {
    lg_fail(LG_ENOMEM, "host memory allocation failed");
    return -1.0;
  }
}

int lg_server_create(const lg_server_config* cfg, lg_server** out) {
  return lg_guard([&]() -> int {
    if (!cfg || !out || cfg->sweeps_per_tick < 1 || !(cfg->budget_bytes > 0) || cfg->lanes < 1 ||
        cfg->lanes > lg_server::MAX_LANES)
      return lg_fail(LG_EINVAL, "bad server configuration");
    lg_server* s = new lg_server();
    s->cfg = *cfg;
    s->nlanes = cfg->lanes;
    s->t0 = std::chrono::steady_clock::now();
    cudaGetDevice(&s->device);
    // lane 0 (the smallest requests) gets the greatest stream priority, so that its short sweeps
    // are scheduled ahead of the long ones of the larger lanes
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess)
      for (int k = 0; k < s->nlanes; ++k) s->lanes[k].priority = std::min(least, greatest + k);
    // a lane that throws stops the server like a failed sweep does (fail: every later call
    // reports it); nothing escapes the thread, which would end the process
    for (int k = 0; k < s->nlanes; ++k)
      s->lanes[k].th = std::thread([s, k] {
        try {
          s->loop(k);
        } catch (const std::bad_alloc&) {
          s->fail(lg_fail(LG_ENOMEM, "server lane %d: host memory allocation failed", k));
        } catch (const std::exception& e) {
          s->fail(lg_fail(LG_EDEVICE, "server lane %d: unexpected exception: %s", k, e.what()));
        } catch (...) {
          s->fail(lg_fail(LG_EDEVICE, "server lane %d: unexpected exception", k));
        }
      });
    *out = s;
    return LG_OK;
  });
}

int lg_server_submit(lg_server* s, const lg_params* p, uint64_t* id) {
  return lg_guard([&]() -> int {
    if (!s || !p) return lg_fail(LG_EINVAL, "null argument");
    lg_server::Req r;
    int rc = r.spec.init(*p);
    if (rc) return rc;
    if (r.spec.sse) return lg_fail(LG_EUNSUPPORTED, "the server runs path-integral chains");
    r.bytes = chain_bytes(r.spec);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
    r.id = s->next_id++;
    r.t_submit = server_now(s->t0);
    r.t_start = -1;
    s->pending[s->lane_of(r.spec)].push_back(r);
    s->stats.submitted++;
    if (id) *id = r.id;
    s->cv.notify_all();
    return LG_OK;
  });
}

int lg_server_poll(lg_server* s, lg_result* out, int cap, int* n) {
  return lg_guard([&]() -> int {
    std::lock_guard<std::mutex> lk(s->mu);
    int m = std::min<int>(cap, (int)s->done.size());
    for (int i = 0; i < m; ++i) out[i] = s->done[i];
    s->done.erase(s->done.begin(), s->done.begin() + m);
    if (n) *n = m;
    if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
    return LG_OK;
  });
}

int lg_server_wait(lg_server* s, double timeout_s) {
  return lg_guard([&]() -> int {
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
      return s->fatal || s->stats.completed + s->stats.rejected >= s->stats.submitted;
    });
    if (s->fatal) return lg_fail(s->fatal, "server stopped: %s", s->fatal_msg.c_str());
    return ok ? LG_OK : lg_fail(LG_ENOTREADY, "requests still running");
  });
}

int lg_server_get_stats(lg_server* s, lg_server_stats* out) {
  return lg_guard([&]() -> int {
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->active_bytes = s->active_bytes;
    out->queued = 0;
    for (int k = 0; k < s->nlanes; ++k) out->queued += (int64_t)s->pending[k].size();
    out->elapsed_s = server_now(s->t0);
    return LG_OK;
  });
}

int lg_server_destroy(lg_server* s) {
  return lg_guard([&]() -> int {
    if (!s) return LG_OK;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
      s->cv.notify_all();
    }
    for (int k = 0; k < s->nlanes; ++k)
      if (s->lanes[k].th.joinable()) s->lanes[k].th.join();
    delete s;
    return LG_OK;
  });
}

}  // extern "C"
