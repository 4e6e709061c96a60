// Exchange Monte Carlo (parallel tempering) over a ladder of inverse temperatures, in one arena.
//
// The reference runs this with ALPS parapack's exchange worker around loop_worker
// (path_integral.C:874-875, sse.C:388).  The worker supplies two hooks (path_integral.C:98-109,
// sse.C:69-71):
// - weight_parameter() = the operator count n of the current configuration (the SSE form: the
//   length of the whole operator string);
// - log_weight(n, beta) = n log beta, since a configuration's weight is proportional to beta^n
//   in normalised imaginary time.
// Here every temperature of the ladder is one chain of a single arena.  Every `interval` sweeps,
// neighbouring temperatures (t, t+1) try to swap, t even and t odd in alternate steps.  The
// acceptance is
//   min(1, exp(log_weight(n_i, beta_{t+1}) + log_weight(n_j, beta_t)
//              - log_weight(n_i, beta_t) - log_weight(n_j, beta_{t+1}))),
// with a Philox uniform keyed by (ladder seed, exchange step, t).  A swap exchanges the two
// chains' inverse temperatures: the configurations stay where they are, and the measurements of
// each sweep go to the accumulator of the temperature the chain had during it.
//
// This translation unit is included at the end of lg_engine.cu (it uses Engine).

struct lg_exchange {
  std::shared_ptr<Engine> eng;
  std::vector<double> betas;           // the ladder
  std::vector<int> chain_of_temp;      // chain holding temperature t
  std::vector<int> temp_of_chain;
  std::vector<uint64_t> attempts, accepts;  // per pair (t, t+1)
  std::vector<lg_chain> views;
  uint64_t seed = 0;
  uint64_t step = 0;                   // exchange steps done
  int since = 0;                       // sweeps since the last exchange step

  int exchange() {
    Engine& e = *eng;
    const int n = (int)betas.size();
    for (int t = (int)(step & 1); t + 1 < n; t += 2) {
      const int c1 = chain_of_temp[t], c2 = chain_of_temp[t + 1];
      const double n1 = (double)e.spec[c1].last_nop, n2 = (double)e.spec[c2].last_nop;
      const double lr = (n1 - n2) * (std::log(betas[t + 1]) - std::log(betas[t]));
      const uint32_t u32 = philox(seed, (uint32_t)step, (uint32_t)t, TAG_EXCHANGE, (uint32_t)(step >> 32)).x;
      const double u = ((double)u32 + 0.5) * std::ldexp(1.0, -32);
      ++attempts[t];
      if (lr >= 0.0 || u < std::exp(lr)) {
        int rc = e.swap_beta(c1, c2);
        if (rc) return rc;
        chain_of_temp[t] = c2;
        chain_of_temp[t + 1] = c1;
        temp_of_chain[c1] = t + 1;
        temp_of_chain[c2] = t;
        e.acc_of_chain[c1] = t + 1;
        e.acc_of_chain[c2] = t;
        ++accepts[t];
      }
    }
    ++step;
    return LG_OK;
  }
};

extern "C" {

uint64_t lg_exchange_chain_seed(uint64_t seed, int i) {
  return seed + (uint64_t)i * 0x9E3779B97F4A7C15ull;
}

int lg_exchange_create(const lg_params* p, int n, const double* betas, lg_exchange** out) {
  return lg_guard([&]() -> int {
    if (!p || !betas || !out || n < 1) return lg_fail(LG_EINVAL, "bad argument");
    std::vector<ChainSpec> specs(n);
    for (int i = 0; i < n; ++i) {
      if (!(betas[i] > 0) || !std::isfinite(betas[i])) return lg_fail(LG_EINVAL, "beta %d must be positive", i);
      lg_params q = *p;
      q.beta = betas[i];
      q.seed = lg_exchange_chain_seed(p->seed, i);
      int rc = specs[i].init(q);
      if (rc) return rc;
    }
    auto e = std::make_shared<Engine>();
    int rc = e->build(specs);
    if (rc) return rc;
    lg_exchange* x = new lg_exchange();
    x->eng = e;
    x->betas.assign(betas, betas + n);
    x->chain_of_temp.resize(n);
    x->temp_of_chain.resize(n);
    for (int i = 0; i < n; ++i) x->chain_of_temp[i] = x->temp_of_chain[i] = i;
    x->attempts.assign(n > 1 ? n - 1 : 0, 0);
    x->accepts.assign(n > 1 ? n - 1 : 0, 0);
    x->views.resize(n);
    for (int i = 0; i < n; ++i) { x->views[i].eng = e; x->views[i].index = i; }
    x->seed = p->seed ^ 0x5851F42D4C957F2Dull;
    *out = x;
    return LG_OK;
  });
}

int lg_exchange_destroy(lg_exchange* x) {
  return lg_guard([&]() -> int {
    delete x; return LG_OK;
  });
}

int lg_exchange_run(lg_exchange* x, int64_t nsweeps, int interval) {
  return lg_guard([&]() -> int {
    if (!x || nsweeps < 0 || interval < 1) return lg_fail(LG_EINVAL, "bad argument");
    while (nsweeps > 0) {
      const int m = (int)std::min<int64_t>(nsweeps, interval - x->since);
      int rc = x->eng->run(m);
      if (rc) return rc;
      nsweeps -= m;
      x->since += m;
      if (x->since >= interval) {
        x->since = 0;
        if ((rc = x->exchange())) return rc;
      }
    }
    return LG_OK;
  });
}

int lg_exchange_observables(lg_exchange* x, int t, lg_obs* out) {
  return lg_guard([&]() -> int {
    if (!x || !out || t < 0 || t >= (int)x->betas.size()) return lg_fail(LG_EINVAL, "bad argument");
    // the chain now at temperature t carries beta_t, which the evaluators need
    const int c = x->chain_of_temp[t];
    x->eng->acc[t].report(x->eng->spec[c], out);
    return LG_OK;
  });
}

int lg_exchange_state(const lg_exchange* x, int32_t* chain_of_temp, uint64_t* attempts,
                      uint64_t* accepts) {
  return lg_guard([&]() -> int {
    if (!x) return lg_fail(LG_EINVAL, "null argument");
    const int n = (int)x->betas.size();
    for (int t = 0; t < n; ++t) {
      if (chain_of_temp) chain_of_temp[t] = x->chain_of_temp[t];
      if (t + 1 < n) {
        if (attempts) attempts[t] = x->attempts[t];
        if (accepts) accepts[t] = x->accepts[t];
      }
    }
    return LG_OK;
  });
}

lg_chain* lg_exchange_chain(lg_exchange* x, int c) {
  return (x && c >= 0 && c < (int)x->views.size()) ? &x->views[c] : nullptr;
}

}  // extern "C"
