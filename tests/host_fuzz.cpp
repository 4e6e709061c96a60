// Host-side fuzz harness for lg_host.cpp, built by tests/test_host_sanitizers.py with gcc's
// address, undefined-behaviour and float-cast-overflow sanitizers (any report aborts the run).
// It covers everything the C ABI takes from a caller before device work:
//   * lg_params_parse on random texts and on random edits of a valid parameter file;
//   * ChainSpec::init on random parameter sets, including NaN, infinities and extreme values;
//   * record_values and the accumulators (ChainAcc) on random record words;
//   * checkpoint_encode / checkpoint_decode: valid blobs round trip, and forged blobs (random bit
//     flips, truncation, huge operator counts, each with a recomputed checksum) are answered
//     without touching memory outside the blob.
// lg_fail, which the library defines next to the device code, is replaced by a stub here.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "lg_host.h"

int lg_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return code;
}

static int fuzz_parser(std::mt19937_64& g, int iterations) {
  const std::string base =
      "LATTICE = \"square lattice\"; L = 16\nT = 1/4 # comment\nJz = 0.5; Jxy = 1; h = 0.2\n"
      "SWEEPS = 1024; THERMALIZATION = 128; SEED = 3; local_S = 1/2\n"
      "MEASURE[Correlations] = true; INITIAL_SITE = 2; INITIAL_SPINS = random\n";
  const std::string alpha = "=;#\"[]/ \n\t.-+eE0123456789abcdfinLTJhSWEPNAMRCU_xyz";
  for (int i = 0; i < iterations; ++i) {
    std::string t;
    if (i % 4 == 0) {
      const int n = (int)(g() % 240);
      for (int k = 0; k < n; ++k) t += alpha[g() % alpha.size()];
    } else {
      t = base;
      const int m = 1 + (int)(g() % 8);
      for (int r = 0; r < m; ++r) {
        const size_t k = g() % (t.size() + 1);
        const int op = (int)(g() % 3);
        if (op == 0 && k < t.size()) t.erase(k, 1);
        else if (op == 1) t.insert(t.begin() + k, alpha[g() % alpha.size()]);
        else if (k < t.size()) t[k] = alpha[g() % alpha.size()];
      }
    }
    lg_params p;
    lg_params_default(&p);
    const int rc = lg_params_parse(t.c_str(), &p);
    if (rc != LG_OK && rc != LG_EINVAL && rc != LG_EUNSUPPORTED) {
      std::printf("parser returned %d for [%s]\n", rc, t.c_str());
      return 1;
    }
  }
  return 0;
}

static int fuzz_model_records_checkpoints(std::mt19937_64& g, int iterations, int* valid) {
  std::uniform_real_distribution<double> U(0, 1);
  const double special[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 1e-300, 1e300, -1e300,
                            NAN, INFINITY, -INFINITY, 3.0, 0.25};
  const int nspecial = (int)(sizeof(special) / sizeof(special[0]));
  auto pick = [&]() { return (g() % 3 == 0) ? special[g() % nspecial] : U(g) * 4 - 2; };
  for (int it = 0; it < iterations; ++it) {
    lg_params p;
    lg_params_default(&p);
    p.lattice = (int)(g() % 5);
    p.L = (int)(g() % 12) - 1;
    p.T = pick();
    p.beta = (g() % 2) ? pick() : 0.0;
    p.J = pick();
    p.Jz = (g() % 2) ? pick() : NAN;
    p.Jxy = (g() % 2) ? pick() : NAN;
    p.h = (g() % 2) ? pick() : 0.0;
    p.force_scatter = (g() % 4 == 0) ? pick() : 0.0;
    p.sweeps = g() % 5000;
    p.thermalization = (int64_t)(g() % 3000) - 1;
    p.spin2 = 1 + (int)(g() % 4);
    p.measure_correlations = (int)(g() % 2);
    p.initial_site = (int)(g() % 20) - 2;
    ChainSpec s;
    if (s.init(p) != LG_OK) continue;
    ++*valid;
    (void)s.expected_vertices();
    ChainAcc acc;
    std::vector<uint64_t> rec(64);
    for (int r = 0; r < 200; ++r) {
      for (auto& w : rec) w = (g() % 4 == 0) ? g() : (g() % 1000);
      double v[64];
      record_values(s, rec.data(), v);
      acc.push(s, rec.data());
    }
    lg_obs o;
    acc.report(s, &o);
    std::vector<int32_t> spins(s.N), bonds, sp2, bd2;
    std::vector<double> times, tm2;
    for (auto& x : spins) x = (int)(g() % 2);
    const int n = (int)(g() % 50);
    for (int i = 0; i < n; ++i) {
      bonds.push_back((int)(g() % (uint64_t)s.NB));
      times.push_back(U(g));
    }
    std::vector<uint8_t> blob;
    checkpoint_encode(s, spins, bonds, times, blob);
    uint64_t mcs = 0;
    if (checkpoint_decode(s, blob.data(), blob.size(), sp2, bd2, tm2, &mcs) != LG_OK ||
        bd2 != bonds || tm2 != times || sp2 != spins) {
      std::printf("checkpoint round trip failed\n");
      return 1;
    }
    for (int f = 0; f < 8; ++f) {
      std::vector<uint8_t> b = blob;
      const int m = 1 + (int)(g() % 6);
      for (int k = 0; k < m; ++k) b[g() % (b.size() - 8)] ^= (uint8_t)(1u << (g() % 8));
      if (g() % 3 == 0) {  // a forged operator count
        const uint64_t big = (g() % 2) ? (1ull << 62) + (g() % 7) : g();
        std::memcpy(b.data() + 24, &big, 8);
      }
      if (g() % 4 == 0) b.resize(g() % (b.size() + 1) + 8);
      const uint64_t h = checkpoint_checksum(b.data(), b.size());
      std::memcpy(b.data() + b.size() - 8, &h, 8);
      const int rc = checkpoint_decode(s, b.data(), b.size(), sp2, bd2, tm2, &mcs);
      if (rc != LG_OK && rc != LG_ECORRUPT) {
        std::printf("checkpoint decode returned %d\n", rc);
        return 1;
      }
    }
  }
  return 0;
}

int main() {
  std::mt19937_64 g(20261204);
  if (fuzz_parser(g, 100000)) return 1;
  int valid = 0;
  if (fuzz_model_records_checkpoints(g, 20000, &valid)) return 1;
  std::printf("ok: %d valid models\n", valid);
  return valid > 100 ? 0 : 1;
}
