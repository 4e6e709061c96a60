// Host-side model setup, observables and checkpoints of the GB300 loop-cluster engine.
#include "lg_host.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

using namespace lg;

// ---------------------------------------------------------------------------------------------
// Parameters
// ---------------------------------------------------------------------------------------------
extern "C" void lg_params_default(lg_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->lattice = LG_CHAIN;
  p->L = 8;
  p->T = 0.2;
  p->beta = 0.0;
  p->J = 1.0;
  p->Jz = NAN;
  p->Jxy = NAN;
  p->h = 0.0;
  p->force_scatter = 0.0;
  p->sweeps = 65536;          // montecarlo.h:41 SWEEPS default [65536:]
  p->thermalization = -1;     // SWEEPS/8 (montecarlo.h:44)
  p->seed = 29833;
  p->init_spins = 0;
  p->disable_improved_estimator = 0;
  p->measure_correlations = 0;
  p->measure_structure_factor = 0;
  p->initial_site = -1;
  p->spin2 = 1;
  p->algorithm = LG_PATH_INTEGRAL;
}

static bool parse_bool(const std::string& v, int* out) {
  if (v == "1" || v == "true" || v == "True" || v == "TRUE") { *out = 1; return true; }
  if (v == "0" || v == "false" || v == "False" || v == "FALSE") { *out = 0; return true; }
  return false;
}

static std::string trim(std::string s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  s = s.substr(a, b - a);
  if (s.size() >= 2 && s.front() == '"' && s.back() == '"') s = s.substr(1, s.size() - 2);
  return s;
}

// number, or number/number (e.g. T = 1/4)
static bool parse_num(const std::string& v, double* out) {
  char* end = nullptr;
  double a = std::strtod(v.c_str(), &end);
  if (end == v.c_str()) return false;
  while (*end == ' ') ++end;
  if (*end == '/') {
    char* e2 = nullptr;
    double b = std::strtod(end + 1, &e2);
    if (e2 == end + 1 || b == 0) return false;
    while (*e2 == ' ') ++e2;
    if (*e2) return false;
    a /= b;
  } else if (*end) {
    return false;
  }
  *out = a;
  return true;
}

extern "C" int lg_params_parse(const char* text, lg_params* p) {
  return lg_guard([&]() -> int {
    if (!text || !p) return lg_fail(LG_EINVAL, "null argument");
    std::string all(text);
    size_t i = 0;
    while (i < all.size()) {
      size_t j = all.find_first_of(";\n", i);
      if (j == std::string::npos) j = all.size();
      std::string line = all.substr(i, j - i);
      i = j + 1;
      size_t hash = line.find('#');
      if (hash != std::string::npos) line = line.substr(0, hash);
      size_t eq = line.find('=');
      if (eq == std::string::npos) continue;
      std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
      double x = 0;
      auto num = [&](double* dst) -> int {
        if (!parse_num(val, &x)) return lg_fail(LG_EINVAL, "bad value for %s: '%s'", key.c_str(), val.c_str());
        *dst = x;
        return LG_OK;
      };
      // integer keys: a finite value within [lo, hi], truncated toward zero as an int conversion
      // of the parameter would (out-of-range and non-finite values are errors, never a cast)
      auto integer = [&](double lo, double hi, double* dst) -> int {
        if (!parse_num(val, &x) || !(x >= lo && x <= hi))
          return lg_fail(LG_EINVAL, "bad value for %s: '%s'", key.c_str(), val.c_str());
        *dst = std::trunc(x);
        return LG_OK;
      };
      const double kInt = 2147483647.0, kExact = 9007199254740992.0;  // 2^31 - 1, 2^53
      int rc = LG_OK;
      if (key == "LATTICE") {
        if (val == "chain lattice" || val == "chain") p->lattice = LG_CHAIN;
        else if (val == "square lattice" || val == "square") p->lattice = LG_SQUARE;
        else if (val == "simple cubic lattice" || val == "cubic lattice" || val == "cubic") p->lattice = LG_CUBIC;
        else return lg_fail(LG_EUNSUPPORTED, "LATTICE '%s' not supported", val.c_str());
      } else if (key == "L") {
        double d = 0; if (!(rc = integer(-kInt, kInt, &d))) p->L = (int)d;
      } else if (key == "T") {
        rc = num(&p->T);
      } else if (key == "BETA" || key == "INVERSE_TEMPERATURE") {
        rc = num(&p->beta);
      } else if (key == "TEMPERATURE") {
        rc = num(&p->T);
      } else if (key == "J") {
        rc = num(&p->J);
      } else if (key == "Jz") {
        rc = num(&p->Jz);
      } else if (key == "Jxy") {
        rc = num(&p->Jxy);
      } else if (key == "h") {
        rc = num(&p->h);
      } else if (key == "FORCE_SCATTER") {
        rc = num(&p->force_scatter);
      } else if (key == "SWEEPS") {
        double d = 0; if (!(rc = integer(0, kExact, &d))) p->sweeps = (uint64_t)d;
      } else if (key == "THERMALIZATION") {
        double d = 0; if (!(rc = integer(-kExact, kExact, &d))) p->thermalization = (int64_t)d;
      } else if (key == "SEED") {
        double d = 0;  // below 2^64
        if (!(rc = integer(0, 18446744073709549568.0, &d))) p->seed = (uint64_t)d;
      } else if (key == "INITIAL_SPINS") {
        if (val == "up") p->init_spins = 0;
        else if (val == "random") p->init_spins = 1;
        else return lg_fail(LG_EINVAL, "INITIAL_SPINS must be up or random");
      } else if (key == "DISABLE_IMPROVED_ESTIMATOR") {
        p->disable_improved_estimator = (val == "0" || val == "false") ? 0 : 1;
      } else if (key == "MEASURE[Correlations]") {
        if (!parse_bool(val, &p->measure_correlations))
          return lg_fail(LG_EINVAL, "MEASURE[Correlations] must be true or false");
      } else if (key == "MEASURE[Structure Factor]") {
        if (!parse_bool(val, &p->measure_structure_factor))
          return lg_fail(LG_EINVAL, "MEASURE[Structure Factor] must be true or false");
      } else if (key == "INITIAL_SITE") {
        double d = 0; if (!(rc = integer(-kInt, kInt, &d))) p->initial_site = (int)d;
      } else if (key == "ALGORITHM") {
        if (val == "loop; path integral" || val == "loop; path integral; exchange")
          p->algorithm = LG_PATH_INTEGRAL;
        else if (val == "loop; sse" || val == "loop; sse; exchange")
          p->algorithm = LG_SSE;
        else
          return lg_fail(LG_EUNSUPPORTED, "ALGORITHM \"%s\" is not a loop worker of this library", val.c_str());
      } else if (key == "local_S") {
        double d = 0; rc = num(&d);
        if (!rc) {
          const double t = 2 * d;
          if (!(t >= 1 && t <= 64) || std::fabs(t - std::round(t)) > 1e-9)
            return lg_fail(LG_EINVAL, "local_S must be a positive multiple of 1/2");
          p->spin2 = (int)std::round(t);
        }
      }
      if (rc) return rc;
    }
    return LG_OK;
  });
}

// ---------------------------------------------------------------------------------------------
// Model
// ---------------------------------------------------------------------------------------------
static double crop0(double x) { return x > 0 ? x : 0; }
static double crop01(double x) { return x < 0 ? 0 : (x > 1 ? 1 : x); }

static uint64_t prob32(double p) {  // round(p 2^32) clamped to [0, 2^32]
  if (!(p > 0)) return 0;
  if (p >= 1) return 1ull << 32;
  return (uint64_t)std::floor(p * 4294967296.0 + 0.5);
}

int ChainSpec::init(const lg_params& p) {
  if (p.lattice < LG_CHAIN || p.lattice > LG_CUBIC) return lg_fail(LG_EUNSUPPORTED, "unknown LATTICE %d", p.lattice);
  if (p.L < 2) return lg_fail(LG_EINVAL, "L must be >= 2 (got %d)", p.L);
  dim = p.lattice;
  L = p.L;
  spin2 = p.spin2 >= 1 ? p.spin2 : 1;
  if (spin2 > 8) return lg_fail(LG_EUNSUPPORTED, "local_S = %d/2 > 4 is not supported", spin2);
  if (2 * p.lattice * spin2 > MAXZ)  // incident virtual bonds of a virtual site
    return lg_fail(LG_EUNSUPPORTED, "local_S = %d/2 on this lattice gives %d incident bonds > %d",
                   spin2, 2 * p.lattice * spin2, MAXZ);
  long long n = 1;
  for (int i = 0; i < dim; ++i) n *= L;
  if (n * spin2 > (1ll << 22))
    return lg_fail(LG_EBUDGET, "%lld sites exceed the per-chain limit of 2^22", n * spin2);
  // spin S = spin2/2: spin2 virtual spin-1/2 sites per real site (v = site*spin2 + a) and the
  // spin2^2 virtual bonds between the virtual sites of a real bond's two ends
  // (b = rbond*spin2^2 + a*spin2 + a'), as looper's virtual graph (lattice.h); every virtual site
  // has its real site's gauge
  volume = (int)n;
  N = (int)n * spin2;
  const int q = spin2 * spin2;
  NB = (int)n * dim * q;
  s0.resize(NB); s1.resize(NB); gauge.resize(N);
  for (int s = 0; s < (int)n; ++s) {
    int x[3] = {0, 0, 0}, r = s, par = 0;
    for (int i = 0; i < dim; ++i) { x[i] = r % L; r /= L; par += x[i]; }
    for (int a = 0; a < spin2; ++a) gauge[s * spin2 + a] = (par % 2 == 0) ? 1 : -1;
    for (int i = 0; i < dim; ++i) {
      int y[3] = {x[0], x[1], x[2]};
      y[i] = (y[i] + 1) % L;
      int t = 0;
      for (int j = dim - 1; j >= 0; --j) t = t * L + y[j];
      for (int a = 0; a < spin2; ++a)
        for (int a2 = 0; a2 < spin2; ++a2) {
          s0[(s * dim + i) * q + a * spin2 + a2] = s * spin2 + a;
          s1[(s * dim + i) * q + a * spin2 + a2] = t * spin2 + a2;
        }
    }
  }
  bipartite = (L % 2 == 0);
  double b = p.beta > 0 ? p.beta : (p.T > 0 ? 1.0 / p.T : -1.0);
  if (!(b > 0) || !std::isfinite(b)) return lg_fail(LG_EINVAL, "temperature must be positive");
  jz = std::isnan(p.Jz) ? p.J : p.Jz;
  jxy = std::isnan(p.Jxy) ? p.J : p.Jxy;
  h = p.h;
  if (!std::isfinite(jz) || !std::isfinite(jxy) || !std::isfinite(h))
    return lg_fail(LG_EINVAL, "couplings must be finite");
  // An antiferromagnetic exchange in the xy plane has negative off-diagonal weights; they cancel
  // only on bipartite lattices (model_parameter.h:615-662).  Signed models are not supported.
  if (jxy > 0 && !bipartite)
    return lg_fail(LG_EUNSUPPORTED, "Jxy > 0 on a non-bipartite lattice (odd L) has a sign problem");
  if (!std::isfinite(p.force_scatter)) return lg_fail(LG_EINVAL, "FORCE_SCATTER must be finite");
  force_scatter = crop01(p.force_scatter);
  // graph weights: weight_impl.h:282-315 with Jx = Jy = Jxy (Jm = 0)
  const double jp = std::fabs(jxy), a = force_scatter;
  v[0] = v[1] = v[2] = v[3] = 0;
  if (jp + std::fabs(jz) > 1e-12) {
    if (jp - jz > 2 * a * jp) {
      v[0] = crop0(std::min(jp / 2, (jp + jz) / 4));
      v[1] = crop0(std::min(jp / 2, (jp - jz) / 4));
      v[2] = crop0(-(jp - jz) / 2);
      v[3] = crop0(-(jp + jz) / 2);
    } else {
      v[0] = (1 - a) * jp / 2;
      v[1] = a * jp / 2;
      v[2] = -((1 - 2 * a) * jp - jz) / 2;
      v[3] = 0;
    }
  }
  W = v[0] + v[1] + v[2] + v[3];
  energy_offset = NB * W / 2;
  field = std::fabs(h) > 1e-12;
  improved = !field && !p.disable_improved_estimator;   // path_integral.C:217
  sweeps = (int64_t)p.sweeps;
  therm = p.thermalization >= 0 ? p.thermalization : (int64_t)(p.sweeps >> 3);
  init_spins = p.init_spins ? 1 : 0;
  mcs = 0;
  dchain = DChain{};
  dchain.seed = p.seed;
  if (W > 0) {
    dchain.T0 = prob32(v[0] / W);
    dchain.T1 = prob32((v[0] + v[1]) / W);
    dchain.T2 = prob32((v[0] + v[1] + v[2]) / W);
  }
  const double s01 = v[0] + v[1];
  dchain.Poff = prob32(s01 > 0 ? v[0] / s01 : 1.0);
  // the SSE worker's diagonal graph choice (graph_impl.h:297-312)
  dchain.Pd0 = prob32(v[0] + v[2] > 0 ? v[0] / (v[0] + v[2]) : 1.0);
  dchain.Pd1 = prob32(v[1] + v[3] > 0 ? v[1] / (v[1] + v[3]) : 1.0);
  sse = p.algorithm == LG_SSE;
  if (p.algorithm != LG_PATH_INTEGRAL && p.algorithm != LG_SSE)
    return lg_fail(LG_EINVAL, "unknown ALGORITHM %d", p.algorithm);
  if (sse) {
    // sse.C:123 checks the model without longitudinal field support; correlations are not
    // built for the SSE form here
    if (field) return lg_fail(LG_EUNSUPPORTED, "the SSE worker supports no longitudinal field");
    if (p.measure_correlations || p.measure_structure_factor)
      return lg_fail(LG_EUNSUPPORTED, "correlations are measured by the path-integral form only");
  }
  dchain.field = field ? 1 : 0;
  // correlations (correlation.h:62-110): the structure factor needs the all-pairs sums; the
  // correlations use them too unless INITIAL_SITE picks one origin
  if (p.initial_site >= volume)
    return lg_fail(LG_EINVAL, "INITIAL_SITE %d out of range (%d sites)", p.initial_site, volume);
  if (spin2 > 1 && (p.measure_correlations || p.measure_structure_factor))
    return lg_fail(LG_EUNSUPPORTED, "correlations are measured for S = 1/2 only");
  measure_corr = p.measure_correlations != 0;
  measure_sfac = p.measure_structure_factor != 0;
  corr_origin = (measure_corr && p.initial_site >= 0) ? p.initial_site : -1;
  dchain.dim = dim;
  dchain.L = L;
  dchain.spin2 = spin2;
  dchain.corr_disp = (measure_sfac || (measure_corr && corr_origin < 0)) ? 1 : 0;
  dchain.corr_origin = corr_origin;
  dchain.corr_from = (uint32_t)std::min<int64_t>(therm, 0xFFFFFFFFll);
  dchain.corr_to = (uint32_t)std::min<int64_t>(therm + sweeps, 0xFFFFFFFFll);
  return set_beta(b);
}

// ---------------------------------------------------------------------------------------------
// Vector observables: exact integer sums per chunk of sweeps, rebinned
// ---------------------------------------------------------------------------------------------
void VecAcc::add_chunk(const int64_t* s, int n, int64_t sweeps) {
  if (sweeps <= 0) return;
  if ((int)sum.size() != n) { sum.assign(n, 0); bins.clear(); bin_count.clear(); count = 0; }
  std::vector<int64_t> b(s, s + n);
  for (int i = 0; i < n; ++i) sum[i] += s[i];
  count += sweeps;
  bins.push_back(std::move(b));
  bin_count.push_back(sweeps);
  if (bins.size() >= 128) {  // merge neighbouring bins: at most 64 remain
    std::vector<std::vector<int64_t>> nb;
    std::vector<int64_t> nc;
    for (size_t k = 0; k + 1 < bins.size(); k += 2) {
      std::vector<int64_t> m = bins[k];
      for (int i = 0; i < n; ++i) m[i] += bins[k + 1][i];
      nb.push_back(std::move(m));
      nc.push_back(bin_count[k] + bin_count[k + 1]);
    }
    if (bins.size() % 2) { nb.push_back(bins.back()); nc.push_back(bin_count.back()); }
    bins.swap(nb);
    bin_count.swap(nc);
  }
}

// Mean per sweep and the standard error from the spread of the bin means (count-weighted).
void VecAcc::mean_err(std::vector<double>& mean, std::vector<double>& err) const {
  const int n = (int)sum.size();
  mean.assign(n, NAN);
  err.assign(n, NAN);
  if (count <= 0) return;
  for (int i = 0; i < n; ++i) mean[i] = (double)sum[i] / (double)count;
  const size_t B = bins.size();
  if (B < 2) return;
  for (int i = 0; i < n; ++i) {
    double v = 0;
    for (size_t k = 0; k < B; ++k) {
      const double d = (double)bins[k][i] / (double)bin_count[k] - mean[i];
      v += (double)bin_count[k] * d * d;
    }
    err[i] = std::sqrt(v / (double)count / (double)(B - 1));
  }
}

int ChainSpec::set_beta(double b) {
  if (!(b > 0) || !std::isfinite(b)) return lg_fail(LG_EINVAL, "beta must be positive");
  beta = b;
  dchain.inv_rate = W > 0 ? (float)(1.0 / (beta * W)) : 0.0f;
  dchain.flip_coef = (float)(beta * h * std::ldexp(1.0, -40));
  dchain.sse_bw = beta * W * NB;
  return LG_OK;
}

double ChainSpec::expected_vertices() const {
  const double m = beta * W * NB;  // expected diagonal proposals per sweep
  return 1.6 * m + 8 * std::sqrt(m) + 64;
}

// ---------------------------------------------------------------------------------------------
// Observables
// ---------------------------------------------------------------------------------------------
static double i64(uint64_t x) { return (double)(int64_t)x; }
static double u128d(const uint64_t* r, int i) { return (double)r[i] + std::ldexp((double)r[i + 1], 64); }

// A susceptibility from its two collector sums: path integral (susceptibility.h:225-226 etc.)
// beta * integral / V, the integral in beta units; SSE (susceptibility.h:224-225, with
// divide_if_positive) beta * (integral / n + tau0) / (n + 1) / V, the integral in operator units.
static double chi(const ChainSpec& s, double nop, double integral, double tau0) {
  const double V = (double)s.volume;
  if (!s.sse) return s.beta * integral / V;
  return s.beta * ((nop > 0 ? integral / nop : 0.0) + tau0) / (nop + 1) / V;
}

void record_values(const ChainSpec& s, const uint64_t* r, double* v) {
  const double beta = s.beta, V = (double)s.volume;
  const double nop = (double)r[R_NOP];
  double ene = s.energy_offset - nop / beta;                       // path_integral.C:850
  if (s.field) ene += -s.h * i64(r[R_FLD]) * std::ldexp(1.0, -40) / 2;  // :852-859
  v[RAW_E] = ene;
  v[RAW_E2] = ene * ene - nop / (beta * beta);                     // energy.h:83
  v[RAW_NC] = (double)r[R_NC];
  v[RAW_NOP] = nop;
  // Stiffness (stiffness.h:116-160): sum over directions of (winding/2)^2 / (beta dim); the
  // improved estimator sums the clusters' squared windings, the normal one squares the total
  const double dim = (double)s.dim;
  if (s.improved) {
    v[RAW_STIFF] = (double)r[R_WSQ] / 4 / (beta * dim);
  } else {
    double w2 = 0;
    for (int d = 0; d < 3; ++d) w2 += i64(r[R_W0 + d]) * i64(r[R_W0 + d]) / 4;
    v[RAW_STIFF] = w2 / (beta * dim);
  }
  // world-line lengths: 2^-40 of beta on the path-integral form, operator indices on the SSE form
  const double u2 = s.sse ? 1.0 : std::ldexp(1.0, -80), u1 = s.sse ? 1.0 : std::ldexp(1.0, -40);
  (void)V;
  if (s.improved) {                                                // susceptibility.h:200-254
    const double m2 = (double)r[R_M0SQ] / 4, m4 = u128d(r, R_M0Q) / 16;
    const double sm2 = (double)r[R_SM0SQ] / 4, sm4 = u128d(r, R_SM0Q) / 16;
    v[RAW_M] = 0.0;
    v[RAW_ABSM] = std::fabs(i64(r[R_M0])) / 2;
    v[RAW_M2] = m2;
    v[RAW_M4] = 3 * m2 * m2 - 2 * m4;
    v[RAW_CHI] = chi(s, nop, u128d(r, R_MSQ) * u2 / 4, m2);
    v[RAW_SM2] = sm2;
    v[RAW_SM4] = 3 * sm2 * sm2 - 2 * sm4;
    v[RAW_SCHI] = chi(s, nop, u128d(r, R_SMSQ) * u2 / 4, sm2);
    v[RAW_GM2] = (double)r[R_N0SQ] / 4;
    v[RAW_GCHI] = chi(s, nop, u128d(r, R_LSQ) * u2 / 4, (double)r[R_N0SQ] / 4);
  } else {                                                         // susceptibility.h:303-335
    const double m = i64(r[R_M0]) / 2, sm = i64(r[R_SM0]) / 2;
    const double ma = i64(r[R_MA]) * u1 / 2, sma = i64(r[R_SMA]) * u1 / 2;
    v[RAW_M] = m;
    v[RAW_ABSM] = std::fabs(m);
    v[RAW_M2] = m * m;
    v[RAW_M4] = m * m * m * m;
    v[RAW_CHI] = chi(s, nop, ma * ma, m * m);
    v[RAW_SM2] = sm * sm;
    v[RAW_SM4] = sm * sm * sm * sm;
    v[RAW_SCHI] = chi(s, nop, sma * sma, sm * sm);
    v[RAW_GM2] = 0;
    v[RAW_GCHI] = 0;
  }
}

uint64_t value_mask(const ChainSpec& s) {
  uint64_t m = 0;
  for (int i = 0; i < LG_NUM_VALUES; ++i) {
    const bool gen = (i >= LG_VAL_GEN_MAGNETIZATION2 && i <= LG_VAL_GEN_SUSCEPTIBILITY) ||
                     (i >= LG_VAL_GEN_STAG_MAGNETIZATION2 && i <= LG_VAL_GEN_STAG_SUSCEPTIBILITY);
    const bool stag = i >= LG_VAL_STAG_MAGNETIZATION && i <= LG_VAL_GEN_STAG_SUSCEPTIBILITY;
    if (gen && !s.improved) continue;      // susceptibility.h:69-75, 86-92
    if (stag && !s.bipartite) continue;    // susceptibility.h:76
    m |= 1ull << i;
  }
  return m;
}

// The pushes of loop_worker::run for one sweep record: path_integral.C:832-836 and 849-860,
// energy.h:76-84, susceptibility.h:200-254 (improved) or :303-335 (normal), stiffness.h:124-127
// (improved) or :160-165 (normal).  The record's integer sums map onto the collector fields:
// umag0 = M0/2, umag2 = M0SQ/4, umag4 = M0Q/16, usize2 = N0SQ/4, usize4 = N0Q/16 (tau = 0
// cluster sums), umag = MSQ 2^-80/4, usize = LSQ 2^-80/4 (time-integrated, 2^-40 units), and the
// staggered ones likewise; the normal estimator's umag = M0/2 and umag_a = MA 2^-40/2.
void record_scalars(const ChainSpec& s, const uint64_t* r, double* v) {
  const double beta = s.beta, vol = (double)s.volume;
  double raw[NUM_RAW];
  record_values(s, r, raw);
  for (int i = 0; i < LG_NUM_VALUES; ++i) v[i] = std::nan("");
  const uint64_t mask = value_mask(s);
  auto p2 = [](double x) { return x * x; };
  auto p4 = [](double x) { return x * x * x * x; };
  v[LG_VAL_TEMPERATURE] = 1 / beta;
  v[LG_VAL_INVERSE_TEMPERATURE] = beta;
  v[LG_VAL_VOLUME] = vol;
  v[LG_VAL_NUMBER_OF_SITES] = vol;
  v[LG_VAL_NUMBER_OF_CLUSTERS] = raw[RAW_NC];
  v[LG_VAL_ENERGY] = raw[RAW_E];
  v[LG_VAL_ENERGY_DENSITY] = raw[RAW_E] / vol;
  v[LG_VAL_ENERGY2] = raw[RAW_E2];
  const double u2 = s.sse ? 1.0 : std::ldexp(1.0, -80), u1 = s.sse ? 1.0 : std::ldexp(1.0, -40);
  const double nop = (double)r[R_NOP];
  if (s.improved) {
    const double umag0 = i64(r[R_M0]) / 2, umag2 = (double)r[R_M0SQ] / 4, umag4 = u128d(r, R_M0Q) / 16;
    const double usize2 = (double)r[R_N0SQ] / 4, usize4 = u128d(r, R_N0Q) / 16;
    const double umag = u128d(r, R_MSQ) * u2 / 4, usize = u128d(r, R_LSQ) * u2 / 4;
    const double smag0 = i64(r[R_SM0]) / 2, smag2 = (double)r[R_SM0SQ] / 4, smag4 = u128d(r, R_SM0Q) / 16;
    const double ssize2 = (double)r[R_SN0SQ] / 4, ssize4 = u128d(r, R_SN0Q) / 16;
    const double smag = u128d(r, R_SMSQ) * u2 / 4, ssize = u128d(r, R_SLSQ) * u2 / 4;
    v[LG_VAL_MAGNETIZATION] = 0.0;
    v[LG_VAL_MAGNETIZATION_DENSITY] = 0.0;
    v[LG_VAL_ABS_MAGNETIZATION] = std::fabs(umag0);
    v[LG_VAL_ABS_MAGNETIZATION_DENSITY] = std::fabs(umag0) / vol;
    v[LG_VAL_MAGNETIZATION2] = umag2;
    v[LG_VAL_MAGNETIZATION_DENSITY2] = umag2 / p2(vol);
    v[LG_VAL_MAGNETIZATION4] = 3 * p2(umag2) - 2 * umag4;
    v[LG_VAL_MAGNETIZATION_DENSITY4] = (3 * p2(umag2) - 2 * umag4) / p4(vol);
    v[LG_VAL_SUSCEPTIBILITY] = chi(s, nop, umag, umag2);
    v[LG_VAL_GEN_MAGNETIZATION2] = usize2;
    v[LG_VAL_GEN_MAGNETIZATION_DENSITY2] = usize2 / p2(vol);
    v[LG_VAL_GEN_MAGNETIZATION4] = 3 * p2(usize2) - 2 * usize4;
    v[LG_VAL_GEN_MAGNETIZATION_DENSITY4] = (3 * p2(usize2) - 2 * usize4) / p4(vol);
    v[LG_VAL_GEN_SUSCEPTIBILITY] = chi(s, nop, usize, usize2);
    v[LG_VAL_STAG_MAGNETIZATION] = 0.0;
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY] = 0.0;
    v[LG_VAL_ABS_STAG_MAGNETIZATION] = std::fabs(smag0);
    v[LG_VAL_ABS_STAG_MAGNETIZATION_DENSITY] = std::fabs(smag0) / vol;
    v[LG_VAL_STAG_MAGNETIZATION2] = smag2;
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY2] = smag2 / p2(vol);
    v[LG_VAL_STAG_MAGNETIZATION4] = 3 * p2(smag2) - 2 * smag4;
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY4] = (3 * p2(smag2) - 2 * smag4) / p4(vol);
    v[LG_VAL_STAG_SUSCEPTIBILITY] = chi(s, nop, smag, smag2);
    v[LG_VAL_GEN_STAG_MAGNETIZATION2] = ssize2;
    v[LG_VAL_GEN_STAG_MAGNETIZATION_DENSITY2] = ssize2 / p2(vol);
    v[LG_VAL_GEN_STAG_MAGNETIZATION4] = 3 * p2(ssize2) - 2 * ssize4;
    v[LG_VAL_GEN_STAG_MAGNETIZATION_DENSITY4] = (3 * p2(ssize2) - 2 * ssize4) / p4(vol);
    v[LG_VAL_GEN_STAG_SUSCEPTIBILITY] = chi(s, nop, ssize, ssize2);
  } else {
    const double umag = i64(r[R_M0]) / 2, smag = i64(r[R_SM0]) / 2;
    const double umag_a = i64(r[R_MA]) * u1 / 2, smag_a = i64(r[R_SMA]) * u1 / 2;
    v[LG_VAL_MAGNETIZATION] = umag;
    v[LG_VAL_MAGNETIZATION_DENSITY] = umag / vol;
    v[LG_VAL_ABS_MAGNETIZATION] = std::fabs(umag);
    v[LG_VAL_ABS_MAGNETIZATION_DENSITY] = std::fabs(umag) / vol;
    v[LG_VAL_MAGNETIZATION2] = p2(umag);
    v[LG_VAL_MAGNETIZATION_DENSITY2] = p2(umag / vol);
    v[LG_VAL_MAGNETIZATION4] = p4(umag);
    v[LG_VAL_MAGNETIZATION_DENSITY4] = p4(umag / vol);
    v[LG_VAL_SUSCEPTIBILITY] = chi(s, nop, p2(umag_a), p2(umag));
    v[LG_VAL_STAG_MAGNETIZATION] = smag;
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY] = smag / vol;
    v[LG_VAL_ABS_STAG_MAGNETIZATION] = std::fabs(smag);
    v[LG_VAL_ABS_STAG_MAGNETIZATION_DENSITY] = std::fabs(smag) / vol;
    v[LG_VAL_STAG_MAGNETIZATION2] = p2(smag);
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY2] = p2(smag / vol);
    v[LG_VAL_STAG_MAGNETIZATION4] = p4(smag);
    v[LG_VAL_STAG_MAGNETIZATION_DENSITY4] = p4(smag / vol);
    v[LG_VAL_STAG_SUSCEPTIBILITY] = chi(s, nop, p2(smag_a), p2(smag));
  }
  v[LG_VAL_STIFFNESS] = raw[RAW_STIFF];
  for (int i = 0; i < LG_NUM_VALUES; ++i)
    if (!(mask >> i & 1)) v[i] = std::nan("");
}

extern "C" const char* lg_value_name(int i) {
  static const char* names[LG_NUM_VALUES] = {
      "Temperature", "Inverse Temperature", "Volume", "Number of Sites", "Number of Clusters",
      "Energy", "Energy Density", "Energy^2",
      "Magnetization", "Magnetization Density", "|Magnetization|", "|Magnetization Density|",
      "Magnetization^2", "Magnetization Density^2", "Magnetization^4", "Magnetization Density^4",
      "Susceptibility",
      "Generalized Magnetization^2", "Generalized Magnetization Density^2",
      "Generalized Magnetization^4", "Generalized Magnetization Density^4",
      "Generalized Susceptibility",
      "Staggered Magnetization", "Staggered Magnetization Density", "|Staggered Magnetization|",
      "|Staggered Magnetization Density|", "Staggered Magnetization^2",
      "Staggered Magnetization Density^2", "Staggered Magnetization^4",
      "Staggered Magnetization Density^4", "Staggered Susceptibility",
      "Generalized Staggered Magnetization^2", "Generalized Staggered Magnetization Density^2",
      "Generalized Staggered Magnetization^4", "Generalized Staggered Magnetization Density^4",
      "Generalized Staggered Susceptibility", "Stiffness"};
  return (i >= 0 && i < LG_NUM_VALUES) ? names[i] : "";
}

void BinAcc::push(double x) {
  ++count;
  sum += x;
  sum2 += x * x;
  cur += x;
  if (++fill == bin_size) {
    bins.push_back(cur / (double)bin_size);
    cur = 0;
    fill = 0;
    if (bins.size() == 128) {
      for (size_t i = 0; i < 64; ++i) bins[i] = 0.5 * (bins[2 * i] + bins[2 * i + 1]);
      bins.resize(64);
      bin_size *= 2;
    }
  }
}

static double bins_error(const std::vector<double>& b) {
  const size_t n = b.size();
  if (n < 2) return INFINITY;
  double m = 0;
  for (double x : b) m += x;
  m /= (double)n;
  double v = 0;
  for (double x : b) v += (x - m) * (x - m);
  return std::sqrt(v / (double)(n - 1) / (double)n);
}

double BinAcc::error() const { return bins_error(bins); }

double BinAcc::tau() const {
  if (count < 2) return 0;
  const double m = mean();
  const double var = std::max(0.0, sum2 / (double)count - m * m);
  const double naive = std::sqrt(var / (double)(count - 1));
  const double e = error();
  if (!(naive > 0) || !std::isfinite(e)) return 0;
  return 0.5 * ((e / naive) * (e / naive) - 1);
}

void ChainAcc::push(const ChainSpec& s, const uint64_t* rec) {
  double v[NUM_RAW];
  record_values(s, rec, v);
  for (int i = 0; i < NUM_RAW; ++i) raw[i].push(v[i]);
}

// jackknife over aligned bins of f(a, b)
template <class F>
static void jackknife2(const BinAcc& A, const BinAcc& B, F f, double* mean, double* err) {
  const size_t n = std::min(A.bins.size(), B.bins.size());
  *mean = f(A.mean(), B.mean());
  if (n < 2) { *err = INFINITY; return; }
  double sa = 0, sb = 0;
  for (size_t i = 0; i < n; ++i) { sa += A.bins[i]; sb += B.bins[i]; }
  std::vector<double> jk(n);
  double m = 0;
  for (size_t i = 0; i < n; ++i) {
    jk[i] = f((sa - A.bins[i]) / (double)(n - 1), (sb - B.bins[i]) / (double)(n - 1));
    m += jk[i];
  }
  m /= (double)n;
  double v = 0;
  for (double x : jk) v += (x - m) * (x - m);
  *err = std::sqrt((double)(n - 1) / (double)n * v);
}

void ChainAcc::report(const ChainSpec& s, lg_obs* out) const {
  std::memset(out, 0, sizeof(*out));
  const double V = (double)s.volume, beta = s.beta;
  out->count = (uint64_t)raw[RAW_E].count;
  out->beta = beta;
  out->volume = V;
  out->improved = s.improved ? 1 : 0;
  auto put = [&](int o, const BinAcc& a, double scale) {
    out->mean[o] = a.mean() * scale;
    out->error[o] = a.error() * scale;
    out->tau[o] = a.tau();
  };
  put(LG_OBS_ENERGY, raw[RAW_E], 1.0);
  put(LG_OBS_ENERGY_DENSITY, raw[RAW_E], 1.0 / V);
  put(LG_OBS_ENERGY2, raw[RAW_E2], 1.0);
  put(LG_OBS_MAGNETIZATION, raw[RAW_M], 1.0);
  put(LG_OBS_ABS_MAGNETIZATION, raw[RAW_ABSM], 1.0);
  put(LG_OBS_MAGNETIZATION2, raw[RAW_M2], 1.0);
  put(LG_OBS_MAGNETIZATION4, raw[RAW_M4], 1.0);
  put(LG_OBS_SUSCEPTIBILITY, raw[RAW_CHI], 1.0);
  put(LG_OBS_STAG_MAGNETIZATION2, raw[RAW_SM2], 1.0);
  put(LG_OBS_STAG_MAGNETIZATION4, raw[RAW_SM4], 1.0);
  put(LG_OBS_STAG_SUSCEPTIBILITY, raw[RAW_SCHI], 1.0);
  put(LG_OBS_GEN_MAGNETIZATION2, raw[RAW_GM2], 1.0);
  put(LG_OBS_GEN_SUSCEPTIBILITY, raw[RAW_GCHI], 1.0);
  put(LG_OBS_NUM_CLUSTERS, raw[RAW_NC], 1.0);
  put(LG_OBS_NUM_OPERATORS, raw[RAW_NOP], 1.0);
  put(LG_OBS_STIFFNESS, raw[RAW_STIFF], 1.0);
  // evaluators: energy.h:89-101, susceptibility.h:340-374
  double m, e;
  jackknife2(raw[RAW_E], raw[RAW_E2], [&](double a, double b) { return beta * beta * (b - a * a) / V; }, &m, &e);
  out->mean[LG_OBS_SPECIFIC_HEAT] = m;
  out->error[LG_OBS_SPECIFIC_HEAT] = e;
  jackknife2(raw[RAW_M2], raw[RAW_M4], [](double a, double b) { return b != 0 ? a * a / b : 0.0; }, &m, &e);
  out->mean[LG_OBS_BINDER] = m;
  out->error[LG_OBS_BINDER] = e;
  jackknife2(raw[RAW_SM2], raw[RAW_SM4], [](double a, double b) { return b != 0 ? a * a / b : 0.0; }, &m, &e);
  out->mean[LG_OBS_STAG_BINDER] = m;
  out->error[LG_OBS_STAG_BINDER] = e;
}

extern "C" const char* lg_obs_name(int i) {
  static const char* names[LG_NUM_OBS] = {
      "Energy", "Energy Density", "Energy^2", "Specific Heat", "Magnetization",
      "|Magnetization|", "Magnetization^2", "Magnetization^4", "Susceptibility",
      "Staggered Magnetization^2", "Staggered Magnetization^4", "Staggered Susceptibility",
      "Generalized Magnetization^2", "Generalized Susceptibility", "Number of Clusters",
      "Number of Operators", "Binder Ratio of Magnetization",
      "Binder Ratio of Staggered Magnetization", "Stiffness"};
  return (i >= 0 && i < LG_NUM_OBS) ? names[i] : "";
}

// ---------------------------------------------------------------------------------------------
// Checkpoint: the worker's save/load content (path_integral.C:111-124: mcs, spins, operators).
// Layout (little endian): "LGCK" u32 version, u32 dim, u32 L, u64 mcs, u64 n_ops,
// N x u8 spins, n_ops x (i32 bond, f64 time), u64 checksum of everything before it.  Version 3:
// the path-integral form, its off-diagonal operators with their times.  Version 4: the SSE form
// (sse.C save: mcs, spins, operators), every operator of the string as bond << 1 | off-diagonal,
// with (index + 1/2) / n_ops as its time (the order).
// The checksum is blocked so that several threads can compute it: FNV-1a (64-bit) of each 1 MiB
// block (over its 64-bit little-endian words, then its remaining bytes), then FNV-1a of those
// block hashes in order.
// ---------------------------------------------------------------------------------------------
static uint64_t fnv1a(const uint8_t* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {  // 64-bit little-endian words (8x fewer dependent multiplies)
    uint64_t w = 0;
    for (int k = 7; k >= 0; --k) w = (w << 8) | p[i + k];
    h ^= w;
    h *= 1099511628211ull;
  }
  for (; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
  return h;
}

size_t checkpoint_blocks(size_t size) {
  const size_t n = size < 8 ? 0 : size - 8;
  return (n + CHECKPOINT_BLOCK - 1) / CHECKPOINT_BLOCK;
}

uint64_t checkpoint_block_hash(const uint8_t* buf, size_t size, size_t block) {
  const size_t n = size < 8 ? 0 : size - 8;
  const size_t b0 = block * CHECKPOINT_BLOCK;
  if (b0 >= n) return 0;
  return fnv1a(buf + b0, std::min(CHECKPOINT_BLOCK, n - b0));
}

uint64_t checkpoint_combine(const uint64_t* block_hash, size_t nblocks) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < nblocks; ++i) {
    h ^= block_hash[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t checkpoint_checksum(const uint8_t* buf, size_t size) {
  const size_t nb = checkpoint_blocks(size);
  std::vector<uint64_t> h(nb);
  for (size_t i = 0; i < nb; ++i) h[i] = checkpoint_block_hash(buf, size, i);
  return checkpoint_combine(h.data(), nb);
}

uint64_t checkpoint_stored_checksum(const uint8_t* buf, size_t size) {
  uint64_t h = 0;
  if (buf && size >= 8) std::memcpy(&h, buf + size - 8, 8);
  return h;
}

bool checkpoint_checksum_ok(const uint8_t* buf, size_t size) {
  if (!buf || size < 8) return false;
  return checkpoint_stored_checksum(buf, size) == checkpoint_checksum(buf, size);
}

void checkpoint_encode(const ChainSpec& s, const std::vector<int32_t>& spins,
                       const std::vector<int32_t>& bonds, const std::vector<double>& times,
                       std::vector<uint8_t>& blob) {
  const size_t head = 4 + 4 + 4 + 4 + 8 + 8;
  blob.resize(head + spins.size() + 12 * bonds.size() + 8);
  uint8_t* p = blob.data();
  const uint32_t ver = s.sse ? CHECKPOINT_VERSION_SSE : CHECKPOINT_VERSION_PI, dim = (uint32_t)s.dim,
                 L = (uint32_t)s.L;
  const uint64_t mcs = s.mcs, n = bonds.size();
  std::memcpy(p, "LGCK", 4);
  std::memcpy(p + 4, &ver, 4);
  std::memcpy(p + 8, &dim, 4);
  std::memcpy(p + 12, &L, 4);
  std::memcpy(p + 16, &mcs, 8);
  std::memcpy(p + 24, &n, 8);
  p += head;
  for (int x : spins) *p++ = (uint8_t)(x & 1);
  for (size_t i = 0; i < bonds.size(); ++i, p += 12) {
    std::memcpy(p, &bonds[i], 4);
    std::memcpy(p + 4, &times[i], 8);
  }
  const uint64_t h = checkpoint_checksum(blob.data(), blob.size());
  std::memcpy(p, &h, 8);
}

int checkpoint_header(const ChainSpec& s, const uint8_t* buf, size_t size, uint64_t* nops,
                      uint64_t* mcs) {
  const size_t head = CHECKPOINT_HEAD;
  if (!buf || size < head + 8) return lg_fail(LG_ECORRUPT, "checkpoint too short");
  if (std::memcmp(buf, "LGCK", 4) != 0) return lg_fail(LG_ECORRUPT, "not a checkpoint");
  uint32_t ver, dim, L;
  uint64_t m, n;
  std::memcpy(&ver, buf + 4, 4);
  std::memcpy(&dim, buf + 8, 4);
  std::memcpy(&L, buf + 12, 4);
  std::memcpy(&m, buf + 16, 8);
  std::memcpy(&n, buf + 24, 8);
  if (ver != (s.sse ? CHECKPOINT_VERSION_SSE : CHECKPOINT_VERSION_PI))
    return lg_fail(LG_ECORRUPT, "checkpoint version %u", ver);
  if ((int)dim != s.dim || (int)L != s.L) return lg_fail(LG_ECORRUPT, "checkpoint lattice mismatch");
  // n is checked against the size without multiplying it (a forged count must not wrap)
  const size_t fixed = head + (size_t)s.N + 8;
  if (size < fixed || (size - fixed) % 12 != 0 || n != (uint64_t)((size - fixed) / 12))
    return lg_fail(LG_ECORRUPT, "checkpoint size mismatch");
  *nops = n;
  *mcs = m;
  return LG_OK;
}

int checkpoint_decode(const ChainSpec& s, const uint8_t* buf, size_t size,
                      std::vector<int32_t>& spins, std::vector<int32_t>& bonds,
                      std::vector<double>& times, uint64_t* mcs) {
  if (!buf || size < CHECKPOINT_HEAD + 8) return lg_fail(LG_ECORRUPT, "checkpoint too short");
  if (!checkpoint_checksum_ok(buf, size)) return lg_fail(LG_ECORRUPT, "checkpoint checksum mismatch");
  uint64_t n = 0, m = 0;
  int rc = checkpoint_header(s, buf, size, &n, &m);
  if (rc) return rc;
  const uint8_t* p = buf + CHECKPOINT_HEAD;
  spins.resize(s.N);
  for (int i = 0; i < s.N; ++i) spins[i] = p[i];
  p += s.N;
  bonds.resize(n);
  times.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    std::memcpy(&bonds[i], p, 4);
    std::memcpy(&times[i], p + 4, 8);
    p += 12;
    if (bonds[i] < 0 || bonds[i] >= (s.sse ? 2 : 1) * s.NB || !(times[i] >= 0.0 && times[i] < 1.0))
      return lg_fail(LG_ECORRUPT, "checkpoint operator %llu out of range", (unsigned long long)i);
  }
  *mcs = m;
  return LG_OK;
}
