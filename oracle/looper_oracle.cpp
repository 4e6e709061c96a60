// CPU ORACLE — test infrastructure only.
//
// This file is the checker for the GPU loop-cluster update. It is never part of the product:
// only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
//
// It restates, serially and in plain C++, the continuous-imaginary-time loop-cluster sweep of
// looper's path-integral worker (path_integral.C:355-864) for S=1/2 XXZ models with a uniform
// longitudinal field on periodic chain / square / simple-cubic lattices:
//
//   * graph weights ............ weight_impl.h:282-315 (xyz helper, default; Jx == Jy here)
//   * graph choice / reconnect .. graph_impl.h:255-328 (xxz_bond_graph_type), :489-494 (loop_*)
//   * insertion/removal ........ path_integral.C:403-577 (time-ordered merge, is_compatible)
//   * union-find ............... union_find.h:57-82 (node), :163-172 (root_index_ph),
//                                 :242-284 (unify_pathhalving; weighted or deterministic root)
//   * temporal closure ......... path_integral.C:584-589
//   * cluster ids .............. union_find.h:324-343 (set_id, copy_id), path_integral.C:625-648
//   * improved estimators ...... susceptibility.h:96-156 (estimate), :158-198 (collector)
//   * field weight / flip ...... cluster.h:54-59, path_integral.C:780-825
//   * normal estimators ........ susceptibility.h:258-337 (field case)
//   * energy ................... path_integral.C:849-860, energy.h:76-84
//
// Two random sources are provided.
//
//  (1) "standalone" mode restates standalone/loop.C:39-195 (Heisenberg AF chain) with the very
//      same std::mt19937 / <random> consumption order, so its output is bit-identical to the
//      golden standalone/loop.op.  This pins the restated cluster machinery against the reference.
//
//  (2) "philox" mode replaces the reference's single exponential stream + alias sampler
//      (path_integral.C:412-425, graph_impl.h:678-681) by per-bond Poisson streams drawn from a
//      counter-based Philox4x32-10 generator.  By the superposition property of Poisson processes
//      this is the same distribution of diagonal proposals.  The cluster-flip coin of each
//      cluster is keyed by a canonical segment index instead of being drawn sequentially.  Time
//      gaps and flip probabilities are evaluated with small float formulas written out below
//      (independently of the GPU code) and imaginary times are held as exact FP64 values on a
//      2^-52 grid; segment lengths are integrated in 2^-40 fixed point.  In this mode the oracle
//      and the GPU path see identical random numbers, so their trajectories agree bit for bit.
//
// Everything is exported through a small extern "C" surface for ctypes.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace orc {

// ----------------------------------------------------------------------------------------------
// Numerics shared (by specification, not by code) with the GPU path.
// ----------------------------------------------------------------------------------------------

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11).  Multipliers and Weyl key increments are those of the paper.
static const uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
static const uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;

static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PH_M0 * c[0];
    uint64_t p1 = (uint64_t)PH_M1 * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += PH_W0; k1 += PH_W1;
  }
}

// Stream tags (third counter word).
enum { TAG_PROPOSAL = 1, TAG_OFFDIAG = 2, TAG_FLIP = 3, TAG_SPIN = 4, TAG_PERM = 6, TAG_TAIL = 7 };

static void rng4(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t out[4]) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
}

static inline float bits_f(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }
static inline uint32_t f_bits(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
static inline double bits_d(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static inline uint64_t d_bits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }

// Open-interval uniform float: (2x+1) * 2^-24 with x the top 23 bits of w.  Exact.
static inline float uniform_open(uint32_t w) {
  return (float)(((w >> 9) << 1) | 1u) * 5.9604644775390625e-8f;
}

// The uniform of an exponential gap (-ln U mean gaps): (2x+1) 2^-24 from the top 23 bits x of w,
// refined in the lowest bin (x = 0, U < 2^-23) by the top 23 bits t of a second word `tail`:
// U = (2t+1) 2^-47, so that the gap's tail reaches -ln 2^-47 = 32.6 mean gaps.
static inline float gap_uniform(uint32_t w, uint32_t tail) {
  return (w >> 9) ? uniform_open(w) : uniform_open(tail) * 1.1920928955078125e-7f;
}

// Natural log for u in (0,1): u = m 2^e with m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
// ln m = 2s + s z (2/3 + z (2/5 + z (2/7 + z 2/9))), z = s^2 (the atanh series), and
// ln u = e ln2_hi + (e ln2_lo + ln m).  Only IEEE +,-,*,/ and fmaf are used, so every
// conforming platform returns the same bits.
static float log_spec(float u) {
  uint32_t b = f_bits(u);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  uint32_t mb = (b & 0x7FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) { mb -= 0x00800000u; e += 1; }
  float m = bits_f(mb);
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  float R = std::fmaf(z, 0.22222222f, 0.28571429f);
  R = std::fmaf(z, R, 0.4f);
  R = std::fmaf(z, R, 0.66666669f);
  R = z * R;
  float two_s = s + s;
  float lnm = std::fmaf(s, R, two_s);
  float ef = (float)e;
  float t = std::fmaf(ef, 1.42860677e-06f, lnm);
  return std::fmaf(ef, 0.693145752f, t);
}

// exp(x) for |x| <= 80: x = k ln2 + r, Taylor polynomial of degree 7 in r, times 2^k.
static float exp_spec(float x) {
  if (x > 80.0f) x = 80.0f;
  if (x < -80.0f) x = -80.0f;
  float kf = std::rint(x * 1.44269502f);
  float r = std::fmaf(-kf, 0.693145752f, x);
  r = std::fmaf(-kf, 1.42860677e-06f, r);
  float p = std::fmaf(r, 1.98412698e-04f, 1.38888889e-03f);
  p = std::fmaf(r, p, 8.33333377e-03f);
  p = std::fmaf(r, p, 4.16666679e-02f);
  p = std::fmaf(r, p, 0.166666672f);
  p = std::fmaf(r, p, 0.5f);
  p = std::fmaf(r, p, 1.0f);
  p = std::fmaf(r, p, 1.0f);
  int k = (int)kf;
  float scale = bits_f((uint32_t)(k + 127) << 23);
  return p * scale;
}

static const uint64_t FIX52_ONE = 1ull << 52;

// floor(g * 2^52) for a non-negative float g < 1, with the bits below the float's own
// resolution filled from `dither` (a uniform spread of the gap over its float ulp, so that
// times are continuous on the 2^-52 grid); *ge1 is set when g >= 1.
static uint64_t float_to_fix52(float g, uint64_t dither, bool* ge1) {
  uint32_t b = f_bits(g);
  *ge1 = false;
  uint32_t ex = (b >> 23) & 0xFFu;
  if (ex == 0) return 0;  // zero (or subnormal, < 2^-126): below the grid
  int e = (int)ex - 127;
  if (e >= 0) { *ge1 = true; return 0; }
  uint64_t m = (uint64_t)((b & 0x7FFFFFu) | 0x800000u);
  int sh = e + 29;
  if (sh < 0) return m >> (-sh);
  return (m << sh) | (dither & ((1ull << sh) - 1));
}

// Exact FP64 value of k * 2^-52 (k < 2^52).
static double fix52_to_double(uint64_t k) {
  if (k == 0) return 0.0;
  int p = 63 - __builtin_clzll(k);
  uint64_t mant = (k << (52 - p)) & ((1ull << 52) - 1);
  uint64_t ex = (uint64_t)(p - 52 + 1023);
  return bits_d((ex << 52) | mant);
}

// floor(t * 2^40) for t in [0, 1], from the FP64 bit pattern.
static int64_t time_fix40(double t) {
  if (t >= 1.0) return (int64_t)1 << 40;
  uint64_t b = d_bits(t);
  if (b == 0) return 0;
  int e = (int)((b >> 52) & 0x7FF) - 1023;
  uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
  int sh = 12 - e;
  if (sh >= 64) return 0;
  return (int64_t)(m >> sh);
}

// ----------------------------------------------------------------------------------------------
// Lattice: periodic hypercubic, real site = x + L*y + L*L*z, real bond = site*dim + d joins
// site -> site+e_d.  gauge = +1 on the even sublattice, -1 on the odd one (lattice.h:601 uses
// 2*parity-1).  Spin S = spin2/2 > 1/2 is represented by spin2 spin-1/2 virtual sites per real
// site, v = site*spin2 + a, and every real bond by the spin2^2 virtual bonds between the virtual
// sites of its two ends, b = rbond*spin2^2 + a*spin2 + a' (the virtual graph of lattice.h); each
// virtual site has its real site's gauge, each virtual bond its real bond's direction.
// ----------------------------------------------------------------------------------------------
struct lattice {
  int dim = 1, L = 0, N = 0, NB = 0, NR = 0, spin2 = 1;
  std::vector<int> s0, s1, gauge, bdir;
  bool bipartite = true;
  void build(int d, int l, int sp2 = 1) {
    dim = d; L = l; spin2 = sp2;
    NR = 1; for (int i = 0; i < dim; ++i) NR *= L;
    N = NR * spin2;
    const int q = spin2 * spin2;
    NB = NR * dim * q;
    s0.resize(NB); s1.resize(NB); gauge.resize(N); bdir.resize(NB);
    for (int s = 0; s < NR; ++s) {
      int x[3] = {0, 0, 0}, r = s, par = 0;
      for (int i = 0; i < dim; ++i) { x[i] = r % L; r /= L; par += x[i]; }
      for (int a = 0; a < spin2; ++a) gauge[s * spin2 + a] = (par % 2 == 0) ? 1 : -1;
      for (int i = 0; i < dim; ++i) {
        int y[3] = {x[0], x[1], x[2]};
        y[i] = (y[i] + 1) % L;
        int t = 0; for (int j = dim - 1; j >= 0; --j) t = t * L + y[j];
        for (int a = 0; a < spin2; ++a)
          for (int a2 = 0; a2 < spin2; ++a2) {
            const int b = (s * dim + i) * q + a * spin2 + a2;
            s0[b] = s * spin2 + a; s1[b] = t * spin2 + a2; bdir[b] = i;
          }
      }
    }
    bipartite = (L % 2 == 0);
  }
};

// Imaginary-time boundary of a real site with spin2 > 1 virtual sites (path_integral.C:590-613,
// permutation.h:91-111): the bottom of virtual site a joins the top of pair[a], and both carry
// the same spin.  For each spin value c the tops with spin c, in index order, are shuffled by
// Fisher-Yates (step i of the shuffle, from the last position down, swaps position i with
// j = floor(w (i+1) / 2^32)), where step k of sector c takes Philox word 8c + k of the key
// (seed, sweep, real site, TAG_PERM).  The bottoms with spin c, in index order, take the
// shuffled tops in order: a uniform matching within each spin sector, like the reference's
// partitioned random shuffle.  Returns false if the sectors differ in size.
static bool boundary_matching(uint64_t seed, uint32_t sweep, uint32_t rs, int spin2,
                              const int* bottom, const int* top, int* pair) {
  for (int c = 0; c < 2; ++c) {
    int T[8], B[8], nt = 0, nb = 0;
    for (int a = 0; a < spin2; ++a) {
      if (top[a] == c) T[nt++] = a;
      if (bottom[a] == c) B[nb++] = a;
    }
    if (nt != nb) return false;
    for (int i = nt - 1, k = 0; i >= 1; --i, ++k) {
      const int q = 8 * c + k;
      uint32_t w[4];
      rng4(seed, sweep, rs, TAG_PERM, (uint32_t)(q >> 2), w);
      const int j = (int)(((uint64_t)w[q & 3] * (uint64_t)(i + 1)) >> 32);
      const int tmp = T[i]; T[i] = T[j]; T[j] = tmp;
    }
    for (int k = 0; k < nb; ++k) pair[B[k]] = T[k];
  }
  return true;
}

// ----------------------------------------------------------------------------------------------
// Graph weights for one S=1/2 XXZ bond: restates weight_impl.h:282-315 with Jx == Jy == Jxy
// (Jm = 0), which is the default weight helper (weight.h:40-42).  v[g] for the xxz graphs
// g = 0..3 (graph_impl.h:255-328).
// ----------------------------------------------------------------------------------------------
struct bond_weight { double v[4] = {0, 0, 0, 0}; double W = 0, offset = 0; };

static inline double crop_0(double x) { return x > 0 ? x : 0; }
static inline double crop_01(double x) { return x < 0 ? 0 : (x > 1 ? 1 : x); }

static bond_weight make_weight(double jxy, double jz, double force_scatter) {
  bond_weight w;
  double jp = std::fabs(jxy);
  double a = crop_01(force_scatter);
  if (jp + std::fabs(jz) > 1e-12) {
    if (jp - jz > 2 * a * jp) {
      w.v[0] = crop_0(std::min(jp / 2, (jp + jz) / 4));
      w.v[1] = crop_0(std::min(jp / 2, (jp - jz) / 4));
      w.v[2] = crop_0(-(jp - jz) / 2);
      w.v[3] = crop_0(-(jp + jz) / 2);
    } else {
      w.v[0] = (1 - a) * jp / 2;
      w.v[1] = a * jp / 2;
      w.v[2] = -((1 - 2 * a) * jp - jz) / 2;
      w.v[3] = 0;
    }
  }
  w.W = w.v[0] + w.v[1] + w.v[2] + w.v[3];
  w.offset = w.W / 2;
  return w;
}

static uint64_t prob_u32(double p) {  // round(p * 2^32) clamped to [0, 2^32]
  if (!(p > 0)) return 0;
  if (p >= 1) return 1ull << 32;
  double x = std::floor(p * 4294967296.0 + 0.5);
  return (uint64_t)x;
}

// ----------------------------------------------------------------------------------------------
// Union-find over cluster fragments: restates union_find.h:57-82 (node: parent+1 / -weight) and
// :163-172, :242-284 (path halving, weighted root by default, smaller index when deterministic).
// ----------------------------------------------------------------------------------------------
struct uf {
  std::vector<int> parent;  // >0: parent+1 ; <=0: -weight (root)
  std::vector<int> id;
  bool deterministic = false;
  void reset(int n) { parent.assign(n, -1); id.assign(n, 0); }
  int add() { parent.push_back(-1); id.push_back(0); return (int)parent.size() - 1; }
  bool is_root(int g) const { return parent[g] <= 0; }
  int par(int g) const { return parent[g] - 1; }
  int weight(int g) const { return -parent[g]; }
  int root_ph(int g) {
    if (is_root(g)) return g;
    while (true) {
      int p = par(g);
      if (is_root(p)) return p;
      parent[g] = parent[p];  // set_parent(parent of p)
      g = p;
    }
  }
  int root(int g) const { while (!is_root(g)) g = par(g); return g; }
  int unify(int g0, int g1) {
    int r0 = root_ph(g0), r1 = root_ph(g1);
    if (r0 != r1) {
      if (!deterministic) { if (weight(r0) < weight(r1)) std::swap(r0, r1); }
      else { if (r0 > r1) std::swap(r0, r1); }
      parent[r0] = -(weight(r0) + weight(r1));
      parent[r1] = r0 + 1;
    }
    return r0;
  }
  int set_ids() {  // set_id over [0,n) then copy_id
    int nc = 0, n = (int)parent.size();
    for (int i = 0; i < n; ++i) if (is_root(i)) id[i] = nc++;
    for (int i = 0; i < n; ++i) id[i] = id[root(i)];
    return nc;
  }
};

// ----------------------------------------------------------------------------------------------
// Chain (one Markov chain) in philox mode.
// ----------------------------------------------------------------------------------------------
struct op_t {
  int bond;
  double t;
  int offdiag;  // 0 diagonal, 1 off-diagonal
  int g;        // graph 0..3
};

// Per-sweep measurement record: every entry is an exact integer function of the configuration.
// u128 quantities are stored as (lo, hi) pairs.
enum {
  R_NOP = 0, R_NC, R_M0, R_SM0,            // counts; sum of (1-2c) and gauge*(1-2c) at t=0
  R_M0SQ, R_N0SQ, R_SM0SQ, R_SN0SQ,        // sum over clusters of squares (u64)
  R_M0Q_LO, R_M0Q_HI, R_N0Q_LO, R_N0Q_HI,  // sum over clusters of 4th powers (u128)
  R_SM0Q_LO, R_SM0Q_HI, R_SN0Q_LO, R_SN0Q_HI,
  R_LSQ_LO, R_LSQ_HI, R_MSQ_LO, R_MSQ_HI,  // sum over clusters of time-integrated squares (u128)
  R_SLSQ_LO, R_SLSQ_HI, R_SMSQ_LO, R_SMSQ_HI,
  R_FLD,                                   // sum_c (flip ? -M_c : M_c)   (2^-40 units)
  R_MA, R_SMA,                             // sum over all segments of (1-2c) len, gauge*(1-2c) len
  R_WSQ,                                   // sum over clusters and directions of winding^2
  R_W0, R_W1, R_W2,                        // total winding per direction (signed)
  R_WORDS = 32
};

typedef unsigned __int128 u128;

static inline void add128(uint64_t* rec, int lo, u128 v) {
  u128 cur = ((u128)rec[lo + 1] << 64) | rec[lo];
  cur += v;
  rec[lo] = (uint64_t)cur;
  rec[lo + 1] = (uint64_t)(cur >> 64);
}

struct chain_t {
  lattice lat;
  bond_weight bw;
  double beta = 1, h = 0;
  uint64_t seed = 0;
  bool field = false;
  bool deterministic_uf = false;
  // derived
  uint64_t T0 = 0, T1 = 0, T2 = 0, Poff = 0;
  float inv_rate = 0;
  float flip_coef = 0;
  // state
  std::vector<int> spins;   // 0 up, 1 down, at tau = 0
  std::vector<op_t> ops;    // operator string, time ordered (after the last flip)
  uint32_t sweep = 0;
  // last sweep (cluster-construction configuration, before the flip)
  std::vector<int> last_spins;
  std::vector<op_t> last_ops;     // with graphs, pre-flip types
  std::vector<int> last_labels;   // reference fragment ids (sites, then g=0 vertices)
  int last_nfrag = 0, last_nc = 0;
  std::vector<uint64_t> records;  // R_WORDS per sweep
  int status = 0;                 // 1: a boundary had spin sectors of different sizes

  void init_derived() {
    double W = bw.W;
    if (W > 0) {
      T0 = prob_u32(bw.v[0] / W);
      T1 = prob_u32((bw.v[0] + bw.v[1]) / W);
      T2 = prob_u32((bw.v[0] + bw.v[1] + bw.v[2]) / W);
      inv_rate = (float)(1.0 / (beta * W));
    }
    double s01 = bw.v[0] + bw.v[1];
    Poff = prob_u32(s01 > 0 ? bw.v[0] / s01 : 1.0);
    flip_coef = (float)(beta * h * std::ldexp(1.0, -40));
  }

  int graph_of(uint32_t w) const {
    return (int)(w >= T0) + (int)(w >= T1) + (int)(w >= T2);
  }

  void sweep_once() {
    const int N = lat.N, NB = lat.NB;
    // ---- diagonal proposals: a Poisson stream per bond (rate beta*W_b) ----
    struct prop { uint64_t tq; int b; int g; };  // generated in (b, k) order, k the draw index
    std::vector<prop> props;
    if (bw.W > 0) {
      for (int b = 0; b < NB; ++b) {
        uint64_t tq = 0;
        uint32_t w[4];
        for (int k = 0;; ++k) {
          if ((k & 1) == 0) rng4(seed, sweep, (uint32_t)b, TAG_PROPOSAL, (uint32_t)(k >> 1), w);
          uint32_t wu = w[(k & 1) * 2], wg = w[(k & 1) * 2 + 1];
          uint32_t tail = 0;
          if ((wu >> 9) == 0) {
            uint32_t t4[4];
            rng4(seed, sweep, (uint32_t)b, TAG_TAIL, (uint32_t)k, t4);
            tail = t4[0];
          }
          float gap = -log_spec(gap_uniform(wu, tail)) * inv_rate;
          bool ge1;
          uint64_t dither = ((uint64_t)(wu & 0x1FFu) << 16) | (wg & 0xFFFFu);
          uint64_t q = float_to_fix52(gap, dither, &ge1);
          if (ge1) break;
          tq += q;
          if (tq >= FIX52_ONE) break;
          props.push_back({tq, b, graph_of(wg)});
        }
      }
    }
    // Order (tq, b, k).  The stream is generated bond by bond and, within a bond, in k order, so
    // a stable sort by tq alone gives that order.  Times are uniform on [0, 1) (52-bit), so: a
    // stable scatter by the top 8 bits, the same inside each of those buckets by the next 8, and
    // a stable insertion sort of each of the small buckets left.
    {
      std::vector<prop> tmp(props.size());
      size_t start[257];
      auto scatter = [&](const prop* src, prop* dst, size_t n, int sh, size_t* st) {
        std::memset(st, 0, 257 * sizeof(size_t));
        for (size_t i = 0; i < n; ++i) ++st[((src[i].tq >> sh) & 0xFFu) + 1];
        for (int k = 0; k < 256; ++k) st[k + 1] += st[k];
        size_t pos[256];
        std::memcpy(pos, st, sizeof(pos));
        for (size_t i = 0; i < n; ++i) dst[pos[(src[i].tq >> sh) & 0xFFu]++] = src[i];
      };
      scatter(props.data(), tmp.data(), props.size(), 44, start);
      size_t sub[257];
      for (int k = 0; k < 256; ++k) {
        const size_t lo = start[k], n = start[k + 1] - lo;
        if (!n) continue;
        prop* dst = props.data() + lo;
        scatter(tmp.data() + lo, dst, n, 36, sub);
        for (int k2 = 0; k2 < 256; ++k2) {
          for (size_t i = sub[k2] + 1; i < sub[k2 + 1]; ++i) {
            const prop x = dst[i];
            size_t j = i;
            while (j > sub[k2] && dst[j - 1].tq > x.tq) { dst[j] = dst[j - 1]; --j; }
            dst[j] = x;
          }
        }
      }
    }
    // ---- old operators: keep the off-diagonal ones (path_integral.C:515-518) ----
    std::vector<op_t> old;
    for (auto& o : ops) if (o.offdiag) old.push_back(o);
    auto time_bond = [](const op_t& a, const op_t& b) {
      uint64_t ta = d_bits(a.t), tb = d_bits(b.t);
      if (ta != tb) return ta < tb;
      return a.bond < b.bond;
    };
    // usually already in order (the previous sweep wrote the string in time order)
    if (!std::is_sorted(old.begin(), old.end(), time_bond))
      std::stable_sort(old.begin(), old.end(), time_bond);

    // ---- merge in time order: insertion/removal + labeling (path_integral.C:484-566) ----
    std::vector<int> spins_c = spins;
    uf frag; frag.deterministic = deterministic_uf; frag.reset(N);
    std::vector<int> current(N);
    for (int s = 0; s < N; ++s) current[s] = s;
    std::vector<op_t> nops; nops.reserve(old.size() + props.size());
    std::vector<int> loop0, loop1, up0, up1;  // per new op: reconnect loops, upper fragments
    loop0.reserve(nops.capacity()); loop1.reserve(nops.capacity());
    up0.reserve(nops.capacity()); up1.reserve(nops.capacity());
    frag.parent.reserve(N + props.size()); frag.id.reserve(N + props.size());
    std::vector<int> cnt(N, 0);  // endpoints per site
    std::vector<int> ordinal(NB, 0);
    size_t ip = 0, io = 0;
    while (ip < props.size() || io < old.size()) {
      // An old operator goes first unless a proposal is strictly earlier (path_integral.C:486);
      // non-negative doubles order like their bit patterns.
      bool take_old;
      if (io >= old.size()) take_old = false;
      else if (ip >= props.size()) take_old = true;
      else take_old = d_bits(old[io].t) <= d_bits(fix52_to_double(props[ip].tq));
      op_t o;
      int s0, s1;
      if (!take_old) {
        const prop& p = props[ip++];
        s0 = lat.s0[p.b]; s1 = lat.s1[p.b];
        // xxz is_compatible: (g & 1) ^ c0 ^ c1   (graph_impl.h:257)
        if (!(((p.g & 1) ^ spins_c[s0] ^ spins_c[s1]) & 1)) continue;
        o.bond = p.b; o.t = fix52_to_double(p.tq); o.offdiag = 0; o.g = p.g;
      } else {
        o = old[io++];
        s0 = lat.s0[o.bond]; s1 = lat.s1[o.bond];
        // choose_offdiagonal (graph_impl.h:323-327)
        int i = ordinal[o.bond]++;
        uint32_t w[4];
        rng4(seed, sweep, (uint32_t)o.bond, TAG_OFFDIAG, (uint32_t)(i >> 2), w);
        o.g = ((uint64_t)w[i & 3] < Poff) ? 0 : 1;
        o.offdiag = 1;
        spins_c[s0] ^= 1; spins_c[s1] ^= 1;
      }
      // reconnect (graph_impl.h:280-295)
      int c0 = current[s0], c1 = current[s1], l0, l1;
      if (o.g & 2) {
        l0 = l1 = current[s0] = current[s1] = frag.unify(c0, c1);
      } else if (o.g == 0) {
        int f = frag.add();
        l0 = frag.unify(c0, c1);
        l1 = current[s0] = current[s1] = f;
      } else {
        l0 = c0; l1 = c1;
        current[s0] = c1; current[s1] = c0;
      }
      nops.push_back(o);
      loop0.push_back(l0); loop1.push_back(l1);
      up0.push_back(current[s0]); up1.push_back(current[s1]);
      ++cnt[s0]; ++cnt[s1];
    }
    // ---- temporal closure (path_integral.C:582-615) ----
    if (lat.spin2 == 1) {
      for (int s = 0; s < N; ++s) frag.unify(s, current[s]);
    } else {
      for (int rs = 0; rs < lat.NR; ++rs) {
        const int off = rs * lat.spin2;
        int pair[8];
        if (!boundary_matching(seed, sweep, (uint32_t)rs, lat.spin2, &spins[off], &spins_c[off], pair)) {
          status = 1;  // not a periodic configuration: each bottom keeps its own top
          for (int a = 0; a < lat.spin2; ++a) pair[a] = a;
        }
        for (int a = 0; a < lat.spin2; ++a) frag.unify(off + a, current[off + pair[a]]);
      }
    }
    int nc = frag.set_ids();

    last_spins = spins;
    last_ops = nops;
    last_nfrag = (int)frag.parent.size();
    last_nc = nc;
    last_labels = frag.id;

    // ---- per-site segment lists (site-major, time-minor; bottom segment first) ----
    std::vector<int64_t> base(N + 1, 0);
    for (int s = 0; s < N; ++s) base[s + 1] = base[s] + cnt[s] + 1;
    // Each site's endpoints in time order: ops are processed in time order, so appending in
    // processing order is already time order per site.  One flat array, site after site, with
    // what the segment walk needs of each endpoint.
    // nextfr: the fragment above the endpoint, later its cluster; wdir -1: no winding
    struct endpoint { int64_t t40; int nextfr; int offdiag; int wdir; };
    std::vector<int64_t> eoff(N + 1, 0);
    for (int s = 0; s < N; ++s) eoff[s + 1] = eoff[s] + cnt[s];
    std::vector<endpoint> E((size_t)eoff[N]);
    {
      std::vector<int64_t> cur(eoff.begin(), eoff.end() - 1);
      for (size_t i = 0; i < nops.size(); ++i) {
        const op_t& o = nops[i];
        const int64_t t40 = time_fix40(o.t);
        for (int side = 0; side < 2; ++side) {
          const int s = side ? lat.s1[o.bond] : lat.s0[o.bond];
          const bool src = lat.s0[o.bond] == s;
          endpoint& e = E[(size_t)cur[s]++];
          e.t40 = t40;
          e.nextfr = src ? up0[i] : up1[i];
          e.offdiag = o.offdiag;
          e.wdir = (src && !(o.g & 2)) ? lat.bdir[o.bond] : -1;
        }
      }
    }
    // cluster accumulators, one record per cluster
    struct cacc {
      int64_t key = INT64_MAX;
      int64_t L = 0, M = 0, SL = 0, SM = 0;
      int64_t n0 = 0, m0 = 0, sn0 = 0, sm0 = 0;
      // winding per direction (stiffness.h:82-130): the improved accumulator calls end_bs /
      // begin_bs for the source-site legs of every non-frozen bond vertex (measurement.h
      // improved_accumulator::end_b / begin_b, path_integral.C:697-709).  The lower leg's
      // cluster gains (1-2c) e_d with c the spin before the vertex, the upper leg's cluster
      // loses (1-2c') e_d with c' the spin after; d is the bond's direction (bond = site*dim + d).
      int64_t w[3] = {0, 0, 0};
    };
    std::vector<cacc> A(nc);
    // the cluster above each endpoint, in one pass of independent reads
    for (endpoint& e : E) e.nextfr = frag.id[e.nextfr];
    int64_t MA = 0, SMA = 0, M0tot = 0, SM0tot = 0;
    for (int s = 0; s < N; ++s) {
      int c = spins[s];
      int g = lat.gauge[s];
      int64_t tprev = 0;
      int cl = frag.id[s];
      const int ne = cnt[s];
      const endpoint* es = E.data() + eoff[s];
      for (int j = 0; j <= ne; ++j) {
        int64_t tnext;
        int nextcl = -1, nextc = c;
        if (j < ne) {
          tnext = es[j].t40;
          nextcl = es[j].nextfr;
          if (es[j].offdiag) nextc = c ^ 1;
          if (j + 8 < ne) __builtin_prefetch(&A[es[j + 8].nextfr]);
        } else {
          tnext = (int64_t)1 << 40;
        }
        cacc& a = A[cl];
        if (j < ne && es[j].wdir >= 0) {
          const int d = es[j].wdir;
          a.w[d] += 1 - 2 * c;                              // end_bs
          A[nextcl].w[d] -= 1 - 2 * nextc;                  // begin_bs
        }
        int64_t segidx = base[s] + j;
        if (segidx < a.key) a.key = segidx;
        int64_t len = tnext - tprev;
        int sg = 1 - 2 * c;
        a.L += len; a.M += sg * len; a.SL += g * len; a.SM += g * sg * len;
        MA += sg * len; SMA += g * sg * len;
        if (j == 0) {
          a.n0 += 1; a.m0 += sg; a.sn0 += g; a.sm0 += g * sg;
          M0tot += sg; SM0tot += g * sg;
        }
        tprev = tnext; c = nextc; cl = nextcl;
      }
    }
    // ---- flips (path_integral.C:780-803) ----
    std::vector<uint8_t> flip(nc);
    for (int cl = 0; cl < nc; ++cl) {
      uint32_t w[4];
      rng4(seed, sweep, (uint32_t)A[cl].key, TAG_FLIP, 0, w);
      if (!field) {
        flip[cl] = (w[0] < 0x80000000u) ? 1 : 0;
      } else {
        float x = (float)A[cl].M * flip_coef;
        float q = exp_spec(x);
        float u = uniform_open(w[0]);
        flip[cl] = (u * (1.0f + q) < 1.0f) ? 1 : 0;
      }
    }
    // ---- record ----
    std::vector<uint64_t> rec(R_WORDS, 0);
    rec[R_NOP] = nops.size();
    rec[R_NC] = (uint64_t)nc;
    rec[R_M0] = (uint64_t)M0tot;
    rec[R_SM0] = (uint64_t)SM0tot;
    int64_t fld = 0;
    for (int cl = 0; cl < nc; ++cl) {
      const cacc& a = A[cl];
      rec[R_M0SQ] += (uint64_t)(a.m0 * a.m0);
      rec[R_N0SQ] += (uint64_t)(a.n0 * a.n0);
      rec[R_SM0SQ] += (uint64_t)(a.sm0 * a.sm0);
      rec[R_SN0SQ] += (uint64_t)(a.sn0 * a.sn0);
      auto q4 = [](int64_t x) { u128 v = (u128)(uint64_t)(x * x); return v * v; };
      add128(rec.data(), R_M0Q_LO, q4(a.m0));
      add128(rec.data(), R_N0Q_LO, q4(a.n0));
      add128(rec.data(), R_SM0Q_LO, q4(a.sm0));
      add128(rec.data(), R_SN0Q_LO, q4(a.sn0));
      auto sq = [](int64_t x) { uint64_t v = (uint64_t)(x < 0 ? -x : x); return (u128)v * v; };
      add128(rec.data(), R_LSQ_LO, sq(a.L));
      add128(rec.data(), R_MSQ_LO, sq(a.M));
      add128(rec.data(), R_SLSQ_LO, sq(a.SL));
      add128(rec.data(), R_SMSQ_LO, sq(a.SM));
      fld += flip[cl] ? -a.M : a.M;
      for (int d = 0; d < 3; ++d) {
        const int64_t w = a.w[d];
        rec[R_WSQ] += (uint64_t)(w * w);
        rec[R_W0 + d] += (uint64_t)w;
      }
    }
    rec[R_FLD] = (uint64_t)fld;
    rec[R_MA] = (uint64_t)MA;
    rec[R_SMA] = (uint64_t)SMA;
    records.insert(records.end(), rec.begin(), rec.end());

    // ---- flip operators & spins (path_integral.C:805-825) ----
    for (size_t i = 0; i < nops.size(); ++i) {
      if (flip[frag.id[loop0[i]]] ^ flip[frag.id[loop1[i]]]) nops[i].offdiag ^= 1;
    }
    for (int s = 0; s < N; ++s) if (flip[frag.id[s]]) spins[s] ^= 1;
    ops.swap(nops);
    ++sweep;
  }
};

// ----------------------------------------------------------------------------------------------
// SSE chain: restates the stochastic-series-expansion loop worker (sse.C:180-371) for spin-S XXZ
// models without field (sse.C:123 refuses a longitudinal field), in philox mode; S > 1/2 on the
// virtual lattice of the path-integral chain.  The configuration is an ordered operator string with no
// times; operator code = bond << 1 | off-diagonal.  One sweep:
//   * diagonal update & labelling (sse.C:201-276): a walk over the old string; before every
//     operator (and once more at the end) an insertion is tried with probability
//     beta W_tot / (n + 1), n the running operator count, and tried again while accepted and
//     compatible; a diagonal operator is removed with probability n / (beta W_tot), otherwise its
//     graph is re-chosen (choose_diagonal, graph_impl.h:297-312); an off-diagonal one re-chooses
//     (choose_offdiagonal, :314-327).  Spins propagate and fragments reconnect (:280-295).
//   * closure of every site's top onto its bottom (sse.C:275-277); for S > 1/2 the bottom of
//     virtual site a joins the top of pair[a], a matching within each spin sector
//     (sse.C:278-296, partitioned_random_shuffle), drawn as in the path-integral chain
//     (boundary_matching)
//   * cluster ids (sse.C:305-306) and the improved estimators in a second pass over the new string
//     with the loop_l / loop_u fragments of each operator (sse.C:314-354; graph_impl.h:489-494);
//     the operator index is the time.  The normal estimator's time-integrated magnetization is
//     accumulated in the first pass at the off-diagonal operators (sse.C:255-259).
//   * a coin per cluster, then operator types and spins flipped (sse.C:359-371)
// Random numbers: the words of Philox(seed; sweep, 0, TAG_SSE, k), k = 0, 1, ..., four per counter,
// consumed in the walk's order: per insertion trial one uniform ((w + 1/2) 2^-32) and, when
// accepted, one word for the bond (floor(w NB / 2^32): the weights of all bonds are equal) and one
// for the graph; per removal trial one uniform and, when kept, one word for the graph choice.  The
// coin of a cluster is keyed by its smallest fragment index (sites first, then one fragment per
// graph-0 operator in string order).
// ----------------------------------------------------------------------------------------------
enum { TAG_SSE = 8 };

struct sse_chain_t {
  lattice lat;
  bond_weight bw;
  double beta = 1, bwt = 0;  // bwt = beta * W * NB (sse.C:203, graph_weight of all bonds)
  uint64_t seed = 0;
  uint64_t T0 = 0, T1 = 0, T2 = 0, Poff = 0, Pd0 = 0, Pd1 = 0;
  std::vector<int> spins;
  std::vector<uint32_t> ops;
  uint32_t sweep = 0;
  std::vector<uint64_t> records;
  int status = 0;  // 1: a boundary had spin sectors of different sizes

  void init_derived() {
    const double W = bw.W;
    if (W > 0) {
      T0 = prob_u32(bw.v[0] / W);
      T1 = prob_u32((bw.v[0] + bw.v[1]) / W);
      T2 = prob_u32((bw.v[0] + bw.v[1] + bw.v[2]) / W);
    }
    const double s01 = bw.v[0] + bw.v[1], s02 = bw.v[0] + bw.v[2], s13 = bw.v[1] + bw.v[3];
    Poff = prob_u32(s01 > 0 ? bw.v[0] / s01 : 1.0);
    Pd0 = prob_u32(s02 > 0 ? bw.v[0] / s02 : 1.0);   // antiparallel: graph 0 or 2
    Pd1 = prob_u32(s13 > 0 ? bw.v[1] / s13 : 1.0);   // parallel: graph 1 or 3
    bwt = beta * W * lat.NB;
  }

  struct stream {
    uint64_t seed;
    uint32_t sweep, ctr = 0;
    int k = 4;
    uint32_t w[4] = {0, 0, 0, 0};
    uint32_t word() {
      if (k == 4) { rng4(seed, sweep, 0u, TAG_SSE, ctr++, w); k = 0; }
      return w[k++];
    }
    double uniform() { return ((double)word() + 0.5) * 2.3283064365386963e-10; }
  };

  struct sop { uint32_t b; int off, g, loop0, loop1; };

  void sweep_once() {
    const int N = lat.N, NB = lat.NB;
    stream r{seed, sweep};
    std::vector<int> sc(spins), current(N);
    uf frag;
    frag.deterministic = true;
    frag.reset(N);
    for (int s = 0; s < N; ++s) current[s] = s;
    std::vector<sop> nops;
    // normal estimator (susceptibility.h:270-300): (1-2c) t at every piece end minus at its begin
    int64_t MA = 0, SMA = 0;
    int nop = (int)ops.size();
    size_t i = 0;
    bool try_gap = true;
    while (try_gap || i < ops.size()) {
      sop o{};
      if (try_gap) {
        if (!((double)(nop + 1) * r.uniform() < bwt)) { try_gap = false; continue; }
        o.b = (uint32_t)(((uint64_t)r.word() * (uint64_t)NB) >> 32);
        const uint32_t wg = r.word();
        o.g = (int)(wg >= T0) + (int)(wg >= T1) + (int)(wg >= T2);
        const int c0 = sc[lat.s0[o.b]], c1 = sc[lat.s1[o.b]];
        if (!((o.g & 1) ^ c0 ^ c1)) { try_gap = false; continue; }   // is_compatible
        o.off = 0;
        ++nop;
      } else {
        o.b = ops[i] >> 1;
        o.off = (int)(ops[i] & 1u);
        const int c0 = sc[lat.s0[o.b]], c1 = sc[lat.s1[o.b]];
        if (!o.off) {
          if (bwt * r.uniform() < (double)nop) { --nop; ++i; continue; }
          const int c = 1 ^ c0 ^ c1;
          o.g = (((uint64_t)r.word() < (c ? Pd1 : Pd0)) ? 0 : 2) ^ c;
        } else {
          o.g = ((uint64_t)r.word() < Poff) ? 0 : 1;
        }
        ++i;
        try_gap = true;
      }
      const int t = (int)nops.size();
      const int s0 = lat.s0[o.b], s1 = lat.s1[o.b];
      if (o.off) {
        for (int s : {s0, s1}) {
          const int sg = 1 - 2 * sc[s];
          MA += 2 * (int64_t)sg * t;                 // end at t with c, begin at t with 1 - c
          SMA += 2 * (int64_t)lat.gauge[s] * sg * t;
          sc[s] ^= 1;
        }
      }
      if (o.g & 2) {
        o.loop0 = o.loop1 = current[s0] = current[s1] = frag.unify(current[s0], current[s1]);
      } else if (o.g == 0) {
        const int f = frag.add();
        o.loop0 = frag.unify(current[s0], current[s1]);
        o.loop1 = current[s0] = current[s1] = f;
      } else {
        o.loop0 = current[s0];
        o.loop1 = current[s1];
        std::swap(current[s0], current[s1]);
      }
      nops.push_back(o);
    }
    const int64_t T = (int64_t)nops.size();
    for (int s = 0; s < N; ++s) {                    // stop_top of the normal estimator
      MA += (int64_t)(1 - 2 * sc[s]) * T;
      SMA += (int64_t)lat.gauge[s] * (1 - 2 * sc[s]) * T;
    }
    if (lat.spin2 <= 1) {
      for (int s = 0; s < N; ++s) frag.unify(s, current[s]);
    } else {
      for (int rs = 0; rs < lat.NR; ++rs) {
        const int off = rs * lat.spin2;
        int pair[8];
        if (!boundary_matching(seed, sweep, (uint32_t)rs, lat.spin2, &spins[off], &sc[off], pair)) {
          status = 1;
          return;
        }
        for (int a = 0; a < lat.spin2; ++a) frag.unify(off + a, current[off + pair[a]]);
      }
    }
    const int nf = (int)frag.parent.size();
    const int nc = frag.set_ids();

    // ---- improved estimators, second pass (sse.C:314-354) ----
    std::vector<int64_t> n0(nc, 0), m0(nc, 0), sn0(nc, 0), sm0(nc, 0);
    std::vector<int64_t> Lc(nc, 0), Mc(nc, 0), SLc(nc, 0), SMc(nc, 0), wind((size_t)nc * 3, 0);
    std::vector<int> key(nc, nf);
    for (int f = 0; f < nf; ++f) key[frag.id[f]] = std::min(key[frag.id[f]], f);
    auto piece = [&](int fr, int sgn, int64_t t, int s, int c) {
      const int cl = frag.id[fr], sg = 1 - 2 * c, g = lat.gauge[s];
      Lc[cl] += sgn * t; Mc[cl] += sgn * sg * t; SLc[cl] += sgn * g * t; SMc[cl] += sgn * g * sg * t;
    };
    std::vector<int> c2(spins);
    int64_t M0tot = 0, SM0tot = 0;
    for (int s = 0; s < N; ++s) {                    // start_bottom
      const int cl = frag.id[s], sg = 1 - 2 * c2[s], g = lat.gauge[s];
      n0[cl] += 1; m0[cl] += sg; sn0[cl] += g; sm0[cl] += g * sg;
      M0tot += sg; SM0tot += g * sg;
    }
    for (int64_t t = 0; t < T; ++t) {
      const sop& o = nops[t];
      if (o.g & 2) continue;                          // frozen graphs contribute nothing
      const int s0 = lat.s0[o.b], s1 = lat.s1[o.b], d = lat.bdir[o.b];
      const int l0 = o.loop0, l1 = (o.g == 0) ? o.loop0 : o.loop1;   // loop_l0, loop_l1
      const int u0 = o.loop1, u1 = (o.g == 0) ? o.loop1 : o.loop0;   // loop_u0, loop_u1
      piece(l0, +1, t, s0, c2[s0]);
      piece(l1, +1, t, s1, c2[s1]);
      wind[(size_t)frag.id[l0] * 3 + d] += 1 - 2 * c2[s0];             // end_bs
      if (o.off) { c2[s0] ^= 1; c2[s1] ^= 1; }
      piece(u0, -1, t, s0, c2[s0]);
      piece(u1, -1, t, s1, c2[s1]);
      wind[(size_t)frag.id[u0] * 3 + d] -= 1 - 2 * c2[s0];             // begin_bs
    }
    for (int s = 0; s < N; ++s) piece(current[s], +1, T, s, c2[s]);    // stop_top

    // ---- coins, record, flips ----
    std::vector<uint8_t> flip(nc);
    for (int cl = 0; cl < nc; ++cl) {
      uint32_t w[4];
      rng4(seed, sweep, (uint32_t)key[cl], TAG_FLIP, 0, w);
      flip[cl] = (w[0] < 0x80000000u) ? 1 : 0;
    }
    std::vector<uint64_t> rec(R_WORDS, 0);
    rec[R_NOP] = (uint64_t)T;
    rec[R_NC] = (uint64_t)nc;
    rec[R_M0] = (uint64_t)M0tot;
    rec[R_SM0] = (uint64_t)SM0tot;
    for (int cl = 0; cl < nc; ++cl) {
      rec[R_M0SQ] += (uint64_t)(m0[cl] * m0[cl]);
      rec[R_N0SQ] += (uint64_t)(n0[cl] * n0[cl]);
      rec[R_SM0SQ] += (uint64_t)(sm0[cl] * sm0[cl]);
      rec[R_SN0SQ] += (uint64_t)(sn0[cl] * sn0[cl]);
      auto q4 = [](int64_t x) { u128 a = (u128)(uint64_t)(x * x); return a * a; };
      add128(rec.data(), R_M0Q_LO, q4(m0[cl]));
      add128(rec.data(), R_N0Q_LO, q4(n0[cl]));
      add128(rec.data(), R_SM0Q_LO, q4(sm0[cl]));
      add128(rec.data(), R_SN0Q_LO, q4(sn0[cl]));
      auto sq = [](int64_t x) { uint64_t a = (uint64_t)(x < 0 ? -x : x); return (u128)a * a; };
      add128(rec.data(), R_LSQ_LO, sq(Lc[cl]));
      add128(rec.data(), R_MSQ_LO, sq(Mc[cl]));
      add128(rec.data(), R_SLSQ_LO, sq(SLc[cl]));
      add128(rec.data(), R_SMSQ_LO, sq(SMc[cl]));
      for (int d = 0; d < 3; ++d) {
        const int64_t w = wind[(size_t)cl * 3 + d];
        rec[R_WSQ] += (uint64_t)(w * w);
        rec[R_W0 + d] += (uint64_t)w;
      }
    }
    rec[R_FLD] = 0;                                   // no field on the SSE form
    rec[R_MA] = (uint64_t)MA;
    rec[R_SMA] = (uint64_t)SMA;
    records.insert(records.end(), rec.begin(), rec.end());
    ops.assign(nops.size(), 0u);
    for (size_t k = 0; k < nops.size(); ++k) {
      const int off = nops[k].off ^ (flip[frag.id[nops[k].loop0]] ^ flip[frag.id[nops[k].loop1]]);
      ops[k] = (nops[k].b << 1) | (uint32_t)off;
    }
    for (int s = 0; s < N; ++s) if (flip[frag.id[s]]) spins[s] ^= 1;
    ++sweep;
  }
};

// ----------------------------------------------------------------------------------------------
// Standalone mode: restates standalone/loop.C:39-195 (Heisenberg AF chain, mt19937(29833)),
// with the weighted union-find of standalone/union_find.h:113-126 (full compression).
// ----------------------------------------------------------------------------------------------
struct sa_node { int parent = -1; int id = 0; };

static int sa_root(std::vector<sa_node>& v, int g) { while (v[g].parent >= 0) g = v[g].parent; return g; }
static void sa_update(std::vector<sa_node>& v, int g, int r) {
  while (g != r) { int p = v[g].parent; v[g].parent = r; g = p; }
}
static int sa_unify(std::vector<sa_node>& v, int g0, int g1) {
  int r0 = sa_root(v, g0), r1 = sa_root(v, g1);
  if (r0 != r1) {
    if (-v[r0].parent < -v[r1].parent) std::swap(r0, r1);
    v[r0].parent += v[r1].parent;
    v[r1].parent = r0;
  }
  sa_update(v, g0, r0);
  sa_update(v, g1, r0);
  return r0;
}

struct sa_obs {
  double sum = 0, esq = 0; unsigned count = 0;
  void add(double x) { sum += x; esq += x * x; ++count; }
  double mean() const { return count > 0 ? sum / count : 0.; }
  double error() const {
    return count > 1 ? std::sqrt((esq / count - mean() * mean()) / (count - 1)) : 0.;
  }
};

static void standalone_run(unsigned L, double T, unsigned sweeps, unsigned therm, double* out,
                           double* speed) {
  const unsigned nsites = L, nbonds = L;
  const double beta = 1 / T;
  std::mt19937 eng(29833);
  std::uniform_real_distribution<> d_uniform;
  std::exponential_distribution<> d_time(beta * nbonds / 2);
  struct sop { int diag; unsigned bond; unsigned up, lo; double time; };
  std::vector<sop> ops, ops_p;
  std::vector<int> spins(nsites, 0), current(nsites);
  std::vector<sa_node> frag;
  std::vector<int> to_flip;
  struct est { double mag = 0, size = 0, length = 0; };
  std::vector<est> ests;
  sa_obs o_nc, o_e, o_us, o_sm, o_ss;
  auto left = [&](unsigned b) { return (int)b; };
  auto right = [&](unsigned b) { return (b == nbonds - 1) ? 0 : (int)b + 1; };
  auto t0 = std::chrono::steady_clock::now();
  for (unsigned mcs = 0; mcs < therm + sweeps; ++mcs) {
    std::swap(ops, ops_p); ops.resize(0);
    frag.resize(0); frag.resize(nsites);
    for (unsigned s = 0; s < nsites; ++s) current[s] = (int)s;
    double t = d_time(eng);
    for (size_t oi = 0; t < 1 || oi != ops_p.size();) {
      if (oi == ops_p.size() || t < ops_p[oi].time) {
        const unsigned b = static_cast<unsigned>(nbonds * d_uniform(eng));
        if (spins[left(b)] != spins[right(b)]) {
          ops.push_back({1, b, 0, 0, t});
          t += d_time(eng);
        } else {
          t += d_time(eng);
          continue;
        }
      } else {
        if (ops_p[oi].diag) { ++oi; continue; }
        ops.push_back(ops_p[oi]);
        ++oi;
      }
      sop& o = ops.back();
      int s0 = left(o.bond), s1 = right(o.bond);
      if (!o.diag) { spins[s0] ^= 1; spins[s1] ^= 1; }
      o.lo = (unsigned)sa_unify(frag, current[s0], current[s1]);
      frag.push_back(sa_node());
      o.up = (unsigned)(frag.size() - 1);
      current[s0] = current[s1] = (int)o.up;
    }
    for (unsigned s = 0; s < nsites; ++s) sa_unify(frag, (int)s, current[s]);
    int nc = 0;
    for (auto& f : frag) if (f.parent < 0) f.id = nc++;
    for (size_t i = 0; i < frag.size(); ++i) frag[i].id = frag[sa_root(frag, (int)i)].id;
    to_flip.assign(nc, 0);
    ests.assign(nc, est());
    for (auto& o : ops) {
      ests[frag[o.lo].id].length += 2 * o.time;
      ests[frag[o.up].id].length -= 2 * o.time;
    }
    for (unsigned s = 0; s < nsites; ++s) {
      int id = frag[s].id;
      ests[id].mag += 1 - 2 * spins[s];
      ests[id].size += 1;
      ests[id].length += 1;
    }
    double usus = 0, smag = 0, ssus = 0;
    for (auto& e : ests) { usus += e.mag * e.mag; smag += e.size * e.size; ssus += e.length * e.length; }
    for (int c = 0; c < nc; ++c) to_flip[c] = (d_uniform(eng) < 0.5);
    for (auto& o : ops) if (to_flip[frag[o.lo].id] ^ to_flip[frag[o.up].id]) o.diag ^= 1;
    for (unsigned s = 0; s < nsites; ++s) if (to_flip[frag[s].id]) spins[s] ^= 1;
    if (mcs >= therm) {
      o_nc.add(nc);
      o_e.add((0.25 * nbonds - (double)ops.size() / beta) / nsites);
      o_us.add(0.25 * beta * usus / nsites);
      o_sm.add(0.25 * smag);
      o_ss.add(0.25 * beta * ssus / nsites);
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  double el = std::chrono::duration<double>(t1 - t0).count();
  if (speed) *speed = (therm + sweeps) / el;
  const sa_obs* o[5] = {&o_nc, &o_e, &o_us, &o_sm, &o_ss};
  for (int i = 0; i < 5; ++i) { out[2 * i] = o[i]->mean(); out[2 * i + 1] = o[i]->error(); }
}

}  // namespace orc

// ================================================================================================
// C surface (ctypes)
// ================================================================================================
extern "C" {

struct orc_params {
  int dim;            // 1 chain, 2 square, 3 cubic
  int L;
  double beta;
  double jxy, jz, h;
  double force_scatter;
  uint64_t seed;
  int random_spins;   // 1: iid spins from the seed; 0: all up
  int deterministic_uf;
  int spin2;          // 2S: virtual sites per real site
};

void* orc_create(const orc_params* p) {
  orc::chain_t* c = new orc::chain_t();
  c->lat.build(p->dim, p->L, p->spin2 > 1 ? p->spin2 : 1);
  c->bw = orc::make_weight(p->jxy, p->jz, p->force_scatter);
  c->beta = p->beta; c->h = p->h; c->seed = p->seed;
  c->field = (std::fabs(p->h) > 1e-12);
  c->deterministic_uf = p->deterministic_uf != 0;
  c->init_derived();
  c->spins.assign(c->lat.N, 0);
  if (p->random_spins) {
    for (int s = 0; s < c->lat.N; ++s) {
      uint32_t w[4];
      orc::rng4(c->seed, 0xFFFFFFFFu, (uint32_t)s, orc::TAG_SPIN, 0, w);
      c->spins[s] = (int)(w[0] & 1u);
    }
  }
  return c;
}

void orc_destroy(void* h) { delete static_cast<orc::chain_t*>(h); }

void orc_sweep(void* h, int n) {
  orc::chain_t* c = static_cast<orc::chain_t*>(h);
  for (int i = 0; i < n; ++i) c->sweep_once();
}

int orc_num_sites(void* h) { return static_cast<orc::chain_t*>(h)->lat.N; }
int orc_status(void* h) { return static_cast<orc::chain_t*>(h)->status; }
int orc_num_ops(void* h) { return (int)static_cast<orc::chain_t*>(h)->ops.size(); }
int orc_num_records(void* h) {
  return (int)(static_cast<orc::chain_t*>(h)->records.size() / orc::R_WORDS);
}
int orc_record_words() { return orc::R_WORDS; }
void orc_get_records(void* h, uint64_t* out) {
  auto& r = static_cast<orc::chain_t*>(h)->records;
  std::memcpy(out, r.data(), r.size() * sizeof(uint64_t));
}
void orc_clear_records(void* h) { static_cast<orc::chain_t*>(h)->records.clear(); }

// Persistent state: spins at tau=0 and the off-diagonal operators (bond, time), time ordered.
int orc_get_state(void* h, int* spins, int* bonds, double* times, int cap) {
  orc::chain_t* c = static_cast<orc::chain_t*>(h);
  for (int s = 0; s < c->lat.N; ++s) spins[s] = c->spins[s];
  std::vector<std::pair<uint64_t, int>> v;
  for (auto& o : c->ops)
    if (o.offdiag) v.push_back({orc::d_bits(o.t), o.bond});
  std::sort(v.begin(), v.end());  // (time, bond)
  int n = (int)v.size();
  for (int i = 0; i < n && i < cap; ++i) { bonds[i] = v[i].second; times[i] = orc::bits_d(v[i].first); }
  return n;
}

int orc_set_state(void* h, const int* spins, const int* bonds, const double* times, int n,
                  uint32_t sweep) {
  orc::chain_t* c = static_cast<orc::chain_t*>(h);
  for (int s = 0; s < c->lat.N; ++s) c->spins[s] = spins[s] & 1;
  c->ops.clear();
  for (int i = 0; i < n; ++i) c->ops.push_back({bonds[i], times[i], 1, 0});
  std::stable_sort(c->ops.begin(), c->ops.end(), [](const orc::op_t& a, const orc::op_t& b) {
    return orc::d_bits(a.t) < orc::d_bits(b.t);
  });
  c->sweep = sweep;
  return 0;
}

// Cluster-construction configuration of the last sweep (before the flip).
int orc_last_config(void* h, int* spins, int* bonds, double* times, int* graphs, int* offdiag,
                    int cap) {
  orc::chain_t* c = static_cast<orc::chain_t*>(h);
  for (int s = 0; s < c->lat.N; ++s) spins[s] = c->last_spins[s];
  int n = (int)c->last_ops.size();
  for (int i = 0; i < n && i < cap; ++i) {
    bonds[i] = c->last_ops[i].bond; times[i] = c->last_ops[i].t;
    graphs[i] = c->last_ops[i].g; offdiag[i] = c->last_ops[i].offdiag;
  }
  return n;
}
int orc_last_labels(void* h, int* labels, int cap) {
  orc::chain_t* c = static_cast<orc::chain_t*>(h);
  for (int i = 0; i < c->last_nfrag && i < cap; ++i) labels[i] = c->last_labels[i];
  return c->last_nfrag;
}
int orc_last_nc(void* h) { return static_cast<orc::chain_t*>(h)->last_nc; }

// SSE chains (sse_chain_t): create from the same parameters (h must be 0), sweep, the
// per-sweep records, and the state (spins at the bottom and the operator codes in order).
void* orc_sse_create(const orc_params* p) {
  if (std::fabs(p->h) > 0) return nullptr;
  orc::sse_chain_t* c = new orc::sse_chain_t();
  c->lat.build(p->dim, p->L, p->spin2 > 1 ? p->spin2 : 1);
  c->bw = orc::make_weight(p->jxy, p->jz, p->force_scatter);
  c->beta = p->beta;
  c->seed = p->seed;
  c->init_derived();
  c->spins.assign(c->lat.N, 0);
  if (p->random_spins) {
    for (int s = 0; s < c->lat.N; ++s) {
      uint32_t w[4];
      orc::rng4(c->seed, 0xFFFFFFFFu, (uint32_t)s, orc::TAG_SPIN, 0, w);
      c->spins[s] = (int)(w[0] & 1u);
    }
  }
  return c;
}
void orc_sse_destroy(void* h) { delete static_cast<orc::sse_chain_t*>(h); }
int orc_sse_status(void* h) { return static_cast<orc::sse_chain_t*>(h)->status; }
void orc_sse_sweep(void* h, int n) {
  orc::sse_chain_t* c = static_cast<orc::sse_chain_t*>(h);
  for (int i = 0; i < n; ++i) c->sweep_once();
}
int orc_sse_num_records(void* h) {
  return (int)(static_cast<orc::sse_chain_t*>(h)->records.size() / orc::R_WORDS);
}
void orc_sse_get_records(void* h, uint64_t* out) {
  auto& r = static_cast<orc::sse_chain_t*>(h)->records;
  std::memcpy(out, r.data(), r.size() * sizeof(uint64_t));
}
void orc_sse_clear_records(void* h) { static_cast<orc::sse_chain_t*>(h)->records.clear(); }
int orc_sse_get_state(void* h, int* spins, uint32_t* ops, int cap) {
  orc::sse_chain_t* c = static_cast<orc::sse_chain_t*>(h);
  for (int s = 0; s < c->lat.N; ++s) spins[s] = c->spins[s];
  const int n = (int)c->ops.size();
  for (int i = 0; i < n && i < cap; ++i) ops[i] = c->ops[i];
  return n;
}
void orc_sse_set_state(void* h, const int* spins, const uint32_t* ops, int n, uint32_t sweep) {
  orc::sse_chain_t* c = static_cast<orc::sse_chain_t*>(h);
  for (int s = 0; s < c->lat.N; ++s) c->spins[s] = spins[s] & 1;
  c->ops.assign(ops, ops + n);
  c->sweep = sweep;
}

// Cluster labels of a given configuration (time-ordered vertex list), following the fragment
// numbering of path_integral.C:482 / graph_impl.h:285-288: sites first, then one fragment per
// g == 0 vertex in time order.  Returns the number of fragments; *nc receives the cluster count.
int orc_uf_label(int dim, int L, int nops, const int* bonds, const int* graphs, int deterministic,
                 int* labels, int cap, int* nc) {
  orc::lattice lat; lat.build(dim, L);
  orc::uf frag; frag.deterministic = deterministic != 0; frag.reset(lat.N);
  std::vector<int> current(lat.N);
  for (int s = 0; s < lat.N; ++s) current[s] = s;
  for (int i = 0; i < nops; ++i) {
    int s0 = lat.s0[bonds[i]], s1 = lat.s1[bonds[i]], g = graphs[i];
    int c0 = current[s0], c1 = current[s1];
    if (g & 2) {
      current[s0] = current[s1] = frag.unify(c0, c1);
    } else if (g == 0) {
      int f = frag.add();
      frag.unify(c0, c1);
      current[s0] = current[s1] = f;
    } else {
      current[s0] = c1; current[s1] = c0;
    }
  }
  for (int s = 0; s < lat.N; ++s) frag.unify(s, current[s]);
  *nc = frag.set_ids();
  int n = (int)frag.parent.size();
  for (int i = 0; i < n && i < cap; ++i) labels[i] = frag.id[i];
  return n;
}

// Replay of a node-pair union sequence (test/union_find.C:45-52): returns parents (-1 for
// roots), roots and root weights after all unions.
void orc_uf_replay(int n, int npairs, const int* pairs, int* parent, int* root, int* weight) {
  orc::uf u; u.reset(n);
  for (int i = 0; i < npairs; ++i) u.unify(pairs[2 * i], pairs[2 * i + 1]);
  for (int i = 0; i < n; ++i) {
    parent[i] = u.is_root(i) ? -1 : u.par(i);
    root[i] = u.root(i);
    weight[i] = u.is_root(i) ? u.weight(i) : 0;
  }
}

// Standalone restatement; out[10] = (mean, error) of Number of Clusters, Energy Density,
// Uniform Susceptibility, Staggered Magnetization^2, Staggered Susceptibility.
void orc_standalone(unsigned L, double T, unsigned sweeps, unsigned therm, double* out,
                    double* speed) {
  orc::standalone_run(L, T, sweeps, therm, out, speed);
}

// Numerics probes (for known-answer tests of the random source).
void orc_philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t* out) {
  orc::rng4(seed, c0, c1, c2, c3, out);
}
void orc_philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  orc::philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = c[i];
}
float orc_log_spec(float u) { return orc::log_spec(u); }
float orc_gap_uniform(uint32_t w, uint32_t tail) { return orc::gap_uniform(w, tail); }
float orc_exp_spec(float x) { return orc::exp_spec(x); }
double orc_weights(double jxy, double jz, double fs, double* v) {
  orc::bond_weight w = orc::make_weight(jxy, jz, fs);
  for (int i = 0; i < 4; ++i) v[i] = w.v[i];
  return w.W;
}

}  // extern "C"
