// The stochastic series expansion (SSE) loop worker of sse.C, batched: one chain per warp.
//
// The SSE representation keeps an ordered operator string without times.  Its diagonal update is
// one sequential walk (sse.C:201-250): at every gap an insertion is tried with probability
// beta W / (n + 1) (n the running operator count) and, when accepted and compatible with the
// spins there, tried again; every existing diagonal operator is removed with probability
// n / (beta W) or re-draws its graph; off-diagonal operators re-draw theirs.  The acceptance
// probabilities depend on the running count, so the walk cannot be split across threads; what
// the GPU offers is thousands of such walks side by side, one per chain, which is the form here:
// one thread (the first lane of a warp) owns a chain for a whole chunk of sweeps (k_sse), and
// the chains of an arena are spread over the grid.
//
// Per sweep and chain the thread does what sse.C does, in the same order:
//   walk           insertions / removals / graph choices (sse.C:201-250), the spin propagation and
//                  the reconnection of graph_impl.h:280-295 (a new fragment per graph-0 vertex),
//                  and the improved estimator's contributions of every world-line piece
//                  (susceptibility.h:116-150, stiffness.h:82-130), added to the fragment the piece
//                  belongs to (the operator index is the SSE "time")
//   closure        every site's top fragment joined to its bottom one (sse.C:275-277); for S > 1/2
//                  the bottom of virtual site a joins the top of pair[a], a matching within each
//                  spin sector of the real site (sse.C:278-296), the path-integral form's
//                  boundary_pairs draw
//   clusters       fragments summed into their roots (the smallest fragment index: deterministic
//                  unify), a coin per cluster keyed by its root, the exact per-sweep sums
//                  (susceptibility.h:182-198) into the record row
//   flips          operator types and spins (sse.C:363-371)
// The random numbers are Philox words of (chain seed, sweep, TAG_SSE, counter), consumed in the
// walk's order; the record row is the path-integral one, with world-line lengths counted in
// operator-index units instead of 2^-40 of beta (the host applies the SSE estimator formulas).
#pragma once
#include "lg_kernels.cuh"

namespace lg {

// Parameters of one k_sse launch (m sweeps of every chain).  Chain c's operator strings start at
// c * ocap (operator code: bond << 1 | off-diagonal), its fragment arrays at c * fcap.
struct SseArgs {
  int m;
  int ocap, fcap;
  const uint8_t* spin_in;     // spins at the start (arena site indexed)
  uint8_t* spin_out;          // and at the end
  const uint32_t* ops_in;     // operator string at the start
  uint32_t* ops_out;          // at the end
  uint32_t* ops_tmp;          // a third string for the sweeps in between
  const int* nop_in;
  int* nop_out;
  int* loops;                 // 2 per operator: fragments below / above (graph_impl.h reconnect)
  int* frag;                  // union-find parent per fragment
  long long* est;             // 8 per fragment: n0, m0, sn0, sm0, L, M, SL, SM
  int* wnd;                   // 3 per fragment: winding per direction
  int* cur;                   // current fragment of every site (arena site indexed)
  uint8_t* spc;               // spins along the walk (arena site indexed)
  uint8_t* flipf;             // flip of every root fragment
};

// Philox words of one chain's sweep, in order.
struct SseRng {
  uint64_t seed;
  uint32_t sweep, ctr;
  int k;
  rnd4 buf;
  __device__ __forceinline__ uint32_t word() {
    if (k == 4) { buf = philox(seed, sweep, 0u, TAG_SSE, ctr++); k = 0; }
    const uint32_t w = k == 0 ? buf.x : k == 1 ? buf.y : k == 2 ? buf.z : buf.w;
    ++k;
    return w;
  }
  // uniform in (0, 1), 32-bit resolution
  __device__ __forceinline__ double uniform() { return ((double)word() + 0.5) * 2.3283064365386963e-10; }
};

__device__ __forceinline__ int sse_find(int* P, int x) {
  int r = x;
  while (P[r] != r) r = P[r];
  while (P[x] != r) { const int n = P[x]; P[x] = r; x = n; }  // full compression
  return r;
}

// union of two fragments: the larger root hooks under the smaller (deterministic unify)
__device__ __forceinline__ int sse_unify(int* P, int a, int b) {
  a = sse_find(P, a);
  b = sse_find(P, b);
  if (a == b) return a;
  if (a < b) { P[b] = a; return a; }
  P[a] = b;
  return b;
}

// A world-line piece of site s with spin c ends (sgn = +1) or begins (sgn = -1) at index t in
// fragment f (susceptibility.h:116-150: end_s adds t, begin_s subtracts it).
__device__ __forceinline__ void sse_piece(long long* e, int sgn, long long t, int c, int gs) {
  const long long mt = (long long)(1 - 2 * c) * t;
  e[4] += sgn * t;
  e[5] += sgn * mt;
  e[6] += sgn * gs * t;
  e[7] += sgn * gs * mt;
}

__device__ void sse_chain(const Arena& A, const SseArgs& S, int c) {
  const DChain ch = A.ch[c];
  const int N = ch.nsites, NB = ch.nbonds, so = ch.site_off, bo = ch.bond_off, dim = ch.dim;
  const size_t obase = (size_t)c * S.ocap, fbase = (size_t)c * S.fcap;
  int* frag = S.frag + fbase;
  long long* est = S.est + 8 * fbase;
  int* wnd = S.wnd + 3 * fbase;
  int* loops = S.loops + 2 * obase;
  uint8_t* flipf = S.flipf + fbase;
  int* cur = S.cur + so;
  uint8_t* spc = S.spc + so;
  uint8_t* spins = S.spin_out + so;
  for (int s = 0; s < N; ++s) spins[s] = S.spin_in[so + s];
  int nop = S.nop_in[c];
  uint32_t sweep = A.ch_sweep[c];
  const double bw = ch.sse_bw;
  const uint32_t q2 = (uint32_t)(ch.spin2 > 1 ? ch.spin2 * ch.spin2 : 1);
  for (int step = 0; step < S.m; ++step, ++sweep) {
    // strings: the launch's input, then alternating so that the last sweep writes ops_out
    const uint32_t* in = step == 0 ? S.ops_in + obase
                                   : (((S.m - step) & 1) ? S.ops_tmp + obase : S.ops_out + obase);
    uint32_t* out = ((S.m - 1 - step) & 1) ? S.ops_tmp + obase : S.ops_out + obase;
    SseRng rng{ch.seed, sweep, 0u, 4, {0, 0, 0, 0}};
    for (int s = 0; s < N; ++s) {
      const int cs = spins[s], gs = A.gauge[so + s];
      spc[s] = (uint8_t)cs;
      cur[s] = s;
      frag[s] = s;
      long long* e = est + 8 * s;
      e[0] = 1; e[1] = 1 - 2 * cs; e[2] = gs; e[3] = gs * (1 - 2 * cs);  // start_bottom
      e[4] = e[5] = e[6] = e[7] = 0;
      wnd[3 * s] = wnd[3 * s + 1] = wnd[3 * s + 2] = 0;
    }
    const int nop_old = nop;
    int fid = N, nn = 0, i = 0;
    bool try_gap = true;
    while (try_gap || i < nop_old) {
      uint32_t b, off, g;
      if (try_gap) {
        if ((double)(nop + 1) * rng.uniform() < bw) {
          b = (uint32_t)(((uint64_t)rng.word() * (uint64_t)NB) >> 32);
          const uint64_t wg = rng.word();
          g = (uint32_t)(wg >= ch.T0) + (uint32_t)(wg >= ch.T1) + (uint32_t)(wg >= ch.T2);
          const int s0 = A.bond_s0[bo + b] - so, s1 = A.bond_s1[bo + b] - so;
          if (!(((g & 1u) ^ spc[s0] ^ spc[s1]) & 1u)) { try_gap = false; continue; }
          off = 0;
          ++nop;
        } else {
          try_gap = false;
          continue;
        }
      } else {
        const uint32_t op = in[i];
        b = op >> 1;
        off = op & 1u;
        const int s0 = A.bond_s0[bo + b] - so, s1 = A.bond_s1[bo + b] - so;
        if (!off) {
          if (bw * rng.uniform() < (double)nop) { --nop; ++i; continue; }
          const uint32_t cc = 1u ^ spc[s0] ^ spc[s1];  // 0 antiparallel, 1 parallel
          g = (((uint64_t)rng.word() < (cc ? ch.Pd1 : ch.Pd0)) ? 0u : 2u) ^ cc;
        } else {
          g = ((uint64_t)rng.word() < ch.Poff) ? 0u : 1u;
        }
        ++i;
        try_gap = true;
      }
      if (nn >= S.ocap || fid >= S.fcap) { atomicExch(&A.ctl->err, ERR_OVERFLOW); return; }
      const int s0 = A.bond_s0[bo + b] - so, s1 = A.bond_s1[bo + b] - so;
      const int gs0 = A.gauge[so + s0], gs1 = A.gauge[so + s1];
      const int d = (int)((b / q2) % (uint32_t)dim);   // bond = (site dim + d) (2S)^2 + pair
      const bool frozen = (g & 2u) != 0;
      const int a0 = cur[s0], a1 = cur[s1];
      const int c0 = spc[s0], c1 = spc[s1];
      if (!frozen) {
        sse_piece(est + 8 * a0, 1, nn, c0, gs0);
        sse_piece(est + 8 * a1, 1, nn, c1, gs1);
        wnd[3 * a0 + d] += 1 - 2 * c0;                         // end_bs at the source
      }
      if (off) { spc[s0] ^= 1u; spc[s1] ^= 1u; }
      int l0, l1;
      if (frozen) {
        l0 = l1 = sse_unify(frag, a0, a1);
        cur[s0] = cur[s1] = l0;
      } else if (g == 0) {
        l0 = sse_unify(frag, a0, a1);
        const int f = fid++;
        frag[f] = f;
        long long* e = est + 8 * f;
        for (int q = 0; q < 8; ++q) e[q] = 0;
        wnd[3 * f] = wnd[3 * f + 1] = wnd[3 * f + 2] = 0;
        l1 = f;
        cur[s0] = cur[s1] = f;
      } else {
        l0 = a0;
        l1 = a1;
        cur[s0] = a1;
        cur[s1] = a0;
      }
      loops[2 * nn] = l0;
      loops[2 * nn + 1] = l1;
      if (!frozen) {
        sse_piece(est + 8 * cur[s0], -1, nn, spc[s0], gs0);
        sse_piece(est + 8 * cur[s1], -1, nn, spc[s1], gs1);
        wnd[3 * cur[s0] + d] -= 1 - 2 * (int)spc[s0];          // begin_bs at the source
      }
      out[nn] = (b << 1) | off;
      ++nn;
    }
    nop = nn;
    for (int s = 0; s < N; ++s) sse_piece(est + 8 * cur[s], 1, nop, spc[s], A.gauge[so + s]);  // stop_top
    const int sp2 = ch.spin2;
    if (sp2 <= 1) {                // the closure in imaginary time
      for (int s = 0; s < N; ++s) sse_unify(frag, s, cur[s]);
    } else {
      for (int off = 0, rs = 0; off < N; off += sp2, ++rs) {
        int pair[8];
        if (!boundary_pairs(ch.seed, sweep, (uint32_t)rs, sp2, spins + off, spc + off, pair)) {
          atomicExch(&A.ctl->err, ERR_BOUNDARY);
          return;
        }
        for (int a = 0; a < sp2; ++a) sse_unify(frag, off + a, cur[off + pair[a]]);
      }
    }
    // clusters: fragment sums into their roots
    for (int f = 0; f < fid; ++f) {
      const int r = sse_find(frag, f);
      if (r == f) continue;
      for (int q = 0; q < 8; ++q) est[8 * r + q] += est[8 * f + q];
      for (int q = 0; q < 3; ++q) wnd[3 * r + q] += wnd[3 * f + q];
    }
    unsigned long long nc = 0, m0 = 0, sm0 = 0, m0sq = 0, n0sq = 0, sm0sq = 0, sn0sq = 0;
    unsigned long long ma = 0, sma = 0, wsq = 0, w0 = 0, w1 = 0, w2 = 0;
    u128 m0q = {0, 0}, n0q = {0, 0}, sm0q = {0, 0}, sn0q = {0, 0};
    u128 lsq = {0, 0}, msq = {0, 0}, slsq = {0, 0}, smsq = {0, 0};
    auto ab = [](long long v) { return (unsigned long long)(v < 0 ? -v : v); };
    for (int f = 0; f < fid; ++f) {
      if (frag[f] != f) continue;
      const long long* e = est + 8 * f;
      ++nc;
      flipf[f] = philox(ch.seed, sweep, (uint32_t)f, TAG_FLIP, 0).x < 0x80000000u ? 1 : 0;
      const unsigned long long n0s = ab(e[0]) * ab(e[0]), m0s = ab(e[1]) * ab(e[1]);
      const unsigned long long sn0s = ab(e[2]) * ab(e[2]), sm0s = ab(e[3]) * ab(e[3]);
      m0 += (unsigned long long)e[1];
      sm0 += (unsigned long long)e[3];
      m0sq += m0s; n0sq += n0s; sm0sq += sm0s; sn0sq += sn0s;
      add_u128(m0q, mul64(m0s, m0s));
      add_u128(n0q, mul64(n0s, n0s));
      add_u128(sm0q, mul64(sm0s, sm0s));
      add_u128(sn0q, mul64(sn0s, sn0s));
      add_u128(lsq, mul64(ab(e[4]), ab(e[4])));
      add_u128(msq, mul64(ab(e[5]), ab(e[5])));
      add_u128(slsq, mul64(ab(e[6]), ab(e[6])));
      add_u128(smsq, mul64(ab(e[7]), ab(e[7])));
      ma += (unsigned long long)e[5];
      sma += (unsigned long long)e[7];
      const int* w = wnd + 3 * f;
      wsq += (unsigned long long)((long long)w[0] * w[0] + (long long)w[1] * w[1] + (long long)w[2] * w[2]);
      w0 += (unsigned long long)(long long)w[0];
      w1 += (unsigned long long)(long long)w[1];
      w2 += (unsigned long long)(long long)w[2];
    }
    // flips (sse.C:363-371): an operator changes type when its two clusters flip differently
    for (int p = 0; p < nop; ++p) {
      const uint8_t fl = flipf[sse_find(frag, loops[2 * p])] ^ flipf[sse_find(frag, loops[2 * p + 1])];
      out[p] ^= fl;
    }
    for (int s = 0; s < N; ++s) spins[s] ^= flipf[sse_find(frag, s)];
    unsigned long long* row = A.rec + ((size_t)step * A.C + c) * REC_WORDS;
    for (int w = 0; w < REC_WORDS; ++w) row[w] = 0ull;
    row[R_NOP] = (unsigned long long)nop;
    row[R_NC] = nc;
    row[R_M0] = m0; row[R_SM0] = sm0;
    row[R_M0SQ] = m0sq; row[R_N0SQ] = n0sq; row[R_SM0SQ] = sm0sq; row[R_SN0SQ] = sn0sq;
    row[R_M0Q] = m0q.lo; row[R_M0Q + 1] = m0q.hi;
    row[R_N0Q] = n0q.lo; row[R_N0Q + 1] = n0q.hi;
    row[R_SM0Q] = sm0q.lo; row[R_SM0Q + 1] = sm0q.hi;
    row[R_SN0Q] = sn0q.lo; row[R_SN0Q + 1] = sn0q.hi;
    row[R_LSQ] = lsq.lo; row[R_LSQ + 1] = lsq.hi;
    row[R_MSQ] = msq.lo; row[R_MSQ + 1] = msq.hi;
    row[R_SLSQ] = slsq.lo; row[R_SLSQ + 1] = slsq.hi;
    row[R_SMSQ] = smsq.lo; row[R_SMSQ + 1] = smsq.hi;
    row[R_MA] = ma; row[R_SMA] = sma;
    row[R_WSQ] = wsq; row[R_W0] = w0; row[R_W1] = w1; row[R_W2] = w2;
  }
  S.nop_out[c] = nop;
  A.ch_sweep[c] = sweep;
}

// One chain per warp, walked by its first lane: the walks are sequential and branchy, so lanes
// of one warp walking different chains would serialise on every divergent branch, and a chain
// per warp spreads an arena over every SM (1024 chains: 7 walks per SM instead of 64 lanes on
// each of 16 SMs).
constexpr int SSE_WARPS = 4;
constexpr int SSE_THREADS = 32 * SSE_WARPS;

__global__ void __launch_bounds__(SSE_THREADS) k_sse(Arena A, SseArgs S) {
  if (A.ctl->err) return;
  if ((threadIdx.x & 31) != 0) return;
  const int warps = gridDim.x * SSE_WARPS;
  for (int c = blockIdx.x * SSE_WARPS + (threadIdx.x >> 5); c < A.C; c += warps) {
    if (!A.all_active && !A.ch_active[c]) continue;
    sse_chain(A, S, c);
  }
}

}  // namespace lg
