// Sweep kernels of the GB300 loop-cluster engine.
//
// One sweep of every chain in the arena (path_integral.C:355-864) is this kernel sequence, one
// CUDA graph per arena.  Chains with few operators per site take the thread-per-element forms
// (*_narrow) on a second stream beside the warp-per-site forms.
//
//   k_insert(_narrow)  per bond: new operator string (time, graph, type), written at a vertex
//                      range claimed with one atomic add; capacity check        (:403-577)
//   k_site_blocks,     per site: number of segments = 1 + incident vertices, and the site
//   k_site_offsets     segment offsets (k_site_count + a three-kernel scan above 2^20 sites)
//   k_merge(_narrow)   per site: time-ordered segment list, union-find init, temporal closure
//                      (:584-589); instanced by the arena's largest site degree
//   k_boundary         spin S > 1/2 only, per real site: the tau = 0 boundary matching of its
//                      virtual sites                                             (:590-613)
//   k_union            per vertex: lock-free unions of its four legs          (graph_impl.h:280-295)
//   k_accumulate       per segment: parent := root, length into the root's class sums (:650-737)
//   k_cluster          per root: flip coin, improved / field sums -> records   (:739-803)
//   k_site_end(_narrow) per site: spin flip; new vertex types from the flips of the clusters
//                      below and above each endpoint; compacted off-diagonal list (:805-823)
//   k_end              per chain, on a third stream beside k_site_end: operator count, sweep
//                      counter; clears the next sweep's record row and claim counters
//   k_corr             with MEASURE[Correlations] / [Structure Factor] only: exact spin
//                      correlation sums per displacement (correlation.h)
//
// Memory layout (HBM, struct of arrays, 32-bit indices):
//   sites    spin0[N] u8, off_base[N], off_cnt[N]     persistent between sweeps
//   bonds    s0/s1[NB], chain[NB], dir0[NB] u8         static
//   vertices (one contiguous time-ordered range per bond: bond_ptr[b], bond_cnt[b], claimed
//            from the vertex region of the bond's source site; a region serves a run of
//            consecutive sites and has its own claim counter, so claims do not contend.  The
//            order of claims changes no result: cluster roots are segment indices and every sum
//            is an exact integer.  Regions keep unused slots at their ends.)
//            vtime u64 (FP64 bits), vcode u8 = g<<1|offdiag,
//            vslot[2] i32 (segment of the leg on source / target site)
//   segments (site-major CSR by sbase, k_s+1 per site, bottom segment first) stime u64,
//            sinfo u8, svert i32, sdir u8, parent i32, flip u8, cls[4] u64, rkw (tau = 0
//            class counts u32[4], winding i32[4]; used at roots)
//   records  rec[step][chain][32] u64 — exact integer sums (see the R_* word map)
#pragma once
#include <cstdint>

#include "lg_numerics.cuh"
#include "lg_types.h"

namespace lg {

// sinfo bits
// SI_SRC: the segment starts at the source-side leg of its vertex; bits 5-6: the vertex's graph;
// SI_OFF: the vertex is off-diagonal
enum : uint8_t { SI_SPIN = 1, SI_GNEG = 2, SI_FIRST = 4, SI_LAST = 8, SI_SRC = 16, SI_OFF = 128 };
constexpr int SI_GSHIFT = 5;

// What k_accumulate gathers for a cluster besides its class lengths, stored at its root's
// segment index (32 bytes, read by k_cluster with the lengths as two requests): the tau = 0
// count of each (spin, gauge sign) class and the winding per lattice direction.  The lengths
// stay in their own array: the counts of a giant cluster's bottom segments and the tiles'
// length flushes then contend on different lines.
struct RootKW {
  unsigned K[4];
  int W[4];
};

struct Arena {
  // static
  const DChain* ch;
  int C, N, NB;
  const int* bond_s0;
  const int* bond_s1;
  const int* bond_chain;
  const uint8_t* bond_dir0;
  const int* inc_off;      // N+1
  const int* inc;          // incident bonds of each site, ascending
  const uint8_t* inc_side; // 0: site is the bond's source, 1: target
  const int* inc_nbr;      // the bond's other site
  const uint8_t* inc_dir;  // the bond's lattice direction (nullptr: 0)
  const int8_t* gauge;     // N
  const int* site_chain;   // N
  // per-chain mutable
  uint32_t* ch_sweep;      // C
  const uint8_t* ch_active;  // C: 0 = retired chain (inserts nothing; its state is dropped)
  int all_active;            // no chain retired: ch_active need not be read
  int* ch_slot_off;        // C+1 (this sweep)
  // persistent site state
  uint8_t* spin0;
  int* off_base;
  int* off_cnt;
  // per-sweep
  int* bond_cnt;           // NB: vertices of the bond this sweep
  int* bond_ptr;           // NB(+1): first vertex of the bond's range
  // vertex regions: site s claims from region site_region[s], whose slots are
  // [region_base[r], region_base[r+1]); region_fill[r] counts the claims (the whole demand,
  // also past the end of the region)
  int R;
  const int* site_region;
  const int* region_base;
  unsigned long long* region_fill;
  int* site_cnt;           // N
  int* sbase;              // N+1
  uint64_t* vtime;
  uint8_t* vcode;
  int* vslot;
  uint64_t* stime;
  uint8_t* sinfo;
  int* svert;
  uint8_t* sdir;
  int* parent;
  uint8_t* flip;
  unsigned long long* cls;  // 4 per segment (used at roots): time-integrated class lengths
  RootKW* rkw;              // per segment (used at roots): tau = 0 class counts, winding
  unsigned long long* rec;  // [rows][C][REC_WORDS]
  Ctl* ctl;
  int rec_rows;             // rows of rec
  // spin correlations (k_corr): work tiles (chain, first entry) and the exact sums per chain
  // entry (arena site index), added over the measured sweeps of the current chunk
  const int2* corr_tiles;
  long long* corr_disp;     // sum_i m_i m_{i+r}, entry r of the chain
  long long* corr_origin;   // m_o m_j, entry j of the chain
};

#define LG_GRID_STRIDE(i, n) \
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__device__ __forceinline__ unsigned long long* rec_row(const Arena& A, int c) {
  return A.rec + ((size_t)A.ctl->step * A.C + c) * REC_WORDS;
}

// ---------------------------------------------------------------------------------------------
// (A sweep starts with its record row and the region claim counters at zero: k_end of the previous
// sweep clears them, the host when it resets the record row counter.)

// ---------------------------------------------------------------------------------------------
// Insertion / removal of operators for one bond (path_integral.C:484-566).
//
// Diagonal proposals: a Poisson stream of rate beta*W_b on [0,1) (superposition of the
// per-graph streams of graph_chooser, graph_impl.h:574-617); graph g with probability v_g/W_b.
// A proposal survives when is_compatible(g, c0(t), c1(t)) = (g&1)^c0^c1 (graph_impl.h:257),
// with the spins at time t read off the previous sweep's off-diagonal lists of both sites
// (diagonal operators never change spins).  The bond's own old off-diagonal operators are kept
// and draw a new graph with probability v0/(v0+v1) for g = 0 (graph_impl.h:323-327).  Old
// diagonal operators are dropped (path_integral.C:515-518).
// The output list is time ordered; at equal times off-diagonal operators come first.
// Returns the number of vertices; with WRITE the list is stored from vertex out0 on.  Without
// WRITE, a LOCAL > 0 keeps the first LOCAL vertices in the caller's buffers lt / lc (thread-local
// memory), so that a short list needs no second walk.
template <bool WRITE, int LOCAL = 0>
__device__ int insert_bond_serial(const Arena& A, int b, int out0, uint64_t* lt = nullptr,
                                  uint8_t* lc = nullptr) {
  {
    const int c = A.bond_chain[b];
    const DChain ch = A.ch[c];
    const uint32_t sweep = A.ch_sweep[c];
    const uint32_t bl = (uint32_t)(b - ch.bond_off);
    const int s0 = A.bond_s0[b], s1 = A.bond_s1[b];
    const uint8_t own = A.bond_dir0[b];
    uint32_t p0 = A.spin0[s0], p1 = A.spin0[s1];
    int i0 = A.off_base[s0], e0 = i0 + A.off_cnt[s0];
    int i1 = A.off_base[s1], e1 = i1 + A.off_cnt[s1];
    uint64_t t0 = i0 < e0 ? A.stime[i0] : TIME_INF;
    uint64_t t1 = i1 < e1 ? A.stime[i1] : TIME_INF;

    // proposal stream state
    uint64_t tq = 0, tp = TIME_INF;
    uint32_t k = 0, gp = 0;
    rnd4 r = {0, 0, 0, 0};
    bool more = ch.inv_rate > 0.0f;
    auto next_prop = [&]() {
      tp = TIME_INF;
      if (!more) return;
      if ((k & 1u) == 0) r = philox(ch.seed, sweep, bl, TAG_PROPOSAL, k >> 1);
      const uint32_t wu = (k & 1u) ? r.z : r.x;
      const uint32_t wg = (k & 1u) ? r.w : r.y;
      ++k;
      const uint32_t tail = (wu >> 9) ? 0u : gap_tail_word(ch.seed, sweep, bl, k - 1);
      const float gap = __fmul_rn(-log_open(gap_uniform(wu, tail)), ch.inv_rate);
      const uint64_t q = gap_fix52(gap, ((uint64_t)(wu & 0x1FFu) << 16) | (wg & 0xFFFFu));
      if (q >= FIX52_ONE) { more = false; return; }
      tq += q;
      if (tq >= FIX52_ONE) { more = false; return; }
      tp = fix52_bits(tq);
      gp = (uint32_t)((uint64_t)wg >= ch.T0) + (uint32_t)((uint64_t)wg >= ch.T1) +
           (uint32_t)((uint64_t)wg >= ch.T2);
    };
    next_prop();

    int out = out0;
    uint32_t ordinal = 0;
    rnd4 ro = {0, 0, 0, 0};
    while (true) {
      if (t0 <= t1 && t0 <= tp) {
        if (t0 == TIME_INF) break;
        p0 ^= 1u;
        if (A.sdir[i0] == own) {
          if (WRITE || LOCAL) {
            if ((ordinal & 3u) == 0) ro = philox(ch.seed, sweep, bl, TAG_OFFDIAG, ordinal >> 2);
            const uint32_t w = (ordinal & 3u) == 0 ? ro.x : (ordinal & 3u) == 1 ? ro.y
                             : (ordinal & 3u) == 2 ? ro.z : ro.w;
            const uint32_t g = ((uint64_t)w < ch.Poff) ? 0u : 1u;
            if (WRITE) {
              A.vtime[out] = t0;
              A.vcode[out] = (uint8_t)((g << 1) | 1u);
            } else if (out - out0 < LOCAL) {
              lt[out - out0] = t0;
              lc[out - out0] = (uint8_t)((g << 1) | 1u);
            }
          }
          ++ordinal;
          ++out;
        }
        ++i0;
        t0 = i0 < e0 ? A.stime[i0] : TIME_INF;
      } else if (t1 <= tp) {
        p1 ^= 1u;
        ++i1;
        t1 = i1 < e1 ? A.stime[i1] : TIME_INF;
      } else {
        if (((gp & 1u) ^ p0 ^ p1) & 1u) {
          if (WRITE) {
            A.vtime[out] = tp;
            A.vcode[out] = (uint8_t)(gp << 1);
          } else if (LOCAL && out - out0 < LOCAL) {
            lt[out - out0] = tp;
            lc[out - out0] = (uint8_t)(gp << 1);
          }
          ++out;
        }
        next_prop();
      }
    }
    return out - out0;
  }
}

// Claims n vertices for bond b from region r; returns the first, or -1 (and flags the sweep)
// when the region is full.  The claim is counted even then, so that region_fill ends at the
// region's demand.
__device__ __forceinline__ int claim_vertices(const Arena& A, int b, int n, int r) {
  if (n == 0) { A.bond_cnt[b] = 0; A.bond_ptr[b] = 0; return 0; }
  const unsigned long long at = atomicAdd(A.region_fill + r, (unsigned long long)n);
  const int base = A.region_base[r];
  A.bond_cnt[b] = n;
  if (at + (unsigned long long)n > (unsigned long long)(A.region_base[r + 1] - base)) {
    A.bond_ptr[b] = 0;
    atomicExch(&A.ctl->err, ERR_OVERFLOW);
    return -1;
  }
  A.bond_ptr[b] = base + (int)at;
  return base + (int)at;
}

// One-thread insertion of bond b: count, claim, write (the same list as the warp form).
__device__ void insert_bond_alone(const Arena& A, int b) {
  const int n = insert_bond_serial<false>(A, b, 0);
  const int at = claim_vertices(A, b, n, A.site_region[A.bond_s0[b]]);
  if (at >= 0) insert_bond_serial<true>(A, b, at);
}


// Warp-parallel form of the same insertion.  One warp per site s handles the bonds s owns
// (s is their source).  The off-diagonal lists of s and of each partner site are staged in
// shared memory; 32 proposals are generated at once (a warp prefix sum of the integer gaps gives
// their times), each proposal's spin parities are binary searches in the staged lists, and the
// time-ordered output is assembled by ranks: an accepted proposal lands after the own
// off-diagonal operators at or before its time, an own off-diagonal operator after the accepted
// proposals strictly before it.  Lists beyond the staging capacity take the serial path, which
// produces the same output.
constexpr int INS_WARPS = 4;
constexpr int INS_CAP = 128;      // staged off-diagonal endpoints per site
constexpr int INS_ACC = 128;      // staged accepted proposals per bond

// Entries of the sorted T[0, n) that are <= t (INCL) or < t.  The probe steps are powers of two
// from the largest one <= n down, so the trip count depends on n only: lanes searching lists of
// the same length never diverge.
template <bool INCL>
__device__ __forceinline__ int count_before(const uint64_t* T, int n, uint64_t t) {
  int pos = 0;
  for (int step = n ? 1 << (31 - __clz(n)) : 0; step > 0; step >>= 1) {
    const int np = pos + step;
    if (np <= n) {
      const uint64_t v = T[np - 1];
      if (INCL ? v <= t : v < t) pos = np;
    }
  }
  return pos;
}
__device__ __forceinline__ int count_le(const uint64_t* T, int n, uint64_t t) {
  return count_before<true>(T, n, t);
}
__device__ __forceinline__ int count_lt(const uint64_t* T, int n, uint64_t t) {
  return count_before<false>(T, n, t);
}

// The vertex count n of a bond is known once its proposals are drawn, so the warp claims its
// range of n vertices (claim_vertices) before it writes the list there: one pass, no scan.
// The warps run over `sites` (nullptr: every site of the arena, in order).
//
// A site that owns two or more bonds (square and cubic lattices) inserts them two at a time, one
// per half-warp: 16 proposals per bond and step instead of 32 for one bond, so two bonds of about
// 32 proposals take about 2.6 steps instead of 3.2, and the staging, the claim and the output of
// the two run side by side.  A proposal's random words, its time and its fate do not depend on the
// lanes it ran on, so both forms produce the same list.

// Staging of one warp: the site's own off-diagonal list, and per half-warp a partner list, the
// bond's own off-diagonal operators and its accepted proposals.
struct InsStage {
  uint64_t offS[INS_CAP];
  uint8_t dirS[INS_CAP];
  uint64_t offT[2][INS_CAP];
  uint64_t ownT[2][INS_CAP];
  uint64_t accT[2][INS_ACC];
  uint8_t accG[2][INS_ACC];
};

// The site's bond of incidence d (its source is the site): the whole warp, staging slot 0.
__device__ __forceinline__ void insert_one(const Arena& A, InsStage& S, int d, int lane, int c,
                                           int reg, int ns_off, uint32_t ps0, int my_b, int my_nt,
                                           int my_tb, uint32_t my_pt, bool s_fits) {
  const unsigned lt = (1u << lane) - 1u;
  const int b = __shfl_sync(0xFFFFFFFFu, my_b, d);
  const int nt_off = __shfl_sync(0xFFFFFFFFu, my_nt, d);
  const int tb_ = __shfl_sync(0xFFFFFFFFu, my_tb, d);
  const uint32_t pt0 = __shfl_sync(0xFFFFFFFFu, my_pt, d);
  if (!s_fits || nt_off > INS_CAP) {
    if (lane == 0) insert_bond_alone(A, b);
    __syncwarp();
    return;
  }
  __syncwarp();
  for (int i = lane; i < nt_off; i += 32) S.offT[0][i] = A.stime[tb_ + i];
  // own off-diagonal operators of bond b, in time order
  int nown = 0;
  for (int i0 = 0; i0 < ns_off; i0 += 32) {
    const int i = i0 + lane;
    const bool own = i < ns_off && S.dirS[i] == (uint8_t)d;
    const unsigned ball = __ballot_sync(0xFFFFFFFFu, own);
    if (own) S.ownT[0][nown + __popc(ball & lt)] = S.offS[i];
    nown += __popc(ball);
  }
  __syncwarp();
  const DChain ch = A.ch[c];
  const uint32_t sweep = A.ch_sweep[c];
  const uint32_t bl = (uint32_t)(b - ch.bond_off);
  // diagonal proposals, 32 at a time
  int nacc = 0;
  bool more = ch.inv_rate > 0.0f;
  uint64_t tbase = 0;
  uint32_t k0 = 0;
  while (more) {
    const uint32_t k = k0 + lane;  // k0 is a multiple of 32: lanes 2i, 2i+1 share a block
    rnd4 r = {0, 0, 0, 0};
    if ((lane & 1) == 0) r = philox(ch.seed, sweep, bl, TAG_PROPOSAL, k >> 1);
    const uint32_t rz = __shfl_xor_sync(0xFFFFFFFFu, r.z, 1);
    const uint32_t rw = __shfl_xor_sync(0xFFFFFFFFu, r.w, 1);
    const uint32_t wu = (k & 1u) ? rz : r.x;
    const uint32_t wg = (k & 1u) ? rw : r.y;
    const uint32_t tail = (wu >> 9) ? 0u : gap_tail_word(ch.seed, sweep, bl, k);
    const float gap = __fmul_rn(-log_open(gap_uniform(wu, tail)), ch.inv_rate);
    uint64_t q = gap_fix52(gap, ((uint64_t)(wu & 0x1FFu) << 16) | (wg & 0xFFFFu));
    const bool stop = q >= FIX52_ONE;
    if (stop) q = 0;
    uint64_t incl = q;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += y;
    }
    const uint64_t tq = tbase + incl;
    const unsigned stops = __ballot_sync(0xFFFFFFFFu, stop);
    const bool valid = ((stops & (lt | (1u << lane))) == 0) && tq < FIX52_ONE;
    const unsigned vb = __ballot_sync(0xFFFFFFFFu, valid);
    bool accept = false;
    uint64_t tp = 0;
    uint32_t g = 0;
    if (valid) {
      tp = fix52_bits(tq);
      g = (uint32_t)((uint64_t)wg >= ch.T0) + (uint32_t)((uint64_t)wg >= ch.T1) +
          (uint32_t)((uint64_t)wg >= ch.T2);
      const uint32_t ps = ps0 ^ (uint32_t)(count_le(S.offS, ns_off, tp) & 1);
      const uint32_t pt = pt0 ^ (uint32_t)(count_le(S.offT[0], nt_off, tp) & 1);
      accept = (((g & 1u) ^ ps ^ pt) & 1u) != 0;
    }
    const unsigned ab = __ballot_sync(0xFFFFFFFFu, accept);
    if (accept) {
      const int pos = nacc + __popc(ab & lt);
      if (pos < INS_ACC) { S.accT[0][pos] = tp; S.accG[0][pos] = (uint8_t)g; }
    }
    nacc += __popc(ab);
    more = vb == 0xFFFFFFFFu;
    tbase = __shfl_sync(0xFFFFFFFFu, tq, 31);
    k0 += 32;
  }
  const int n = nacc + nown;
  int out0 = 0;
  if (lane == 0) out0 = claim_vertices(A, b, n, reg);
  out0 = __shfl_sync(0xFFFFFFFFu, out0, 0);
  if (out0 >= 0 && nacc > INS_ACC) {
    // more accepted proposals than the staging holds: the one-thread form writes the list
    if (lane == 0) insert_bond_serial<true>(A, b, out0);
  } else if (out0 >= 0) {
    for (int j = lane; j < nacc; j += 32) {
      const uint64_t tp = S.accT[0][j];
      const int pos = j + count_le(S.ownT[0], nown, tp);
      A.vtime[out0 + pos] = tp;
      A.vcode[out0 + pos] = (uint8_t)(S.accG[0][j] << 1);
    }
    for (int i = lane; i < nown; i += 32) {
      const uint64_t to = S.ownT[0][i];
      const int pos = i + count_lt(S.accT[0], nacc, to);
      const rnd4 ro = philox(ch.seed, sweep, bl, TAG_OFFDIAG, (uint32_t)i >> 2);
      const uint32_t wv = (i & 3) == 0 ? ro.x : (i & 3) == 1 ? ro.y : (i & 3) == 2 ? ro.z : ro.w;
      const uint32_t g = ((uint64_t)wv < ch.Poff) ? 0u : 1u;
      A.vtime[out0 + pos] = to;
      A.vcode[out0 + pos] = (uint8_t)((g << 1) | 1u);
    }
  }
  __syncwarp();
}

// The site's bonds of incidences da (lanes 0-15, staging slot 0) and db (lanes 16-31, slot 1),
// both with lists that fit the staging.  The same steps as insert_one, 16 proposals per bond and
// step, prefix sums and ballots restricted to the half.
__device__ __forceinline__ void insert_two(const Arena& A, InsStage& S, int da, int db, int lane,
                                           int c, int reg, int ns_off, uint32_t ps0, int my_b,
                                           int my_nt, int my_tb, uint32_t my_pt) {
  const int h = lane >> 4, hl = lane & 15;
  const unsigned hshift = 16u * (unsigned)h;
  const unsigned hlt = (1u << hl) - 1u;
  const int d = h ? db : da;
  const int b = __shfl_sync(0xFFFFFFFFu, my_b, d);
  const int nt_off = __shfl_sync(0xFFFFFFFFu, my_nt, d);
  const int tb_ = __shfl_sync(0xFFFFFFFFu, my_tb, d);
  const uint32_t pt0 = __shfl_sync(0xFFFFFFFFu, my_pt, d);
  uint64_t* offT = S.offT[h];
  uint64_t* ownT = S.ownT[h];
  uint64_t* accT = S.accT[h];
  uint8_t* accG = S.accG[h];
  __syncwarp();
  for (int i = hl; i < nt_off; i += 16) offT[i] = A.stime[tb_ + i];
  // own off-diagonal operators of each half's bond, in time order
  int nown = 0;
  for (int i0 = 0; i0 < ns_off; i0 += 16) {
    const int i = i0 + hl;
    const bool own = i < ns_off && S.dirS[i] == (uint8_t)d;
    const unsigned hb = (__ballot_sync(0xFFFFFFFFu, own) >> hshift) & 0xFFFFu;
    if (own) ownT[nown + __popc(hb & hlt)] = S.offS[i];
    nown += __popc(hb);
  }
  __syncwarp();
  const DChain ch = A.ch[c];
  const uint32_t sweep = A.ch_sweep[c];
  const uint32_t bl = (uint32_t)(b - ch.bond_off);
  int nacc = 0;
  bool more = ch.inv_rate > 0.0f;  // this half's bond still proposes
  uint64_t tbase = 0;
  uint32_t k0 = 0;
  while (__any_sync(0xFFFFFFFFu, more)) {
    const uint32_t k = k0 + (uint32_t)hl;  // k0 is a multiple of 16: lanes 2i, 2i+1 share a block
    rnd4 r = {0, 0, 0, 0};
    if (more && (hl & 1) == 0) r = philox(ch.seed, sweep, bl, TAG_PROPOSAL, k >> 1);
    const uint32_t rz = __shfl_xor_sync(0xFFFFFFFFu, r.z, 1);
    const uint32_t rw = __shfl_xor_sync(0xFFFFFFFFu, r.w, 1);
    const uint32_t wu = (k & 1u) ? rz : r.x;
    const uint32_t wg = (k & 1u) ? rw : r.y;
    uint64_t q = 0;
    bool stop = true;
    if (more) {
      const uint32_t tail = (wu >> 9) ? 0u : gap_tail_word(ch.seed, sweep, bl, k);
      const float gap = __fmul_rn(-log_open(gap_uniform(wu, tail)), ch.inv_rate);
      q = gap_fix52(gap, ((uint64_t)(wu & 0x1FFu) << 16) | (wg & 0xFFFFu));
      stop = q >= FIX52_ONE;
      if (stop) q = 0;
    }
    uint64_t incl = q;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
      const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o, 16);
      if (hl >= o) incl += y;
    }
    const uint64_t tq = tbase + incl;
    const unsigned stops = (__ballot_sync(0xFFFFFFFFu, stop) >> hshift) & 0xFFFFu;
    const bool valid = more && ((stops & (hlt | (1u << hl))) == 0) && tq < FIX52_ONE;
    const unsigned vb = (__ballot_sync(0xFFFFFFFFu, valid) >> hshift) & 0xFFFFu;
    bool accept = false;
    uint64_t tp = 0;
    uint32_t g = 0;
    if (valid) {
      tp = fix52_bits(tq);
      g = (uint32_t)((uint64_t)wg >= ch.T0) + (uint32_t)((uint64_t)wg >= ch.T1) +
          (uint32_t)((uint64_t)wg >= ch.T2);
      const uint32_t ps = ps0 ^ (uint32_t)(count_le(S.offS, ns_off, tp) & 1);
      const uint32_t pt = pt0 ^ (uint32_t)(count_le(offT, nt_off, tp) & 1);
      accept = (((g & 1u) ^ ps ^ pt) & 1u) != 0;
    }
    const unsigned ab = (__ballot_sync(0xFFFFFFFFu, accept) >> hshift) & 0xFFFFu;
    if (accept) {
      const int pos = nacc + __popc(ab & hlt);
      if (pos < INS_ACC) { accT[pos] = tp; accG[pos] = (uint8_t)g; }
    }
    nacc += __popc(ab);
    more = more && vb == 0xFFFFu;
    tbase = __shfl_sync(0xFFFFFFFFu, tq, 15, 16);
    k0 += 16;
  }
  const int n = nacc + nown;
  int out0 = 0;
  if (hl == 0) out0 = claim_vertices(A, b, n, reg);
  out0 = __shfl_sync(0xFFFFFFFFu, out0, 0, 16);
  __syncwarp();
  if (out0 >= 0 && nacc > INS_ACC) {
    // more accepted proposals than the staging holds: the one-thread form writes the list
    if (hl == 0) insert_bond_serial<true>(A, b, out0);
  } else if (out0 >= 0) {
    for (int j = hl; j < nacc; j += 16) {
      const uint64_t tp = accT[j];
      const int pos = j + count_le(ownT, nown, tp);
      A.vtime[out0 + pos] = tp;
      A.vcode[out0 + pos] = (uint8_t)(accG[j] << 1);
    }
    for (int i = hl; i < nown; i += 16) {
      const uint64_t to = ownT[i];
      const int pos = i + count_lt(accT, nacc, to);
      const rnd4 ro = philox(ch.seed, sweep, bl, TAG_OFFDIAG, (uint32_t)i >> 2);
      const uint32_t wv = (i & 3) == 0 ? ro.x : (i & 3) == 1 ? ro.y : (i & 3) == 2 ? ro.z : ro.w;
      const uint32_t g = ((uint64_t)wv < ch.Poff) ? 0u : 1u;
      A.vtime[out0 + pos] = to;
      A.vcode[out0 + pos] = (uint8_t)((g << 1) | 1u);
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(INS_WARPS * 32, 7) k_insert(Arena A, const int* sites, int nsites) {
  if (A.ctl->err) return;
  __shared__ InsStage stage[INS_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  InsStage& S = stage[w];
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; si < nsites; si += warps) {
    const int s = sites ? sites[si] : si;
    // everything the site's bonds need, loaded up front: lane d < z holds incidence d and, for a
    // bond s owns, the partner site's list and spin
    const int j0 = A.inc_off[s];
    const int z = A.inc_off[s + 1] - j0;
    const int c = A.site_chain[s];
    const int reg = A.site_region[s];
    const int ns_off = A.off_cnt[s];
    const int sb = A.off_base[s];
    const uint32_t ps0 = A.spin0[s];
    int my_b = 0, my_side = 1, my_nt = 0, my_tb = 0;
    uint32_t my_pt = 0;
    if (lane < z) {
      my_b = A.inc[j0 + lane];
      my_side = A.inc_side[j0 + lane];
      const int my_t = A.inc_nbr[j0 + lane];
      if (my_side == 0) { my_nt = A.off_cnt[my_t]; my_tb = A.off_base[my_t]; my_pt = A.spin0[my_t]; }
    }
    if (!A.all_active && !A.ch_active[c]) {
      if (lane < z && my_side == 0) { A.bond_cnt[my_b] = 0; A.bond_ptr[my_b] = 0; }
      continue;
    }
    const bool s_fits = ns_off <= INS_CAP;
    if (s_fits) {
      for (int i = lane; i < ns_off; i += 32) { S.offS[i] = A.stime[sb + i]; S.dirS[i] = A.sdir[sb + i]; }
    }
    // bonds owned by s (s is the source), two at a time where both partner lists fit
    const unsigned owned = __ballot_sync(0xFFFFFFFFu, lane < z && my_side == 0);
    const unsigned fits = __ballot_sync(0xFFFFFFFFu, lane < z && my_side == 0 && my_nt <= INS_CAP);
    unsigned rest = owned;
    while (rest) {
      const int da = __ffs(rest) - 1;
      rest &= rest - 1;
      const unsigned pair_ok = s_fits && rest && ((fits >> da) & 1u) ? rest & fits : 0u;
      if (pair_ok) {
        const int db = __ffs(pair_ok) - 1;
        rest &= ~(1u << db);
        insert_two(A, S, da, db, lane, c, reg, ns_off, ps0, my_b, my_nt, my_tb, my_pt);
      } else {
        insert_one(A, S, da, lane, c, reg, ns_off, ps0, my_b, my_nt, my_tb, my_pt, s_fits);
      }
    }
  }
}

// Thread-per-bond form for chains with few operators per bond, where a warp per site would idle:
// the 32 bonds of a warp count their vertices, claim one range with a single atomic add (a warp
// prefix sum places each bond), and write their lists.  A list of up to INS_LOCAL vertices is
// kept in thread-local memory by the counting walk; longer ones are walked again to write them.
constexpr int INS_LOCAL = 16;

__global__ void __launch_bounds__(256, 4) k_insert_narrow(Arena A, const int* bonds, int nb) {
  if (A.ctl->err) return;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;        // a multiple of 32
  const int nround = (nb + 31) & ~31;               // same trip count for every lane of a warp
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += stride) {
    const bool ok = i < nb;
    const int b = ok ? bonds[i] : 0;
    int n = 0;
    uint64_t lt[INS_LOCAL];
    uint8_t lc[INS_LOCAL];
    if (ok && (A.all_active || A.ch_active[A.bond_chain[b]]))
      n = insert_bond_serial<false, INS_LOCAL>(A, b, 0, lt, lc);
    // the bonds of a warp are consecutive, so their regions form runs of lanes: a segmented
    // prefix sum over each run, and one claim per run by its last lane
    const int r = ok ? A.site_region[A.bond_s0[b]] : 0x7FFFFFFF;
    const int rprev = __shfl_up_sync(0xFFFFFFFFu, r, 1);
    const unsigned heads = __ballot_sync(0xFFFFFFFFu, lane == 0 || r != rprev);
    const int seg0 = 31 - __clz(heads & (0xFFFFFFFFu >> (31 - lane)));
    const unsigned later = lane == 31 ? 0u : heads & (0xFFFFFFFEu << lane);
    const int seg1 = later ? __ffs(later) - 2 : 31;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane - o >= seg0) incl += y;
    }
    const int total = __shfl_sync(0xFFFFFFFFu, incl, seg1);
    unsigned long long fill = 0;
    if (lane == seg1 && ok && total) fill = atomicAdd(A.region_fill + r, (unsigned long long)total);
    fill = __shfl_sync(0xFFFFFFFFu, fill, seg1);
    bool room = true;
    int base = 0;
    if (ok) {
      base = A.region_base[r];
      room = fill + (unsigned long long)total <= (unsigned long long)(A.region_base[r + 1] - base);
      if (!room && lane == seg1) atomicExch(&A.ctl->err, ERR_OVERFLOW);
    }
    if (ok) {
      const int at = room ? base + (int)fill + (incl - n) : 0;
      A.bond_cnt[b] = n;
      A.bond_ptr[b] = at;
      if (room && n && n <= INS_LOCAL) {
        for (int j = 0; j < n; ++j) { A.vtime[at + j] = lt[j]; A.vcode[at + j] = lc[j]; }
      } else if (room && n) {
        insert_bond_serial<true>(A, b, at);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Exclusive scan (three phases, fixed grid so the sweep can be captured in a CUDA graph).
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_scan(int v, int* smem_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? smem_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    smem_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  int excl = x - v + (wid > 0 ? smem_warp[wid - 1] : 0);
  *total = smem_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return excl;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int* in, int n, int* partial,
                                                              const Ctl* ctl) {
  if (ctl->err) return;
  __shared__ int sw[32];
  const int base = blockIdx.x * SCAN_TILE;
  int s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int i = base + threadIdx.x * SCAN_ITEMS + j;
    if (i < n) s += in[i];
  }
  int tot;
  block_exclusive_scan(s, sw, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Single block: exclusive scan of the tile partials; writes the grand total to *total_out and
// checks it against cap (sets ERR_OVERFLOW).
__global__ void __launch_bounds__(1024) k_scan_partials(int* partial, int nparts, int* total_out,
                                                        int cap, int per_item, int extra,
                                                        Ctl* ctl) {
  if (ctl->err) return;
  __shared__ int sw[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nparts; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < nparts ? partial[i] : 0;
    int tot;
    int ex = block_exclusive_scan(v, sw, &tot);
    if (i < nparts) partial[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *total_out = carry;
    if ((long long)carry * per_item + extra > (long long)cap) ctl->err = ERR_OVERFLOW;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int* in, int* out, int n,
                                                             const int* partial, const Ctl* ctl) {
  if (ctl->err) return;
  __shared__ int sw[32];
  const int base = blockIdx.x * SCAN_TILE;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int i = base + threadIdx.x * SCAN_ITEMS + j;
    v[j] = i < n ? in[i] : 0;
    s += v[j];
  }
  int tot;
  int ex = block_exclusive_scan(s, sw, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int i = base + threadIdx.x * SCAN_ITEMS + j;
    if (i < n) out[i] = ex;
    ex += v[j];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = ex;
}

// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int site_segments(const Arena& A, int s) {
  int k = 1;
  for (int j = A.inc_off[s]; j < A.inc_off[s + 1]; ++j) k += A.bond_cnt[A.inc[j]];
  return k;
}

// Segment offsets of an arena of at most SITE_SCAN_MAX sites in two launches.  k_site_blocks:
// one site per thread, the block's total into partial[block].  k_site_offsets: every block scans
// the (at most 1024) block totals for its own offset, then its sites; the last block writes the
// total, ns_total, and checks it against ns_cap.  (One block doing all of a 16384-site arena in
// one launch measured 20 against 11.5 us.)
constexpr int SITE_SCAN_BLOCK = 1024;
constexpr int SITE_SCAN_MAX = SITE_SCAN_BLOCK * SITE_SCAN_BLOCK;

__global__ void __launch_bounds__(SITE_SCAN_BLOCK) k_site_blocks(Arena A, int* partial) {
  if (A.ctl->err) return;
  __shared__ int sw[32];
  const int s = blockIdx.x * SITE_SCAN_BLOCK + threadIdx.x;
  int k = 0;
  if (s < A.N) {
    k = site_segments(A, s);
    A.site_cnt[s] = k;
  }
  int tot;
  block_exclusive_scan(k, sw, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SITE_SCAN_BLOCK) k_site_offsets(Arena A, const int* partial) {
  if (A.ctl->err) return;
  __shared__ int sw[32];
  __shared__ int base;
  const int nparts = gridDim.x;
  const int pv = (int)threadIdx.x < nparts ? partial[threadIdx.x] : 0;
  int ptot;
  const int pex = block_exclusive_scan(pv, sw, &ptot);
  if ((int)threadIdx.x == (int)blockIdx.x) base = pex;
  __syncthreads();
  const int s = blockIdx.x * SITE_SCAN_BLOCK + threadIdx.x;
  const int k = s < A.N ? A.site_cnt[s] : 0;
  int tot;
  const int ex = block_exclusive_scan(k, sw, &tot);
  if (s < A.N) A.sbase[s] = base + ex;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    A.sbase[A.N] = ptot;
    A.ctl->ns_total = ptot;
    if (ptot > A.ctl->ns_cap) A.ctl->err = ERR_OVERFLOW;
  }
}

// Per site: number of segments.
__global__ void k_site_count(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(s, A.N) A.site_cnt[s] = site_segments(A, s);
}

// ---------------------------------------------------------------------------------------------
// Per site: merge the time-ordered vertex lists of its incident bonds into the site's segment
// list.  Segment j (0 <= j <= k) starts at the j-th endpoint (the bottom segment j = 0 starts at
// tau = 0) and carries the spin after that endpoint.  Ties: (time, off-diagonal first, bond).
// Also: union-find initialisation and the temporal closure (top segment hooked to the bottom,
// path_integral.C:584-589).
//
// One warp per site.  The incident lists (<= MERGE_CAP endpoints) are staged in shared memory;
// every endpoint finds its merged rank by binary search in the other lists (no sequential
// merge), the spins follow from a warp prefix-XOR of the off-diagonal flags in merged order, and
// the segment arrays are written coalesced.  Sites with more endpoints use the one-thread merge.
constexpr int MERGE_WARPS = 4;
constexpr int MERGE_CAP = 384;        // largest staging capacity per warp
// shared memory of k_merge per warp for a staging capacity of cap endpoints
__host__ __device__ constexpr int merge_smem_per_warp(int cap) { return cap * (8 + 8 + 2 + 2 + 1); }

// Merge key of an endpoint: (time bits << 1) | diagonal.  Times are FP64 bit patterns of values
// in [0, 1), below 2^62, so the key fits; key order is (time, off-diagonal first).
__device__ __forceinline__ uint64_t merge_key(uint64_t t, uint8_t code) {
  return (t << 1) | (uint64_t)(~code & 1u);
}

// One two-way merge by a warp (merge path).  X (nx keys at XK) goes before Y (ny keys at YK) at
// equal keys.  Indices travel with the keys: XI[i], or xb + i when XI is null (the same for Y).
// Each lane takes a contiguous chunk of the output, finds where its chunk starts in X and Y by
// one binary search along its diagonal (the co-rank), then merges the chunk sequentially.
__device__ __forceinline__ void warp_merge2(const uint64_t* XK, const uint16_t* XI, int xb, int nx,
                                            const uint64_t* YK, const uint16_t* YI, int yb, int ny,
                                            uint64_t* OK, uint16_t* OI, int lane) {
  const int n = nx + ny;
  const int per = (n + 31) >> 5;
  const int d0 = min(lane * per, n), d1 = min(d0 + per, n);
  if (d0 >= d1) return;
  int lo = max(0, d0 - ny), hi = min(d0, nx);
  while (lo < hi) {  // smallest i with Y[d0 - i - 1] < X[i]
    const int i = (lo + hi) >> 1;
    if (XK[i] <= YK[d0 - i - 1]) lo = i + 1; else hi = i;
  }
  int i = lo, j = d0 - lo;
  // the head key of each side in a register; an exhausted side reads as ~0 (keys are below 2^63)
  uint64_t xk = i < nx ? XK[i] : ~0ull, yk = j < ny ? YK[j] : ~0ull;
  for (int d = d0; d < d1; ++d) {
    if (xk <= yk) {
      OK[d] = xk;
      OI[d] = XI ? XI[i] : (uint16_t)(xb + i);
      ++i;
      xk = i < nx ? XK[i] : ~0ull;
    } else {
      OK[d] = yk;
      OI[d] = YI ? YI[j] : (uint16_t)(yb + j);
      ++j;
      yk = j < ny ? YK[j] : ~0ull;
    }
  }
}

// Z: the largest site degree of the arena (2, 4, 6, 12 or MAXZ), the bound of every per-list loop.
template <int Z>
__device__ void merge_site_serial(Arena& A, int s) {
  const int j0 = A.inc_off[s];
  const int z = A.inc_off[s + 1] - j0;
  const int base = A.sbase[s];
  const int k = A.sbase[s + 1] - base - 1;
  const uint8_t gneg = A.gauge[s] < 0 ? SI_GNEG : 0;
  int cur[Z], end[Z];
  uint64_t ht[Z];
  uint8_t hc[Z], side[Z];
#pragma unroll
  for (int d = 0; d < Z; ++d) {
    if (d < z) {
      const int b = A.inc[j0 + d];
      cur[d] = A.bond_ptr[b];
      end[d] = cur[d] + A.bond_cnt[b];
      side[d] = A.inc_side[j0 + d];
      ht[d] = cur[d] < end[d] ? A.vtime[cur[d]] : TIME_INF;
      hc[d] = cur[d] < end[d] ? A.vcode[cur[d]] : 0;
    } else {
      cur[d] = end[d] = 0; ht[d] = TIME_INF; hc[d] = 0; side[d] = 0;
    }
  }
  uint8_t spin = A.spin0[s];
  A.stime[base] = 0ull;
  A.sinfo[base] = (uint8_t)(spin | gneg | SI_FIRST | (k == 0 ? SI_LAST : 0));
  A.svert[base] = -1;
  A.sdir[base] = 0xFF;
  A.parent[base] = base;
  for (int j = 1; j <= k; ++j) {
    int best = 0;
    uint64_t bt = ht[0];
    uint8_t bdiag = (uint8_t)(~hc[0] & 1u);
#pragma unroll
    for (int d = 1; d < Z; ++d) {
      const uint8_t dg = (uint8_t)(~hc[d] & 1u);
      if (ht[d] < bt || (ht[d] == bt && dg < bdiag)) { best = d; bt = ht[d]; bdiag = dg; }
    }
    const int x = base + j;
    int v = 0;
    uint8_t sd = 0, code = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) {
      if (d == best) {
        v = cur[d]; sd = side[d]; code = hc[d];
        ++cur[d];
        ht[d] = cur[d] < end[d] ? A.vtime[cur[d]] : TIME_INF;
        hc[d] = cur[d] < end[d] ? A.vcode[cur[d]] : 0;
      }
    }
    if (code & 1u) spin ^= 1u;
    A.stime[x] = bt;
    A.sinfo[x] = (uint8_t)(spin | gneg | (j == k ? SI_LAST : 0) | (sd == 0 ? SI_SRC : 0) |
                           ((code >> 1) << SI_GSHIFT) | ((code & 1u) ? SI_OFF : 0));
    A.svert[x] = v;
    A.sdir[x] = (uint8_t)(best | (A.inc_dir ? A.inc_dir[j0 + best] << SD_DSHIFT : 0));
    A.parent[x] = x;
    A.vslot[2 * v + sd] = x;
  }
  // closure (path_integral.C:584-589); spin-S sites close in k_boundary instead
  if (k > 0 && A.ch[A.site_chain[s]].spin2 <= 1) A.parent[base + k] = base;
}

// `cap` (a multiple of 32, at most MERGE_CAP) is the staging capacity per warp, sized by the
// engine from the arena's largest expected endpoint count per site; the dynamic shared memory is
// MERGE_WARPS * merge_smem_per_warp(cap) bytes.
template <int Z>
__global__ void __launch_bounds__(MERGE_WARPS * 32, 8) k_merge(Arena A, const int* sites, int nsites,
                                                              int cap) {
  if (A.ctl->err) return;
  extern __shared__ __align__(16) unsigned char merge_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned char* wb = merge_smem + (size_t)w * merge_smem_per_warp(cap);
  uint64_t* const wsK = reinterpret_cast<uint64_t*>(wb);              // staged merge keys, list by list
  uint64_t* const wmK = wsK + cap;                                    // merge output (keys)
  uint16_t* const wsI = reinterpret_cast<uint16_t*>(wmK + cap);       // index of the keys in sK (levels >= 2)
  uint16_t* const wmI = wsI + cap;                                    // merge output (staged indices)
  uint8_t* const wsC = reinterpret_cast<uint8_t*>(wmI + cap);         // staged codes
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; si < nsites; si += warps) {
    const int s = sites ? sites[si] : si;
    const int j0 = A.inc_off[s];
    const int z = A.inc_off[s + 1] - j0;
    const int base = A.sbase[s];
    const int k = A.sbase[s + 1] - base - 1;
    const int c = A.site_chain[s];
    if (lane == 0) {
      if (s == A.ch[c].site_off) A.ch_slot_off[c] = base;
      if (s == A.N - 1) A.ch_slot_off[A.C] = base + k + 1;
    }
    if (k > cap) {
      if (lane == 0) merge_site_serial<Z>(A, s);
      __syncwarp();
      continue;
    }
    // stage the incident lists: list d occupies [off[d], off[d+1])
    int off[Z + 1];
    int ptr[Z];
    uint8_t sdv[Z];  // per list: the segment's sdir value (incidence | direction << 5) | side << 7
    off[0] = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) {
      if (d < z) {
        const int b = A.inc[j0 + d];
        ptr[d] = A.bond_ptr[b];
        off[d + 1] = off[d] + A.bond_cnt[b];
        sdv[d] = (uint8_t)(d | (A.inc_dir ? A.inc_dir[j0 + d] << SD_DSHIFT : 0) | (A.inc_side[j0 + d] << 7));
      } else {
        ptr[d] = 0; off[d + 1] = off[d]; sdv[d] = 0;
      }
    }
    // one pass over the site's endpoints, list after list (no lane idles at the end of a list)
    for (int i = lane; i < off[Z]; i += 32) {
      int d = 0;
#pragma unroll
      for (int q = 1; q < Z; ++q) if (i >= off[q]) d = q;
      int v = 0;
#pragma unroll
      for (int q = 0; q < Z; ++q) if (q == d) v = ptr[q] + (i - off[q]);
      const uint8_t c = A.vcode[v];
      wsK[i] = merge_key(A.vtime[v], c);
      wsC[i] = c;
    }
    __syncwarp();
    // The merged order is (time, off-diagonal first, list).  Up to 32 endpoints: every lane
    // takes one and computes its rank directly (its place in its own list plus, per other list,
    // the entries before it; equal keys of an earlier list count as before).  More: the lists
    // are merged pairwise, level by level, in list order (warp_merge2), ping-ponging between sK
    // and mK.  Either way the final keys and staged indices end in fK / fI.
    if (k <= 32) {
      uint64_t key = 0;
      int r = 0;
      if (lane < k) {
        int d = 0;
#pragma unroll
        for (int q = 1; q < Z; ++q) if (lane >= off[q]) d = q;
        key = wsK[lane];
#pragma unroll
        for (int q = 0; q < Z; ++q) {  // lists q >= z are empty
          // keys are below 2^63, so "< key + 1" is "<= key"
          const int c = count_before<false>(wsK + off[q], off[q + 1] - off[q], key + (q < d ? 1u : 0u));
          r += q == d ? lane - off[q] : c;
        }
      }
      __syncwarp();
      if (lane < k) { wmK[r] = key; wmI[r] = (uint16_t)lane; }
      __syncwarp();
    }
    int rs[Z], rn[Z];
#pragma unroll
    for (int q = 0; q < Z; ++q) { rs[q] = off[q]; rn[q] = off[q + 1] - off[q]; }
    int nr = k <= 32 ? 1 : z;
    uint64_t* curK = k <= 32 ? wmK : wsK;
    const uint16_t* curI = k <= 32 ? wmI : nullptr;  // level 0: the index of a key is its position
    bool in_m = k <= 32;
    constexpr int LEVELS = Z <= 2 ? 1 : Z <= 4 ? 2 : Z <= 8 ? 3 : Z <= 16 ? 4 : 5;  // pairwise rounds
#pragma unroll
    for (int level = 0; level < LEVELS; ++level) {
      if (nr <= 1) break;
      uint64_t* nK = in_m ? wsK : wmK;
      uint16_t* nI = in_m ? wsI : wmI;
      int ns2[Z], nn2[Z];
      int o = 0, nn = 0;
#pragma unroll
      for (int p = 0; p < Z; p += 2) {
        if (p + 1 < nr) {
          warp_merge2(curK + rs[p], curI ? curI + rs[p] : nullptr, rs[p], rn[p],
                      curK + rs[p + 1], curI ? curI + rs[p + 1] : nullptr, rs[p + 1], rn[p + 1],
                      nK + o, nI + o, lane);
          ns2[p >> 1] = o; nn2[p >> 1] = rn[p] + rn[p + 1];
          o += rn[p] + rn[p + 1];
          ++nn;
        } else if (p < nr) {  // an odd run out: copied
          for (int i = lane; i < rn[p]; i += 32) {
            nK[o + i] = curK[rs[p] + i];
            nI[o + i] = curI ? curI[rs[p] + i] : (uint16_t)(rs[p] + i);
          }
          ns2[p >> 1] = o; nn2[p >> 1] = rn[p];
          o += rn[p];
          ++nn;
        }
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < Z / 2; ++q) { rs[q] = ns2[q]; rn[q] = nn2[q]; }
      nr = nn;
      curK = nK;
      curI = nI;
      in_m = !in_m;
    }
    if (!curI) {  // a single list: its indices are its positions
      for (int i = lane; i < k; i += 32) { wmK[i] = wsK[i]; wmI[i] = (uint16_t)i; }
      __syncwarp();
      curK = wmK;
      curI = wmI;
    }
    const uint64_t* fK = curK;
    const uint16_t* fI = curI;
    // segments: prefix XOR of off-diagonal flags gives each segment's spin
    const uint8_t gneg = A.gauge[s] < 0 ? SI_GNEG : 0;
    const bool close = A.ch[c].spin2 <= 1;  // spin-S sites close in k_boundary
    uint32_t carry = A.spin0[s];
    if (lane == 0) {
      A.stime[base] = 0ull;
      A.sinfo[base] = (uint8_t)(carry | gneg | SI_FIRST | (k == 0 ? SI_LAST : 0));
      A.svert[base] = -1;
      A.sdir[base] = 0xFF;
      A.parent[base] = base;
    }
    for (int r0 = 0; r0 < k; r0 += 32) {
      const int r = r0 + lane;
      const bool ok = r < k;
      const int e = ok ? fI[r] : 0;
      const uint8_t cd = ok ? wsC[e] : 0;
      const unsigned ball = __ballot_sync(0xFFFFFFFFu, ok && (cd & 1u));
      const uint32_t spin = carry ^ (__popc(ball & (0xFFFFFFFFu >> (31 - lane))) & 1u);
      if (ok) {
        int d = 0;
#pragma unroll
        for (int q = 1; q < Z; ++q) if (e >= off[q]) d = q;
        int pd = 0, od = 0;
        uint8_t sv = 0;
#pragma unroll
        for (int q = 0; q < Z; ++q) if (q == d) { pd = ptr[q]; od = off[q]; sv = sdv[q]; }
        const int v = pd + (e - od);
        const int x = base + 1 + r;
        const uint8_t side = sv >> 7;
        A.stime[x] = fK[r] >> 1;
        A.sinfo[x] = (uint8_t)(spin | gneg | (r == k - 1 ? SI_LAST : 0) | (side == 0 ? SI_SRC : 0) |
                               ((cd >> 1) << SI_GSHIFT) | ((cd & 1u) ? SI_OFF : 0));
        A.svert[x] = v;
        A.sdir[x] = (uint8_t)(sv & 0x7F);
        A.parent[x] = (r == k - 1 && close) ? base : x;  // closure: top segment joins the bottom one
        A.vslot[2 * v + side] = x;
      }
      carry ^= __popc(ball) & 1u;
    }
    __syncwarp();
  }
}

// Thread-per-site form of the merge for sites with few endpoints.
template <int Z>
__global__ void __launch_bounds__(256) k_merge_narrow(Arena A, const int* sites, int nsites) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(i, nsites) {
    const int s = sites[i];
    const int c = A.site_chain[s];
    if (s == A.ch[c].site_off) A.ch_slot_off[c] = A.sbase[s];
    if (s == A.N - 1) A.ch_slot_off[A.C] = A.sbase[s + 1];
    merge_site_serial<Z>(A, s);
  }
}

// The merge kernels for an arena whose sites have at most zmax incident bonds: the instance
// with the smallest list bound Z >= zmax (fewer registers and pairwise rounds).
inline int merge_z(int zmax) {
  return zmax <= 2 ? 2 : zmax <= 4 ? 4 : zmax <= 6 ? 6 : zmax <= 12 ? 12 : MAXZ;
}

inline void launch_merge(int zmax, int grid, size_t smem, cudaStream_t st, const Arena& A,
                         const int* sites, int n, int cap) {
  const int z = merge_z(zmax);
  if (z == 2) k_merge<2><<<grid, MERGE_WARPS * 32, smem, st>>>(A, sites, n, cap);
  else if (z == 4) k_merge<4><<<grid, MERGE_WARPS * 32, smem, st>>>(A, sites, n, cap);
  else if (z == 6) k_merge<6><<<grid, MERGE_WARPS * 32, smem, st>>>(A, sites, n, cap);
  else if (z == 12) k_merge<12><<<grid, MERGE_WARPS * 32, smem, st>>>(A, sites, n, cap);
  else k_merge<MAXZ><<<grid, MERGE_WARPS * 32, smem, st>>>(A, sites, n, cap);
}

inline void launch_merge_narrow(int zmax, int grid, cudaStream_t st, const Arena& A,
                                const int* sites, int n) {
  const int z = merge_z(zmax);
  if (z == 2) k_merge_narrow<2><<<grid, 256, 0, st>>>(A, sites, n);
  else if (z == 4) k_merge_narrow<4><<<grid, 256, 0, st>>>(A, sites, n);
  else if (z == 6) k_merge_narrow<6><<<grid, 256, 0, st>>>(A, sites, n);
  else if (z == 12) k_merge_narrow<12><<<grid, 256, 0, st>>>(A, sites, n);
  else k_merge_narrow<MAXZ><<<grid, 256, 0, st>>>(A, sites, n);
}

// Imaginary-time boundary of a spin-S site (spin2 > 1 virtual sites, path_integral.C:590-613 with
// permutation.h:91-111): the bottom of virtual site a joins the top of virtual site pair[a], and
// both carry the same spin.  Per spin value c the tops with spin c, in index order, are shuffled
// by Fisher-Yates: step k (from the last position down; position i swaps with
// j = floor(w (i+1) / 2^32)) takes Philox word 8c + k of (seed, sweep, real site, TAG_PERM).  The
// bottoms with spin c, in index order, take the shuffled tops in order.  This is a uniform
// matching within each spin sector, as the reference's partitioned random shuffle.  False if the
// two sectors differ in size (a configuration that is not periodic in imaginary time).
__device__ __forceinline__ bool boundary_pairs(uint64_t seed, uint32_t sweep, uint32_t rs, int spin2,
                                               const uint8_t* bottom, const uint8_t* top, int* pair) {
  for (int c = 0; c < 2; ++c) {
    int T[8], B[8], nt = 0, nb = 0;
    for (int a = 0; a < spin2; ++a) {
      if (top[a] == c) T[nt++] = a;
      if (bottom[a] == c) B[nb++] = a;
    }
    if (nt != nb) return false;
    for (int i = nt - 1, k = 0; i >= 1; --i, ++k) {
      const int q = 8 * c + k;
      const rnd4 r = philox(seed, sweep, rs, TAG_PERM, (uint32_t)(q >> 2));
      const uint32_t w = (q & 3) == 0 ? r.x : (q & 3) == 1 ? r.y : (q & 3) == 2 ? r.z : r.w;
      const int j = (int)(((uint64_t)w * (uint64_t)(i + 1)) >> 32);
      const int t = T[i]; T[i] = T[j]; T[j] = t;
    }
    for (int k = 0; k < nb; ++k) pair[B[k]] = T[k];
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Lock-free union-find on segments.  Roots are hooked larger-index -> smaller-index with
// atomicCAS, so the root of every cluster is its smallest segment index whatever the order of
// the unions (the deterministic unify of union_find.h:231-233,270-273).  Finds halve paths with
// plain stores: a store only ever replaces a non-root's parent by one of its ancestors.
// uf_find with the first parent read, p = P[x], already made by the caller.
__device__ __forceinline__ int uf_find_from(int* P, int x, int p) {
  while (true) {
    if (p == x) return x;
    const int gp = __ldcg(P + p);
    if (gp == p) return p;
    P[x] = gp;
    x = gp;
    p = __ldcg(P + x);
  }
}

// The retry cap of the unions of a sweep: Ctl::iter_cap, 0 meaning ITER_CAP; a negative value
// lets no union run at all (a test seam for the LG_EITERCAP path).
__device__ __forceinline__ int iter_cap_of(const Ctl* c) {
  const int v = c->iter_cap;
  return v < 0 ? 0 : (v == 0 ? ITER_CAP : v);
}

// The first parent reads of both finds are issued together (one round trip instead of two when
// both nodes are roots).  Hooks always go from a larger to a smaller index, so parent pointers
// decrease along every path and no interleaving of unions can close a cycle.
__device__ __forceinline__ bool uf_union(int* P, int a, int b, int cap = ITER_CAP) {
  for (int it = 0; it < cap; ++it) {
    const int pa = __ldcg(P + a), pb = __ldcg(P + b);
    a = uf_find_from(P, a, pa);
    b = uf_find_from(P, b, pb);
    if (a == b) return true;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int old = atomicCAS(P + hi, hi, lo);
    if (old == hi) return true;
    a = lo;
    b = old;
  }
  return false;
}

// One thread per spin-S real site: the boundary pairs are united (uf_union: hooks from the larger
// segment index to the smaller).  A virtual site without operators has one segment, which is both
// its bottom and its top and so can be in two pairs; the unions keep both links.  The segments
// of a real site belong to its thread alone until k_union starts.
__global__ void __launch_bounds__(256) k_boundary(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(s, A.N) {
    const int c = A.site_chain[s];
    const int sp2 = A.ch[c].spin2;
    if (sp2 <= 1) continue;
    const int loc = s - A.ch[c].site_off;
    if (loc % sp2) continue;
    int bot[8], top[8], pair[8];
    uint8_t bs[8], ts[8];
    for (int a = 0; a < sp2; ++a) {
      bot[a] = A.sbase[s + a];
      top[a] = A.sbase[s + a + 1] - 1;
      bs[a] = A.spin0[s + a];
      ts[a] = A.sinfo[top[a]] & SI_SPIN;
    }
    if (!boundary_pairs(A.ch[c].seed, A.ch_sweep[c], (uint32_t)(loc / sp2), sp2, bs, ts, pair)) {
      atomicExch(&A.ctl->err, ERR_BOUNDARY);
      continue;
    }
    bool ok = true;
    const int cap = iter_cap_of(A.ctl);
    for (int a = 0; a < sp2; ++a) ok &= uf_union(A.parent, bot[a], top[pair[a]], cap);
    if (!ok) atomicExch(&A.ctl->err, ERR_ITERCAP);
  }
}

// reconnect (graph_impl.h:280-295) in segment form: g = 0 joins the two lower legs and the two
// upper legs; g = 1 joins lower-left with upper-right and lower-right with upper-left; frozen
// graphs (g & 2) join all four legs.
//
// The warps run over chunks of 64 consecutive segments (site-major order); the source-side
// segments of a chunk, about half of them, are compacted so that every lane makes the unions of
// one vertex.  Neighbouring warps so work on neighbouring sites, whatever order the vertex
// ranges were claimed in, which keeps the union-find trees of concurrently running blocks local.
constexpr int UN_WARPS = 8;   // default warps per block
constexpr int UN_CHUNK = 64;

// The lower-leg pairs first (arenas of spin-1/2 chains only).  Every segment ends at exactly one
// vertex (the top segment of a site at tau = 1 instead), so the lower-leg unions (a-1, b-1) of the
// non-crossing vertices (g != 1) form a matching, and every segment in it is still a root when this
// kernel runs: k_merge hooks only top segments (the closure), which end at no vertex.  Each pair is
// therefore hooked with one plain store, P[max] = min, no find and no CAS.  This is half of the
// unions of a loop model with g = 0 graphs (the antiferromagnetic Heisenberg model); k_union<W,
// true> then makes the rest on a forest of depth-one trees.  The pass also replaces svert[x] of
// every source-side segment x by the target-side segment b of its vertex (nothing after the
// unions reads svert), so that k_union<W, true> finds b in the same round trip as the segment's
// info.  With spin S > 1/2, k_boundary unites bottom segments before k_union, so the matching's
// segments need not be roots and this pass is not used.
constexpr int UP_PER = 4;  // segments per thread and step of k_union_pairs, loads issued together

__global__ void __launch_bounds__(256) k_union_pairs(Arena A) {
  if (A.ctl->err) return;
  if (iter_cap_of(A.ctl) == 0) return;  // the test seam that lets no union run
  const int ns = A.ctl->ns_total;
  const long long step = (long long)gridDim.x * 256 * UP_PER;
  for (long long x0 = (long long)blockIdx.x * 256 * UP_PER + threadIdx.x; x0 < ns; x0 += step) {
    uint8_t info[UP_PER];
    int v[UP_PER], b[UP_PER];
#pragma unroll
    for (int j = 0; j < UP_PER; ++j) {
      const long long x = x0 + j * 256;
      info[j] = x < ns ? A.sinfo[x] : 0;
      v[j] = x < ns ? A.svert[x] : 0;
    }
#pragma unroll
    for (int j = 0; j < UP_PER; ++j) b[j] = (info[j] & SI_SRC) ? A.vslot[2 * v[j] + 1] : 0;
#pragma unroll
    for (int j = 0; j < UP_PER; ++j) {
      if (!(info[j] & SI_SRC)) continue;
      const int x = (int)(x0 + j * 256);
      A.svert[x] = b[j];
      if (((info[j] >> SI_GSHIFT) & 3) == 1) continue;
      const int lo = min(x, b[j]) - 1, hi = max(x, b[j]) - 1;
      A.parent[hi] = lo;
    }
  }
}

// PAIRS_DONE: k_union_pairs has made the lower-leg unions of the non-crossing vertices and left
// the target-side segment of each source-side segment's vertex in svert.
template <int WARPS = UN_WARPS, bool PAIRS_DONE = false>
__global__ void __launch_bounds__(WARPS * 32) k_union(Arena A) {
  if (A.ctl->err) return;
  __shared__ int pend[WARPS][UN_CHUNK];   // source-side segment a
  __shared__ int pb[WARPS][UN_CHUNK];     // target-side segment b of the same vertex
  __shared__ uint8_t pg[WARPS][UN_CHUNK]; // graph
  const int ns = A.ctl->ns_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const long long stride = (long long)gridDim.x * WARPS * UN_CHUNK;
  const int cap = iter_cap_of(A.ctl);
  bool ok = true;
  for (long long c0 = ((long long)blockIdx.x * WARPS + w) * UN_CHUNK; c0 < ns; c0 += stride) {
    const int x0 = (int)c0 + lane, x1 = x0 + 32;
    // segment info and vertex of both halves of the chunk in one round trip, then the target
    // leg of the source-side ones
    const uint8_t i0 = x0 < ns ? A.sinfo[x0] : 0;
    const uint8_t i1 = x1 < ns ? A.sinfo[x1] : 0;
    const int v0 = x0 < ns ? A.svert[x0] : 0;
    const int v1 = x1 < ns ? A.svert[x1] : 0;
    const bool s0 = (i0 & SI_SRC) != 0, s1 = (i1 & SI_SRC) != 0;
    // after k_union_pairs, svert of a source-side segment is already the target-side segment
    const int b0 = s0 ? (PAIRS_DONE ? v0 : A.vslot[2 * v0 + 1]) : 0;
    const int b1 = s1 ? (PAIRS_DONE ? v1 : A.vslot[2 * v1 + 1]) : 0;
    const unsigned m0 = __ballot_sync(0xFFFFFFFFu, s0), m1 = __ballot_sync(0xFFFFFFFFu, s1);
    const int n0 = __popc(m0), tot = n0 + __popc(m1);
    if (s0) { const int q = __popc(m0 & lt); pend[w][q] = x0; pb[w][q] = b0; pg[w][q] = (i0 >> SI_GSHIFT) & 3; }
    if (s1) { const int q = n0 + __popc(m1 & lt); pend[w][q] = x1; pb[w][q] = b1; pg[w][q] = (i1 >> SI_GSHIFT) & 3; }
    __syncwarp();
    for (int j = lane; j < tot; j += 32) {
      const int a = pend[w][j], b = pb[w][j], g = pg[w][j];
      int* P = A.parent;
      if (g == 1) {
        ok &= uf_union(P, a - 1, b, cap);
        ok &= uf_union(P, b - 1, a, cap);
      } else {
        if (!PAIRS_DONE) ok &= uf_union(P, a - 1, b - 1, cap);
        ok &= uf_union(P, a, b, cap);
        if (g & 2) ok &= uf_union(P, a - 1, a, cap);
      }
    }
    __syncwarp();
  }
  if (!ok) atomicExch(&A.ctl->err, ERR_ITERCAP);
}

// The same unions with the work of a warp balanced over its lanes.  In k_union every lane makes the
// unions of one vertex, and the warp runs until its slowest lane is done: the longest find path of
// 32.  Here each warp keeps the unions of its chunks in a shared-memory queue, and every step a
// lane that has finished takes the next one, so a long path holds up one lane, not 32.  A step is
// one round trip: the parents of both current nodes are read together; a node whose parent is
// not itself moves to it, and the node it came from is pointed at that parent (path splitting:
// every pointer only moves to an ancestor, which keeps parents below their children); when both
// are roots, the larger is hooked under the smaller with a CAS (a failed CAS continues from the
// root that won).  The warps are persistent (one grid over the GPU) and stride over the chunks.
// PAIRS_DONE: k_union_pairs has run (the lower-leg pairs are hooked, svert holds the target-side
// segment of each source-side one).
constexpr int UB_WARPS = 8;
// Pending unions per warp: fewer than 32 before a chunk is added, and a chunk adds at most 3 per
// source-side segment, 3 * UN_CHUNK = 192: never more than 223 at once.
constexpr int UB_QUEUE = 256;

template <bool PAIRS_DONE>
__global__ void __launch_bounds__(UB_WARPS * 32, 8) k_union_bal(Arena A) {
  if (A.ctl->err) return;
  __shared__ int qa[UB_WARPS][UB_QUEUE];
  __shared__ int qb[UB_WARPS][UB_QUEUE];
  const int ns = A.ctl->ns_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int nwarps = gridDim.x * UB_WARPS;
  const int nchunks = (ns + UN_CHUNK - 1) / UN_CHUNK;
  const int cap = iter_cap_of(A.ctl);
  if (cap == 0) {  // the test seam that lets no union run: the sweep stops with LG_EITERCAP
    if (blockIdx.x == 0 && threadIdx.x == 0 && nchunks > 0) atomicExch(&A.ctl->err, ERR_ITERCAP);
    return;
  }
  int* P = A.parent;
  int chunk = blockIdx.x * UB_WARPS + w;
  unsigned head = 0, tail = 0;  // the warp's queue is [head, tail), indices mod UB_QUEUE
  int x = 0, y = 0, prevx = -1, prevy = -1, iters = 0;
  bool busy = false, ok = true;
  while (true) {
    // refill while the queue cannot feed every lane and chunks remain (warp-uniform)
    while (tail - head < 32u && chunk < nchunks) {
      // both halves of the chunk: info and vertex (or, after k_union_pairs, the target-side
      // segment) in one round trip
      const int xh0 = chunk * UN_CHUNK + lane, xh1 = xh0 + 32;
      const uint8_t ih0 = xh0 < ns ? A.sinfo[xh0] : 0, ih1 = xh1 < ns ? A.sinfo[xh1] : 0;
      const int vh0 = xh0 < ns ? A.svert[xh0] : 0, vh1 = xh1 < ns ? A.svert[xh1] : 0;
      int bh0 = vh0, bh1 = vh1;
      if (!PAIRS_DONE) {
        bh0 = (ih0 & SI_SRC) ? A.vslot[2 * vh0 + 1] : 0;
        bh1 = (ih1 & SI_SRC) ? A.vslot[2 * vh1 + 1] : 0;
      }
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int xs = half ? xh1 : xh0;
        const uint8_t info = half ? ih1 : ih0;
        int n = 0, u0a = 0, u0b = 0, u1a = 0, u1b = 0, u2a = 0, u2b = 0;
        if (info & SI_SRC) {
          const int a = xs;
          const int b = half ? bh1 : bh0;
          const int g = (info >> SI_GSHIFT) & 3;
          if (g == 1) {
            u0a = a - 1; u0b = b; u1a = b - 1; u1b = a; n = 2;
          } else {
            u0a = a; u0b = b; n = 1;
            if (g & 2) { u1a = a - 1; u1b = a; n = 2; }
            if (!PAIRS_DONE) {
              if (n == 1) { u1a = a - 1; u1b = b - 1; } else { u2a = a - 1; u2b = b - 1; }
              ++n;
            }
          }
        }
        // exclusive prefix of n over the warp
        int pre = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xFFFFFFFFu, pre, o);
          if (lane >= o) pre += v;
        }
        const int tot = __shfl_sync(0xFFFFFFFFu, pre, 31);
        const unsigned at = tail + (unsigned)(pre - n);
        if (n > 0) { qa[w][at % UB_QUEUE] = u0a; qb[w][at % UB_QUEUE] = u0b; }
        if (n > 1) { qa[w][(at + 1) % UB_QUEUE] = u1a; qb[w][(at + 1) % UB_QUEUE] = u1b; }
        if (n > 2) { qa[w][(at + 2) % UB_QUEUE] = u2a; qb[w][(at + 2) % UB_QUEUE] = u2b; }
        tail += (unsigned)tot;
      }
      chunk += nwarps;
    }
    __syncwarp();
    // lanes without a union take the next pending ones, in queue order
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !busy);
    const unsigned avail = tail - head;
    if (!busy) {
      const unsigned r = (unsigned)__popc(idle & lt);
      if (r < avail) {
        x = qa[w][(head + r) % UB_QUEUE];
        y = qb[w][(head + r) % UB_QUEUE];
        prevx = prevy = -1;
        iters = 0;
        busy = true;
      }
    }
    head += min(avail, (unsigned)__popc(idle));
    if (!__any_sync(0xFFFFFFFFu, busy)) break;  // queue empty and no chunk left
    __syncwarp();
    if (busy) {
      const int px = __ldcg(P + x), py = __ldcg(P + y);
      // path splitting: the node a step came from now points at its grandparent
      if (prevx >= 0 && px != x) P[prevx] = px;
      if (prevy >= 0 && py != y) P[prevy] = py;
      if (x == y || px == py || px == y || py == x) {
        busy = false;  // a common ancestor: already one set
      } else if (px == x && py == y) {
        const int lo = x < y ? x : y, hi = x < y ? y : x;
        const int old = atomicCAS(P + hi, hi, lo);
        if (old == hi) {
          busy = false;
        } else {  // hi was hooked meanwhile: go on from the root it went under
          x = lo; y = old;
          prevx = prevy = -1;
        }
      } else {
        if (px != x) { prevx = x; x = px; } else prevx = -1;
        if (py != y) { prevy = y; y = py; } else prevy = -1;
      }
      if (busy && ++iters >= cap) { ok = false; busy = false; }
    }
  }
  if (!ok) atomicExch(&A.ctl->err, ERR_ITERCAP);
}

__global__ void __launch_bounds__(256) k_compress(Arena A) {
  if (A.ctl->err) return;
  const int ns = A.ctl->ns_total;
  LG_GRID_STRIDE(x, ns) {
    int r = x;
    int p = A.parent[r];
    while (p != r) { r = p; p = A.parent[r]; }
    A.parent[x] = r;
    if (r == x && A.rkw) {
#pragma unroll
      for (int q = 0; q < 4; ++q) A.cls[4 * (size_t)x + q] = 0ull;
      A.rkw[x] = RootKW{};
    }
  }
}

// Per segment: find its cluster root (and store it: parent := root), then add the segment's
// length in 2^-40 units to one of four class sums of the root, class = (spin, gauge sign).
// Bottom segments also count into the tau = 0 class counts.  These eight integers per cluster
// determine every improved estimator of susceptibility.h:96-156 and the field weight of
// cluster.h:54-59.
//
// At low temperature a few clusters own a large share of all segments, so the additions are
// combined before they reach global memory: each block keeps a shared-memory hash of (root,
// class) sums for its tile of ACC_TILE consecutive segments, flushed with one global atomic per
// entry.  (Summing the lanes of a warp with the same (root, class) first, with match_any and
// reductions, removes most same-address conflicts of the shared atomics but doubles the
// instructions; it measured 76 -> 137 us on the 128^2, beta = 64 sweep.)
// The class sums are zero on entry: k_cluster clears what it consumes.
constexpr int ACC_TILE = 1024;
constexpr int ACC_HASH = 1024;   // power of two

// What one segment adds to its cluster: its length in 2^-40 units to class q = (spin, gauge
// sign), and the winding per lattice direction (stiffness.h:82-130 through
// improved_accumulator::begin_b / end_b): at the source-side leg of a non-frozen bond vertex, the
// segment starting there loses (1-2c) e_d and the segment ending there gains (1-2c) e_d, c being
// the segment's spin and d the bond's direction (sdir bits 3-4).  info1 / tb / dir1 describe the
// next segment of the site (unused for the top segment, which ends at tau = 1).
struct SegContrib {
  unsigned long long len;
  int q;
  int w[3];
};

__device__ __forceinline__ SegContrib seg_contrib(uint8_t info, uint8_t info1, uint64_t ta,
                                                  uint64_t tb, uint8_t dir, uint8_t dir1) {
  SegContrib c;
  const int64_t lo = bits_fix40(ta);
  const int64_t hi = (info & SI_LAST) ? ((int64_t)1 << 40) : bits_fix40(tb);
  c.len = (unsigned long long)(hi - lo);
  c.q = (info & SI_SPIN) * 2 + ((info & SI_GNEG) ? 1 : 0);
  c.w[0] = c.w[1] = c.w[2] = 0;
  const int sg = (info & SI_SPIN) ? -1 : 1;
  if ((info & SI_SRC) && !((info >> SI_GSHIFT) & 2)) c.w[(dir >> SD_DSHIFT) & 3] -= sg;
  if (!(info & SI_LAST) && (info1 & SI_SRC) && !((info1 >> SI_GSHIFT) & 2))
    c.w[(dir1 >> SD_DSHIFT) & 3] += sg;
  return c;
}

template <int TILE = ACC_TILE>
__global__ void __launch_bounds__(256, 4) k_accumulate(Arena A) {
  if (A.ctl->err) return;
  __shared__ int hkey[ACC_HASH];
  // class sums of the hash entries as two 32-bit words: 32-bit shared-memory atomics are
  // single instructions, 64-bit ones are not.  hhi counts every wrap of hlo once, whatever the
  // order of the additions, so hhi * 2^32 + hlo is the exact sum (below 2^50 per tile).
  __shared__ unsigned hlo[ACC_HASH * 4];
  __shared__ unsigned hhi[ACC_HASH * 4];
  // winding sums of the hash entries: w0 + 65536 w1 in hwa, w2 in hwb (a tile's sums stay
  // within +-2 TILE, so both fields of hwa decode exactly)
  __shared__ int hwa[ACC_HASH];
  __shared__ int hwb[ACC_HASH];
  const int ns = A.ctl->ns_total;
  const int ntiles = (ns + TILE - 1) / TILE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int i = threadIdx.x; i < ACC_HASH; i += blockDim.x) {
      hkey[i] = -1;
      hlo[4 * i] = hlo[4 * i + 1] = hlo[4 * i + 2] = hlo[4 * i + 3] = 0u;
      hhi[4 * i] = hhi[4 * i + 1] = hhi[4 * i + 2] = hhi[4 * i + 3] = 0u;
      hwa[i] = hwb[i] = 0;
    }
    __syncthreads();
    const int t0 = tile * TILE;
    constexpr int PER = TILE / 256;  // segments per thread (blockDim.x == 256)
    // Each segment is reduced to what it adds as soon as its loads arrive: its length (u64) and
    // one packed word, class q (bits 0-1), first segment (bit 2), winding + 2 per direction (3
    // bits each from bit 3; each is in [-2, 2]).  Eight segments then keep 4 registers each
    // instead of their raw fields, so the 2048-segment tile does not halve the occupancy.
    int par[PER];
    unsigned long long len[PER];
    unsigned meta[PER];
    // issue every load of this thread's segments first, then walk and add
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int x = t0 + threadIdx.x + j * 256;
      par[j] = x;
      len[j] = 0;
      meta[j] = 0;
      if (x < ns) {
        par[j] = A.parent[x];
        const uint8_t info = A.sinfo[x];
        const uint8_t dir = A.sdir[x];
        const uint64_t ta = A.stime[x];
        const bool last = info & SI_LAST;
        const uint64_t tb = last ? 0ull : A.stime[x + 1];
        const uint8_t info1 = last ? 0 : A.sinfo[x + 1];
        const uint8_t dir1 = last ? 0 : A.sdir[x + 1];
        const SegContrib sc = seg_contrib(info, info1, ta, tb, dir, dir1);
        len[j] = sc.len;
        meta[j] = (unsigned)sc.q | ((info & SI_FIRST) ? 4u : 0u) | ((unsigned)(sc.w[0] + 2) << 3) |
                  ((unsigned)(sc.w[1] + 2) << 6) | ((unsigned)(sc.w[2] + 2) << 9);
      }
    }
    // root walks of this thread's segments in lockstep (their parent reads in flight together)
    int rt[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) rt[j] = t0 + threadIdx.x + j * 256;
    for (int it = 0; it < ITER_CAP; ++it) {
      unsigned moved = 0;
#pragma unroll
      for (int j = 0; j < PER; ++j)
        if (par[j] != rt[j]) { rt[j] = par[j]; moved |= 1u << j; }
      if (!moved) break;
#pragma unroll
      for (int j = 0; j < PER; ++j)
        if (moved & (1u << j)) par[j] = A.parent[rt[j]];
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int x = t0 + threadIdx.x + j * 256;
      if (x >= ns) continue;
      const int r = rt[j];
      if (r != x) A.parent[x] = r;
      const unsigned long long ln = len[j];
      const unsigned mt = meta[j];
      const int q = (int)(mt & 3u);
      const int w[3] = {(int)((mt >> 3) & 7u) - 2, (int)((mt >> 6) & 7u) - 2, (int)((mt >> 9) & 7u) - 2};
      if (mt & 4u) atomicAdd(&A.rkw[r].K[q], 1u);
      const bool wnz = (w[0] | w[1] | w[2]) != 0;
      if (ln || wnz) {
        unsigned h = ((unsigned)r * 2654435761u) >> 22;  // 10-bit hash
        bool done = false;
        for (int probe = 0; probe < 32; ++probe) {
          // a slot's key never changes once set: read it first, CAS only an empty one
          int k = hkey[h];
          if (k == -1) k = atomicCAS(hkey + h, -1, r);
          if (k == -1 || k == r) {
            if (ln) {
              const unsigned lo = (unsigned)ln, hi = (unsigned)(ln >> 32);
              const unsigned old = atomicAdd(hlo + 4 * h + q, lo);
              const unsigned carry = (old + lo < old) ? 1u : 0u;
              if (hi + carry) atomicAdd(hhi + 4 * h + q, hi + carry);
            }
            if (w[0] | w[1]) atomicAdd(hwa + h, w[0] + 65536 * w[1]);
            if (w[2]) atomicAdd(hwb + h, w[2]);
            done = true;
            break;
          }
          h = (h + 1) & (ACC_HASH - 1);
        }
        if (!done) {
          if (ln) atomicAdd(A.cls + 4 * (size_t)r + q, ln);
#pragma unroll
          for (int d = 0; d < 3; ++d)
            if (w[d]) atomicAdd(&A.rkw[r].W[d], w[d]);
        }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ACC_HASH; i += blockDim.x) {
      const int k = hkey[i];
      if (k >= 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const unsigned long long v = ((unsigned long long)hhi[4 * i + q] << 32) | hlo[4 * i + q];
          if (v) atomicAdd(A.cls + 4 * (size_t)k + q, v);
        }
        const int wa = hwa[i];
        const int w0 = ((wa + 32768) & 0xFFFF) - 32768;
        const int w1 = (wa - w0) / 65536;
        if (w0) atomicAdd(&A.rkw[k].W[0], w0);
        if (w1) atomicAdd(&A.rkw[k].W[1], w1);
        if (hwb[i]) atomicAdd(&A.rkw[k].W[2], hwb[i]);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// 128-bit helpers for the exact per-sweep sums.
struct u128 { unsigned long long lo, hi; };

__device__ __forceinline__ u128 mul64(unsigned long long a, unsigned long long b) {
  return {a * b, __umul64hi(a, b)};
}

__device__ __forceinline__ void atomic_add_u128(unsigned long long* p, u128 v) {
  const unsigned long long old = atomicAdd(p, v.lo);
  const unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
  if (v.hi + carry) atomicAdd(p + 1, v.hi + carry);
}

__device__ __forceinline__ int chain_of_segment(const Arena& A, int x) {
  int lo = 0, hi = A.C - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (A.ch_slot_off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The 18 per-sweep sums a cluster root contributes to its chain's record.
constexpr int NQ = 14;  // u64 sums of a root
struct RootSums {
  unsigned long long q[NQ];  // R_NC, R_M0, R_SM0, R_M0SQ, R_N0SQ, R_SM0SQ, R_SN0SQ, R_FLD, R_MA, R_SMA,
                             // R_WSQ, R_W0, R_W1, R_W2
  u128 w[8];                 // R_M0Q, R_N0Q, R_SM0Q, R_SN0Q, R_LSQ, R_MSQ, R_SLSQ, R_SMSQ
};
__device__ __constant__ int kRecQ[NQ] = {R_NC, R_M0, R_SM0, R_M0SQ, R_N0SQ, R_SM0SQ, R_SN0SQ,
                                         R_FLD, R_MA, R_SMA, R_WSQ, R_W0, R_W1, R_W2};
__device__ __constant__ int kRecW[8] = {R_M0Q, R_N0Q, R_SM0Q, R_SN0Q, R_LSQ, R_MSQ, R_SLSQ, R_SMSQ};
constexpr int QLIMB = NQ * 4;            // 16-bit limbs of the u64 sums
constexpr int NLIMB = QLIMB + 8 * 8;      // and of the u128 ones

__device__ __forceinline__ void add_u128(u128& a, u128 b) {
  const unsigned long long lo = a.lo + b.lo;
  a.hi += b.hi + (lo < a.lo ? 1ull : 0ull);
  a.lo = lo;
}

// The class integers of a root: four time-integrated length sums, four tau = 0 counts, and the
// winding per direction.
struct RootClass { unsigned long long S[4]; unsigned K[4]; int Wd[3]; };

__device__ __forceinline__ RootClass load_root_class(const Arena& A, int x) {
  RootClass rc;
  const ulonglong2* S = reinterpret_cast<const ulonglong2*>(A.cls + 4 * (size_t)x);
  const ulonglong2 a = S[0], b = S[1];
  rc.S[0] = a.x; rc.S[1] = a.y; rc.S[2] = b.x; rc.S[3] = b.y;
  const uint4 k = *reinterpret_cast<const uint4*>(A.rkw[x].K);
  rc.K[0] = k.x; rc.K[1] = k.y; rc.K[2] = k.z; rc.K[3] = k.w;
  const int4 wd = *reinterpret_cast<const int4*>(A.rkw[x].W);
  rc.Wd[0] = wd.x; rc.Wd[1] = wd.y; rc.Wd[2] = wd.z;
  return rc;
}

// Flip decision of a cluster whose root has the chain-local segment index `key`, and its record
// contribution (from its class integers rcl), added into R.  Returns the flip.
__device__ __forceinline__ uint8_t root_record(const DChain& ch, uint32_t sweep, uint32_t key,
                                               const RootClass& rcl, RootSums& R) {
  const long long s0 = (long long)rcl.S[0], s1 = (long long)rcl.S[1], s2 = (long long)rcl.S[2],
                  s3 = (long long)rcl.S[3];
  const long long k0 = rcl.K[0], k1 = rcl.K[1], k2 = rcl.K[2], k3 = rcl.K[3];
  const long long Ms = s0 + s1 - s2 - s3, SMs = s0 - s1 - s2 + s3;
  const rnd4 r = philox(ch.seed, sweep, key, TAG_FLIP, 0);
  uint8_t f;
  if (!ch.field) {
    f = r.x < 0x80000000u ? 1 : 0;
  } else {
    const float xf = __fmul_rn(__ll2float_rn(Ms), ch.flip_coef);
    const float e = exp_clamped(xf);
    f = __fmul_rn(uniform_open(r.x), __fadd_rn(1.0f, e)) < 1.0f ? 1 : 0;
  }
  auto ab = [](long long v) { return (unsigned long long)(v < 0 ? -v : v); };
  {
    const long long n0 = k0 + k1 + k2 + k3, m0 = k0 + k1 - k2 - k3;
    const long long sn0 = k0 - k1 + k2 - k3, sm0 = k0 - k1 - k2 + k3;
    const unsigned long long m0sq = (unsigned long long)(m0 * m0), n0sq = (unsigned long long)(n0 * n0);
    const unsigned long long sm0sq = (unsigned long long)(sm0 * sm0), sn0sq = (unsigned long long)(sn0 * sn0);
    R.q[0] += 1ull;
    R.q[1] += (unsigned long long)m0;
    R.q[2] += (unsigned long long)sm0;
    R.q[3] += m0sq;
    R.q[4] += n0sq;
    R.q[5] += sm0sq;
    R.q[6] += sn0sq;
    add_u128(R.w[0], mul64(m0sq, m0sq));
    add_u128(R.w[1], mul64(n0sq, n0sq));
    add_u128(R.w[2], mul64(sm0sq, sm0sq));
    add_u128(R.w[3], mul64(sn0sq, sn0sq));
  }
  R.q[7] += (unsigned long long)(f ? -Ms : Ms);
  R.q[8] += (unsigned long long)Ms;
  R.q[9] += (unsigned long long)SMs;
  // winding (stiffness.h collector: sum over clusters of the squared winding per direction)
  R.q[10] += (unsigned long long)((long long)rcl.Wd[0] * rcl.Wd[0] + (long long)rcl.Wd[1] * rcl.Wd[1] +
                                  (long long)rcl.Wd[2] * rcl.Wd[2]);
  R.q[11] += (unsigned long long)(long long)rcl.Wd[0];
  R.q[12] += (unsigned long long)(long long)rcl.Wd[1];
  R.q[13] += (unsigned long long)(long long)rcl.Wd[2];
  const unsigned long long L = ab(s0 + s1 + s2 + s3), SL = ab(s0 - s1 + s2 - s3);
  add_u128(R.w[4], mul64(L, L));
  add_u128(R.w[5], mul64(ab(Ms), ab(Ms)));
  add_u128(R.w[6], mul64(SL, SL));
  add_u128(R.w[7], mul64(ab(SMs), ab(SMs)));
  return f;
}

// Flip decision of root x of chain c and its record contribution, added into R; clears the
// root's class sums.
__device__ __forceinline__ void root_sums(const Arena& A, int x, int c, const RootClass& rcl,
                                          RootSums& R) {
  ulonglong2* S = reinterpret_cast<ulonglong2*>(A.cls + 4 * (size_t)x);
  S[0] = make_ulonglong2(0ull, 0ull);
  S[1] = make_ulonglong2(0ull, 0ull);
  *reinterpret_cast<uint4*>(A.rkw[x].K) = make_uint4(0u, 0u, 0u, 0u);
  *reinterpret_cast<int4*>(A.rkw[x].W) = make_int4(0, 0, 0, 0);
  A.flip[x] = root_record(A.ch[c], A.ch_sweep[c], (uint32_t)(x - A.ch_slot_off[c]), rcl, R);
}

__device__ __forceinline__ void record_atomics(const Arena& A, int c, const RootSums& R) {
  unsigned long long* row = rec_row(A, c);
#pragma unroll
  for (int i = 0; i < NQ; ++i) if (R.q[i]) atomicAdd(row + kRecQ[i], R.q[i]);
#pragma unroll
  for (int i = 0; i < 8; ++i) if (R.w[i].lo | R.w[i].hi) atomic_add_u128(row + kRecW[i], R.w[i]);
}

// Sum of a u64 over the lanes of `grp` (16-bit limbs, exact).
__device__ __forceinline__ unsigned long long group_sum_u64(unsigned grp, unsigned long long v) {
  unsigned long long s = 0;
#pragma unroll
  for (int l = 0; l < 4; ++l)
    s += (unsigned long long)__reduce_add_sync(grp, (unsigned)((v >> (16 * l)) & 0xFFFFull)) << (16 * l);
  return s;
}

__device__ __forceinline__ u128 group_sum_u128(unsigned grp, u128 v) {
  u128 s = {0, 0};
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const unsigned long long w = l < 4 ? v.lo : v.hi;
    const unsigned long long t = __reduce_add_sync(grp, (unsigned)((w >> (16 * (l & 3))) & 0xFFFFull));
    const int sh = 16 * l;
    u128 add;
    add.lo = sh < 64 ? (t << sh) : 0ull;
    add.hi = sh == 0 ? 0ull : (sh < 64 ? (t >> (64 - sh)) : (t << (sh - 64)));
    add_u128(s, add);
  }
  return s;
}

// Adds every lane's root sums into its chain's record (c < 0: nothing).  Lanes of the same chain
// are reduced first, so that a chain takes one set of atomics per warp rather than per root.
// Warp-collective: every lane calls it.
__device__ __forceinline__ void record_by_chain(const Arena& A, int c, const RootSums& R) {
  const unsigned grp = __match_any_sync(0xFFFFFFFFu, c);
  if (c < 0) return;
  if (__popc(grp) == 1) { record_atomics(A, c, R); return; }
  const bool leader = (threadIdx.x & 31) == __ffs(grp) - 1;
  unsigned long long* row = rec_row(A, c);
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    const unsigned long long v = group_sum_u64(grp, R.q[i]);
    if (leader && v) atomicAdd(row + kRecQ[i], v);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const u128 v = group_sum_u128(grp, R.w[i]);
    if (leader && (v.lo | v.hi)) atomic_add_u128(row + kRecW[i], v);
  }
}

// Per cluster root: flip decision (path_integral.C:780-803) and the exact per-sweep sums of the
// improved estimator collector (susceptibility.h:182-198), cluster count (:774-778), field
// energy (:852-859) and the normal time-integrated magnetisations (susceptibility.h:283-297).
// Each block handles one tile of TILE consecutive segments.  A tile inside one chain is reduced
// in registers and shared memory (16-bit limbs, exact) and adds to the record once; a tile that
// spans chains reduces each warp's roots per chain (record_by_chain).
// A tile that spans chains.  A thread's roots come in segment order, so its chain never
// decreases: it sums its roots of one chain in registers and hands them to the per-chain warp
// reduction (record_by_chain) when its chain changes and at the end (every thread calls it on
// every step, with chain -1 when it has nothing to hand over).  Kept out of line so that its
// registers do not weigh on the single-chain path of k_cluster.
__device__ __noinline__ void cluster_spanning_tile(const Arena& A, const int* roots, int nr) {
  const int iters = (nr + (int)blockDim.x - 1) / (int)blockDim.x;
  int i = threadIdx.x;
  int x = i < nr ? roots[i] : 0;
  RootClass cur = i < nr ? load_root_class(A, x) : RootClass{};
  RootSums R;
#pragma unroll
  for (int k = 0; k < NQ; ++k) R.q[k] = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) R.w[k] = {0, 0};
  int cc = -1;
  for (int it = 0; it < iters; ++it) {
    const int inext = i + blockDim.x;
    const int xnext = inext < nr ? roots[inext] : 0;
    RootClass nxt = inext < nr ? load_root_class(A, xnext) : RootClass{};
    const int c = i < nr ? chain_of_segment(A, x) : -1;
    const bool hand = cc >= 0 && c >= 0 && c != cc;
    record_by_chain(A, hand ? cc : -1, R);
    if (hand) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) R.q[k] = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) R.w[k] = {0, 0};
    }
    if (i < nr) {
      root_sums(A, x, c, cur, R);
      cc = c;
    }
    i = inext;
    x = xnext;
    cur = nxt;
  }
  record_by_chain(A, cc, R);
}

constexpr int CL_TILE = 4096;
constexpr int CL_THREADS = 256;

template <int TILE = CL_TILE>
__global__ void __launch_bounds__(CL_THREADS) k_cluster(Arena A) {
  if (A.ctl->err) return;
  __shared__ unsigned limbs[CL_THREADS / 32][NLIMB];
  __shared__ unsigned long long tot[NLIMB];
  __shared__ int roots[TILE];
  __shared__ int nroots;
  const int ns = A.ctl->ns_total;
  const int ntiles = (ns + TILE - 1) / TILE;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int t0 = tile * TILE;
    const int t1 = min(t0 + TILE, ns);
    if (threadIdx.x == 0) nroots = 0;
    __syncthreads();
    // compact this tile's roots so that every lane works on one
    for (int b = t0 + wid * 32; b < t1; b += blockDim.x) {
      const int x = b + lane;
      const bool r = x < t1 && A.parent[x] == x;
      const unsigned ball = __ballot_sync(0xFFFFFFFFu, r);
      int base = 0;
      if (lane == 0 && ball) base = atomicAdd(&nroots, __popc(ball));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (r) roots[base + __popc(ball & ((1u << lane) - 1u))] = x;
    }
    __syncthreads();
    const int nr = nroots;
    const int cf = chain_of_segment(A, t0), cl = chain_of_segment(A, t1 - 1);
    if (cf != cl) {
      cluster_spanning_tile(A, roots, nr);
    } else {
      // software-pipelined: the next root's class sums are loaded while this one is processed
      int i = threadIdx.x;
      int x = i < nr ? roots[i] : 0;
      RootClass cur = i < nr ? load_root_class(A, x) : RootClass{};
      RootSums acc;
#pragma unroll
      for (int k = 0; k < NQ; ++k) acc.q[k] = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) acc.w[k] = {0, 0};
      while (i < nr) {
        const int inext = i + blockDim.x;
        const int xnext = inext < nr ? roots[inext] : 0;
        RootClass nxt = inext < nr ? load_root_class(A, xnext) : RootClass{};
        root_sums(A, x, cf, cur, acc);
        i = inext;
        x = xnext;
        cur = nxt;
      }
#pragma unroll
      for (int i = 0; i < NQ; ++i)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          const unsigned v = __reduce_add_sync(0xFFFFFFFFu, (unsigned)((acc.q[i] >> (16 * l)) & 0xFFFFull));
          if (lane == 0) limbs[wid][4 * i + l] = v;
        }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const unsigned long long wv = l < 4 ? acc.w[i].lo : acc.w[i].hi;
          const unsigned v = __reduce_add_sync(0xFFFFFFFFu, (unsigned)((wv >> (16 * (l & 3))) & 0xFFFFull));
          if (lane == 0) limbs[wid][QLIMB + 8 * i + l] = v;
        }
      __syncthreads();
      for (int j = threadIdx.x; j < NLIMB; j += blockDim.x) {
        unsigned long long sum = 0;
        for (int w = 0; w < CL_THREADS / 32; ++w) sum += limbs[w][j];
        tot[j] = sum;
      }
      __syncthreads();
      if (threadIdx.x < NQ + 8) {
        unsigned long long* row = rec_row(A, cf);
        const int i = threadIdx.x;
        if (i < NQ) {
          unsigned long long v = 0;
          for (int l = 0; l < 4; ++l) v += tot[4 * i + l] << (16 * l);
          if (v) atomicAdd(row + kRecQ[i], v);
        } else {
          const int k = i - NQ;
          u128 v = {0, 0};
          for (int l = 0; l < 8; ++l) {
            const unsigned long long t = tot[QLIMB + 8 * k + l];
            const int sh = 16 * l;
            u128 add;
            add.lo = sh < 64 ? (t << sh) : 0ull;
            add.hi = sh == 0 ? 0ull : (sh < 64 ? (t >> (64 - sh)) : (t << (sh - 64)));
            add_u128(v, add);
          }
          if (v.lo | v.hi) atomic_add_u128(row + kRecW[k], v);
        }
      }
    }
    __syncthreads();
  }
}

// Root of segment x (after k_accumulate every parent is a root).
__device__ __forceinline__ int seg_root(const int* P, int x) { return P[x]; }

// Per site (one warp each): flip the tau = 0 spin with its bottom segment's cluster
// (path_integral.C:822-823) and keep, in time order and in place at the start of the site's
// segment range, the endpoints whose vertex is off-diagonal after the flips: the next sweep's
// off-diagonal list.  A vertex changes type when its two clusters flip differently
// (path_integral.C:815-818, loop0 / loop1 of graph_impl.h:489-494), and at either endpoint those
// are the clusters of the segments below and above it: g = 0 joins the two lower legs and the
// two upper legs, g = 1 crosses them, and a frozen graph has all four legs in one cluster.  So
// the new type at endpoint x is its old type ^ flip(cluster of x-1) ^ flip(cluster of x), the
// same at both of its sites.  Every lane reads its step's segments before any lane writes, and a kept
// endpoint never moves forward, so the in-place compaction reads no overwritten slot.
__global__ void __launch_bounds__(256) k_site_end(Arena A, const int* sites, int nsites) {
  if (A.ctl->err) return;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; si < nsites; si += warps) {
    const int s = sites ? sites[si] : si;
    const int base = A.sbase[s];
    const int k = A.sbase[s + 1] - base - 1;
    const uint8_t fb = A.flip[seg_root(A.parent, base)];
    if (lane == 0 && fb) A.spin0[s] ^= 1u;
    uint8_t below = fb;   // flip of the cluster under the step's first segment
    int n = 0;
    // 64 segments per step (two per lane), every load of the step issued before any use
    for (int j0 = 1; j0 <= k; j0 += 64) {
      const int ja = j0 + lane, jb = ja + 32;
      uint8_t ia = 0, ib = 0, fa = 0, fbb = 0;
      int pa = 0, pb = 0;
      if (ja <= k) { ia = A.sinfo[base + ja]; pa = A.parent[base + ja]; }
      if (jb <= k) { ib = A.sinfo[base + jb]; pb = A.parent[base + jb]; }
      if (ja <= k) fa = A.flip[pa];
      if (jb <= k) fbb = A.flip[pb];
      uint8_t prev_a = (uint8_t)__shfl_up_sync(0xFFFFFFFFu, (unsigned)fa, 1);
      uint8_t prev_b = (uint8_t)__shfl_up_sync(0xFFFFFFFFu, (unsigned)fbb, 1);
      const uint8_t top_a = (uint8_t)__shfl_sync(0xFFFFFFFFu, (unsigned)fa, 31);
      if (lane == 0) { prev_a = below; prev_b = top_a; }
      below = (uint8_t)__shfl_sync(0xFFFFFFFFu, (unsigned)fbb, 31);
      const bool ka = ja <= k && ((((ia & SI_OFF) ? 1u : 0u) ^ prev_a ^ fa) != 0);
      const bool kb = jb <= k && ((((ib & SI_OFF) ? 1u : 0u) ^ prev_b ^ fbb) != 0);
      uint64_t ta = 0, tb = 0;
      uint8_t da = 0, db = 0;
      if (ka) { ta = A.stime[base + ja]; da = A.sdir[base + ja] & SD_IMASK; }  // the list keeps
      if (kb) { tb = A.stime[base + jb]; db = A.sdir[base + jb] & SD_IMASK; }  // the incidence
      const unsigned balla = __ballot_sync(0xFFFFFFFFu, ka);
      const unsigned ballb = __ballot_sync(0xFFFFFFFFu, kb);
      __syncwarp();
      const unsigned lt = (1u << lane) - 1u;
      if (ka) {
        const int pos = n + __popc(balla & lt);
        A.stime[base + pos] = ta;
        A.sdir[base + pos] = da;
      }
      n += __popc(balla);
      if (kb) {
        const int pos = n + __popc(ballb & lt);
        A.stime[base + pos] = tb;
        A.sdir[base + pos] = db;
      }
      n += __popc(ballb);
      __syncwarp();
    }
    if (lane == 0) { A.off_base[s] = base; A.off_cnt[s] = n; }
  }
}

// Thread-per-site form of k_site_end for sites with few endpoints (kept entries never move
// forward, so the in-place compaction reads no overwritten slot).
__global__ void __launch_bounds__(256) k_site_end_narrow(Arena A, const int* sites, int nsites) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(i, nsites) {
    const int s = sites[i];
    const int base = A.sbase[s];
    const int k = A.sbase[s + 1] - base - 1;
    uint8_t fprev = A.flip[seg_root(A.parent, base)];
    if (fprev) A.spin0[s] ^= 1u;
    int n = 0;
    for (int j = 1; j <= k; ++j) {
      const int x = base + j;
      const uint8_t fx = A.flip[seg_root(A.parent, x)];
      if ((((A.sinfo[x] & SI_OFF) ? 1u : 0u) ^ fprev ^ fx) != 0) {
        A.stime[base + n] = A.stime[x];
        A.sdir[base + n] = A.sdir[x] & SD_IMASK;  // the list keeps the incidence index
        ++n;
      }
      fprev = fx;
    }
    A.off_base[s] = base;
    A.off_cnt[s] = n;
  }
}

// Spin correlations from the tau = 0 spins after the flips (the normal estimator of
// correlation.h:222-266, which reads `spins` at commit time).  One block per tile of
// CORR_THREADS entries of one chain; the chain's spins are staged in shared memory (up to
// CORR_SMEM sites; larger chains read them from global memory).  Entry r of the all-pairs sums
// is sum_i m_i m_{i+r} over every site i, i + r taken with periodic wrap per dimension and
// m = 1 - 2 s, an exact integer; with an origin o, entry j adds m_o m_j.  Only sweeps in the
// chain's measurement window [corr_from, corr_to) are added.
constexpr int CORR_THREADS = 256;
constexpr int CORR_SMEM = 64 * 1024;

__global__ void __launch_bounds__(CORR_THREADS) k_corr(Arena A) {
  if (A.ctl->err) return;
  extern __shared__ uint8_t corr_sp[];
  const int2 tl = A.corr_tiles[blockIdx.x];
  const int c = tl.x;
  const DChain ch = A.ch[c];
  const uint32_t sw = A.ch_sweep[c];
  if (sw < ch.corr_from || sw >= ch.corr_to) return;
  const int N = ch.nsites, so = ch.site_off, L = ch.L;
  const uint8_t* sp = A.spin0 + so;
  if (N <= CORR_SMEM) {
    for (int i = threadIdx.x; i < N; i += CORR_THREADS) corr_sp[i] = A.spin0[so + i];
    __syncthreads();
    sp = corr_sp;
  }
  const int r = tl.y + threadIdx.x;
  if (r >= N) return;
  if (ch.corr_origin >= 0)
    A.corr_origin[so + r] += (sp[ch.corr_origin] == sp[r]) ? 1 : -1;
  if (!ch.corr_disp) return;
  const int rx = r % L, ry = ch.dim > 1 ? (r / L) % L : 0, rz = ch.dim > 2 ? r / (L * L) : 0;
  const int Ly = ch.dim > 1 ? L : 1, Lz = ch.dim > 2 ? L : 1;
  int sum = 0;
  for (int z = 0; z < Lz; ++z) {
    const int jz = z + rz < Lz ? z + rz : z + rz - Lz;
    for (int y = 0; y < Ly; ++y) {
      const int jy = y + ry < Ly ? y + ry : y + ry - Ly;
      const uint8_t* row = sp + (z * Ly + y) * L;
      const uint8_t* jrow = sp + (jz * Ly + jy) * L;
      int x = 0;
      for (; x + rx < L; ++x) sum += row[x] == jrow[x + rx] ? 1 : -1;
      for (; x < L; ++x) sum += row[x] == jrow[x + rx - L] ? 1 : -1;
    }
  }
  A.corr_disp[so + r] += sum;
}

// One block: per chain the operator count and the sweep counter; then the next sweep's record
// row (if the chunk has one) and the region claim counters are cleared, and the record row
// counter advances.
__global__ void __launch_bounds__(1024) k_end(Arena A) {
  if (A.ctl->err) return;
  const uint32_t step = A.ctl->step;
  for (int c = threadIdx.x; c < A.C; c += blockDim.x) {
    // every vertex adds one segment at each of its two sites
    const int nv = (A.ch_slot_off[c + 1] - A.ch_slot_off[c] - A.ch[c].nsites) / 2;
    rec_row(A, c)[R_NOP] = (unsigned long long)nv;
    A.ch_sweep[c] += 1u;
  }
  if ((int)step + 1 < A.rec_rows)
    for (int i = threadIdx.x; i < A.C * REC_WORDS; i += blockDim.x)
      A.rec[((size_t)step + 1) * A.C * REC_WORDS + i] = 0ull;
  for (int r = threadIdx.x; r < A.R; r += blockDim.x) A.region_fill[r] = 0ull;
  __syncthreads();
  if (threadIdx.x == 0) A.ctl->step = step + 1u;
}

// Structural invariants after a stage of a sweep (the test seam lg_validate_sweeps; never on the
// hot path).  Every index the sweep kernels dereference comes from these structures: the bonds'
// vertex ranges, the site segment offsets, the vertex <-> segment links, the union-find forest
// and the off-diagonal lists.  Each index is range-checked here before it is used.  A failed
// check counts in bad[0]; the first failure's code (stage * 10 + check) is kept in bad[1].
__device__ __forceinline__ void val_fail(int* bad, int code) {
  atomicAdd(bad, 1);
  atomicCAS(bad + 1, 0, code);
}

__global__ void __launch_bounds__(256) k_validate(Arena A, int stage, int* bad) {
  if (A.ctl->err) return;
  const int nv_cap = A.ctl->nv_cap, ns_cap = A.ctl->ns_cap, ns = A.ctl->ns_total;
  if (stage == 0) {  // after insertion: each bond's vertices inside its region, time ordered
    LG_GRID_STRIDE(b, A.NB) {
      const int n = A.bond_cnt[b];
      if (n < 0) { val_fail(bad, 1); continue; }
      if (n == 0) continue;
      const int p = A.bond_ptr[b];
      const int r = A.site_region[A.bond_s0[b]];
      if (r < 0 || r >= A.R) { val_fail(bad, 2); continue; }
      if (p < A.region_base[r] || p + n > A.region_base[r + 1] || A.region_base[r + 1] > nv_cap) {
        val_fail(bad, 3);
        continue;
      }
      uint64_t prev = 0;
      for (int i = p; i < p + n; ++i) {
        const uint64_t t = A.vtime[i];
        if (t >= 0x3FF0000000000000ull || t < prev) { val_fail(bad, 4); break; }  // [0,1), ordered
        if (A.vcode[i] > 7) { val_fail(bad, 5); break; }
        prev = t;
      }
    }
  } else if (stage == 2) {  // after the merge: segment ranges, vertex links, forest pointers
    if (blockIdx.x == 0 && threadIdx.x == 0 && (ns > ns_cap || ns < A.N)) val_fail(bad, 21);
    LG_GRID_STRIDE(s, A.N) {
      const int base = A.sbase[s], end = A.sbase[s + 1];
      if (base < 0 || end <= base || end > ns) { val_fail(bad, 22); continue; }
      int deg = 0;
      for (int j = A.inc_off[s]; j < A.inc_off[s + 1]; ++j) deg += A.bond_cnt[A.inc[j]];
      if (end - base != deg + 1) { val_fail(bad, 23); continue; }
      if (A.stime[base] != 0ull) val_fail(bad, 24);
      for (int x = base; x < end; ++x) {
        if (x > base && A.stime[x] < A.stime[x - 1]) { val_fail(bad, 25); break; }
        const int p = A.parent[x];
        if (p < 0 || p > x) { val_fail(bad, 26); break; }  // hooks go to smaller indices
        if (x == base) continue;
        const int v = A.svert[x];
        if (v < 0 || v >= nv_cap) { val_fail(bad, 27); break; }
        const int side = (A.sinfo[x] & SI_SRC) ? 0 : 1;
        if (A.vslot[2 * v + side] != x) { val_fail(bad, 28); break; }
      }
    }
  } else if (stage == 4) {  // after the cluster sums: every parent is a root
    LG_GRID_STRIDE(x, ns) {
      const int r = A.parent[x];
      if (r < 0 || r > x) { val_fail(bad, 41); continue; }
      if (A.parent[r] != r) val_fail(bad, 42);
    }
  } else if (stage == 6) {  // after the sweep: the next sweep's off-diagonal lists
    LG_GRID_STRIDE(s, A.N) {
      const int b0 = A.off_base[s], n = A.off_cnt[s];
      const int k = A.sbase[s + 1] - A.sbase[s] - 1;
      if (b0 != A.sbase[s] || n < 0 || n > k) { val_fail(bad, 61); continue; }
      const int z = A.inc_off[s + 1] - A.inc_off[s];
      for (int i = 0; i < n; ++i) {
        if (A.sdir[b0 + i] >= z) { val_fail(bad, 62); break; }
        if (i > 0 && A.stime[b0 + i] < A.stime[b0 + i - 1]) { val_fail(bad, 63); break; }
      }
      // a spin-1/2 site's spin is periodic in imaginary time: an even number of flips
      if ((n & 1) && A.ch[A.site_chain[s]].spin2 <= 1) val_fail(bad, 64);
    }
  }
}

// Moving chains into a new arena: site s of the new arena takes the state of site map[s] of
// the old one (map[s] < 0: a new chain, left as initialised).  Pass 1 gathers list lengths.
__global__ void k_repack_count(Arena A, const int* map, const int* old_off_cnt, int* cnt) {
  LG_GRID_STRIDE(s, A.N) cnt[s] = map[s] >= 0 ? old_off_cnt[map[s]] : 0;
}

// Pass 2 (one warp per site): copy the spin and the off-diagonal list to its new place.
__global__ void k_repack_copy(Arena A, const int* map, const uint8_t* old_spin0,
                              const int* old_off_base, const uint64_t* old_stime,
                              const uint8_t* old_sdir, const int* new_base) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < A.N; s += warps) {
    const int o = map[s];
    if (o < 0) continue;
    const int n = A.off_cnt[s], src = old_off_base[o], dst = new_base[s];
    for (int i = lane; i < n; i += 32) {
      A.stime[dst + i] = old_stime[src + i];
      A.sdir[dst + i] = old_sdir[src + i];
    }
    if (lane == 0) { A.spin0[s] = old_spin0[o]; A.off_base[s] = dst; }
  }
}

// Initial spins: all up, or iid from the chain's seed.
__global__ void k_init_spins(Arena A, int random) {
  LG_GRID_STRIDE(s, A.N) {
    const int c = A.site_chain[s];
    const DChain ch = A.ch[c];
    uint8_t v = 0;
    if (random) v = (uint8_t)(philox(ch.seed, 0xFFFFFFFFu, (uint32_t)(s - ch.site_off), TAG_SPIN, 0).x & 1u);
    A.spin0[s] = v;
    A.off_cnt[s] = 0;
    A.off_base[s] = 0;
  }
}

}  // namespace lg
