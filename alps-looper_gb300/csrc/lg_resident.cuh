// Chain-resident sweeps: one CTA runs whole sweeps of one chain with all of its per-sweep data in
// shared memory (path_integral.C:355-864), many sweeps per launch.
//
// For chains small enough that a sweep's vertices, segments and union-find forest fit in one
// CTA's shared memory (e.g. the 64-site chain at beta = 10: ~440 operators, ~950 segments), the
// nine grid-wide launches of the arena sweep cost far more than the work: every launch waits for
// the previous one, and a small chain fills a tiny fraction of the GPU.  Here a CTA owns a chain
// for the whole launch, the phases of a sweep are separated by __syncthreads instead of kernel
// boundaries, the union-find runs on shared-memory atomics, and an arena of many such chains fills
// the GPU with one persistent launch (CTAs stride over the chains).
//
// The sweep is the same computation as the grid path, step for step, so that every trajectory and
// every record is bit-identical between the two:
//   insertion      per bond, the serial three-way walk of insert_bond_serial (same Philox keys)
//   segments       per site, the serial z-way merge of merge_site_serial (same numbering: site-major,
//                  bottom segment first, chain-local segment index = the grid path's index minus
//                  the chain's first slot)
//   union-find     the same hooks (larger root index -> smaller), so the roots are the same
//   class sums     seg_contrib per segment, summed per root in global memory (exact integers)
//   flips, sums    root_record per root (the cluster coin keyed by the root's chain-local index)
//   end            the flip / compaction rule of k_site_end_narrow, and the record row
//
// Persistent state moves between launches in double-buffered global arrays: a launch reads the
// spins and off-diagonal lists from the `in` set and writes them to the `out` set, so that a launch
// that fails (a chain outgrowing its shared-memory capacity, an exhausted union retry budget)
// leaves the state it started from untouched and the host can replay it elsewhere.
#pragma once
#include "lg_kernels.cuh"

namespace lg {

constexpr int RES_THREADS = 256;

// Shared-memory layout of one chain's sweep for at most n sites, nb bonds and v vertices
// (s = n + 2 v segments).  Offsets in bytes from the start of the dynamic shared memory.
struct ResLayout {
  int n, nb, v, s;
  unsigned o_st, o_vt, o_tot, o_par, o_sv, o_vslot, o_sbase, o_obase, o_ocnt, o_bcnt, o_bptr,
      o_limb, o_si, o_sd, o_flip, o_vc, o_spin, bytes;
};

__host__ __device__ inline unsigned res_take(unsigned& o, unsigned bytes) {
  o = (o + 15u) & ~15u;
  const unsigned r = o;
  o += bytes;
  return r;
}

__host__ __device__ inline ResLayout res_layout(int n, int nb, int v) {
  ResLayout L;
  L.n = n; L.nb = nb; L.v = v; L.s = n + 2 * v;
  unsigned o = 0;
  L.o_st = res_take(o, 8u * L.s);                               // segment start times
  L.o_vt = res_take(o, 8u * v);                                 // vertex times
  L.o_tot = res_take(o, 8u * (NLIMB + REC_WORDS));              // record reduction
  L.o_par = res_take(o, 4u * L.s);                              // union-find forest
  L.o_sv = res_take(o, 4u * L.s);                               // vertex of each segment
  L.o_vslot = res_take(o, 8u * v);                              // start segments of each vertex
  L.o_sbase = res_take(o, 4u * (n + 1));                        // segment offsets per site
  L.o_obase = res_take(o, 4u * n);                              // off-diagonal list per site
  L.o_ocnt = res_take(o, 4u * n);
  L.o_bcnt = res_take(o, 4u * nb);                              // vertex range per bond
  L.o_bptr = res_take(o, 4u * (nb + 1));
  L.o_limb = res_take(o, 4u * (RES_THREADS / 32) * NLIMB);      // per-warp limb sums
  L.o_si = res_take(o, (unsigned)L.s);                          // segment info
  L.o_sd = res_take(o, (unsigned)L.s);                          // incidence | direction << 5
  L.o_flip = res_take(o, (unsigned)L.s);                        // flip of each root
  L.o_vc = res_take(o, (unsigned)v);                            // vertex code
  L.o_spin = res_take(o, (unsigned)n);                          // spins at tau = 0
  L.bytes = (o + 15u) & ~15u;
  return L;
}

// Parameters of one launch.
struct ResArgs {
  int m;                        // sweeps per chain in this launch (record rows 0..m-1)
  int nmax, nbmax, vcap;        // the shared-memory layout's capacities
  int lcap;                     // off-diagonal list entries per chain in the out arrays
  int scap;                     // class-sum slots per chain in A.cls / A.rkw
  const uint8_t* spin_in;       // persistent state the launch starts from (arena site indexed)
  const int* obase_in;
  const int* ocnt_in;
  const uint64_t* st_in;
  const uint8_t* sd_in;
  uint8_t* spin_out;            // and where it leaves it (chain c's lists at c * lcap)
  int* obase_out;
  int* ocnt_out;
  uint64_t* st_out;
  uint8_t* sd_out;
};

// Pointers into the dynamic shared memory.
struct ResSmem {
  uint64_t* st; uint64_t* vt; unsigned long long* tot;
  int* par; int* sv; int* vslot; int* sbase; int* obase; int* ocnt; int* bcnt; int* bptr;
  unsigned* limb;
  uint8_t* si; uint8_t* sd; uint8_t* flip; uint8_t* vc; uint8_t* spin;
};

__device__ __forceinline__ ResSmem res_smem(unsigned char* b, const ResLayout& L) {
  ResSmem m;
  m.st = reinterpret_cast<uint64_t*>(b + L.o_st);
  m.vt = reinterpret_cast<uint64_t*>(b + L.o_vt);
  m.tot = reinterpret_cast<unsigned long long*>(b + L.o_tot);
  m.par = reinterpret_cast<int*>(b + L.o_par);
  m.sv = reinterpret_cast<int*>(b + L.o_sv);
  m.vslot = reinterpret_cast<int*>(b + L.o_vslot);
  m.sbase = reinterpret_cast<int*>(b + L.o_sbase);
  m.obase = reinterpret_cast<int*>(b + L.o_obase);
  m.ocnt = reinterpret_cast<int*>(b + L.o_ocnt);
  m.bcnt = reinterpret_cast<int*>(b + L.o_bcnt);
  m.bptr = reinterpret_cast<int*>(b + L.o_bptr);
  m.limb = reinterpret_cast<unsigned*>(b + L.o_limb);
  m.si = b + L.o_si;
  m.sd = b + L.o_sd;
  m.flip = b + L.o_flip;
  m.vc = b + L.o_vc;
  m.spin = b + L.o_spin;
  return m;
}

// Exclusive scan of a[0, n) into out (may alias a) by the whole block; returns the total.
__device__ __forceinline__ int res_scan(const int* a, int n, int* out, int* sw) {
  int carry = 0;
  for (int base = 0; base < n; base += RES_THREADS) {
    const int i = base + (int)threadIdx.x;
    const int v = i < n ? a[i] : 0;
    int tot;
    const int ex = block_exclusive_scan(v, sw, &tot);
    if (i < n) out[i] = carry + ex;
    carry += tot;
  }
  return carry;
}

// insert_bond_serial on the shared-memory state of one chain: bond bl (chain-local) of chain ch
// at sweep `sweep`.  Returns the vertex count; with WRITE the time-ordered list is stored from
// vertex out0 on.
template <bool WRITE>
__device__ int res_insert_bond(const Arena& A, const ResSmem& M, const DChain& ch, uint32_t sweep,
                               int bl, int out0) {
  const int b = ch.bond_off + bl;
  const int s0 = A.bond_s0[b] - ch.site_off, s1 = A.bond_s1[b] - ch.site_off;
  const uint8_t own = A.bond_dir0[b];
  uint32_t p0 = M.spin[s0], p1 = M.spin[s1];
  int i0 = M.obase[s0], e0 = i0 + M.ocnt[s0];
  int i1 = M.obase[s1], e1 = i1 + M.ocnt[s1];
  uint64_t t0 = i0 < e0 ? M.st[i0] : TIME_INF;
  uint64_t t1 = i1 < e1 ? M.st[i1] : TIME_INF;
  uint64_t tq = 0, tp = TIME_INF;
  uint32_t k = 0, gp = 0;
  rnd4 r = {0, 0, 0, 0};
  bool more = ch.inv_rate > 0.0f;
  auto next_prop = [&]() {
    tp = TIME_INF;
    if (!more) return;
    if ((k & 1u) == 0) r = philox(ch.seed, sweep, (uint32_t)bl, TAG_PROPOSAL, k >> 1);
    const uint32_t wu = (k & 1u) ? r.z : r.x;
    const uint32_t wg = (k & 1u) ? r.w : r.y;
    ++k;
    const uint32_t tail = (wu >> 9) ? 0u : gap_tail_word(ch.seed, sweep, (uint32_t)bl, k - 1);
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
      if (M.sd[i0] == own) {
        if (WRITE) {
          if ((ordinal & 3u) == 0) ro = philox(ch.seed, sweep, (uint32_t)bl, TAG_OFFDIAG, ordinal >> 2);
          const uint32_t w = (ordinal & 3u) == 0 ? ro.x : (ordinal & 3u) == 1 ? ro.y
                           : (ordinal & 3u) == 2 ? ro.z : ro.w;
          const uint32_t g = ((uint64_t)w < ch.Poff) ? 0u : 1u;
          M.vt[out] = t0;
          M.vc[out] = (uint8_t)((g << 1) | 1u);
        }
        ++ordinal;
        ++out;
      }
      ++i0;
      t0 = i0 < e0 ? M.st[i0] : TIME_INF;
    } else if (t1 <= tp) {
      p1 ^= 1u;
      ++i1;
      t1 = i1 < e1 ? M.st[i1] : TIME_INF;
    } else {
      if (((gp & 1u) ^ p0 ^ p1) & 1u) {
        if (WRITE) {
          M.vt[out] = tp;
          M.vc[out] = (uint8_t)(gp << 1);
        }
        ++out;
      }
      next_prop();
    }
  }
  return out - out0;
}

// merge_site_serial on the shared-memory state: the segments of chain-local site i.
template <int Z>
__device__ void res_merge_site(const Arena& A, const ResSmem& M, const DChain& ch, int i) {
  const int gs = ch.site_off + i;
  const int j0 = A.inc_off[gs];
  const int z = A.inc_off[gs + 1] - j0;
  const int base = M.sbase[i];
  const int k = M.sbase[i + 1] - base - 1;
  const uint8_t gneg = A.gauge[gs] < 0 ? SI_GNEG : 0;
  int cur[Z], end[Z];
  uint64_t ht[Z];
  uint8_t hc[Z], side[Z], dirb[Z];
#pragma unroll
  for (int d = 0; d < Z; ++d) {
    if (d < z) {
      const int bl = A.inc[j0 + d] - ch.bond_off;
      cur[d] = M.bptr[bl];
      end[d] = cur[d] + M.bcnt[bl];
      side[d] = A.inc_side[j0 + d];
      dirb[d] = (uint8_t)(d | (A.inc_dir ? A.inc_dir[j0 + d] << SD_DSHIFT : 0));
      ht[d] = cur[d] < end[d] ? M.vt[cur[d]] : TIME_INF;
      hc[d] = cur[d] < end[d] ? M.vc[cur[d]] : 0;
    } else {
      cur[d] = end[d] = 0; ht[d] = TIME_INF; hc[d] = 0; side[d] = 0; dirb[d] = 0;
    }
  }
  uint8_t spin = M.spin[i];
  M.st[base] = 0ull;
  M.si[base] = (uint8_t)(spin | gneg | SI_FIRST | (k == 0 ? SI_LAST : 0));
  M.sv[base] = -1;
  M.sd[base] = 0xFF;
  M.par[base] = base;
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
    uint8_t sd = 0, code = 0, db = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) {
      if (d == best) {
        v = cur[d]; sd = side[d]; code = hc[d]; db = dirb[d];
        ++cur[d];
        ht[d] = cur[d] < end[d] ? M.vt[cur[d]] : TIME_INF;
        hc[d] = cur[d] < end[d] ? M.vc[cur[d]] : 0;
      }
    }
    if (code & 1u) spin ^= 1u;
    M.st[x] = bt;
    M.si[x] = (uint8_t)(spin | gneg | (j == k ? SI_LAST : 0) | (sd == 0 ? SI_SRC : 0) |
                        ((code >> 1) << SI_GSHIFT) | ((code & 1u) ? SI_OFF : 0));
    M.sv[x] = v;
    M.sd[x] = db;
    M.par[x] = x;
    M.vslot[2 * v + sd] = x;
  }
  if (k > 0) M.par[base + k] = base;  // temporal closure (path_integral.C:584-589)
}

// Union-find on the shared-memory forest: the hooks of uf_union (larger root -> smaller index),
// with path halving; loads are volatile because other threads hook and halve concurrently.
__device__ __forceinline__ int res_find(int* P, int x) {
  volatile int* V = P;
  int p = V[x];
  while (p != x) {
    const int g = V[p];
    if (g == p) return p;
    V[x] = g;
    x = g;
    p = V[x];
  }
  return x;
}

__device__ __forceinline__ bool res_union(int* P, int a, int b, int cap) {
  for (int it = 0; it < cap; ++it) {
    a = res_find(P, a);
    b = res_find(P, b);
    if (a == b) return true;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int old = atomicCAS(P + hi, hi, lo);
    if (old == hi) return true;
    a = lo;
    b = old;
  }
  return false;
}

// The whole chunk of R.m sweeps of every chain of the arena, chains strided over the CTAs.
// Z: the arena's largest site degree (2, 4 or MAXZ), as for the merge kernels.  Registers are
// capped at 64 so that four CTAs share an SM: a lone chain's sweep gets 17% slower (86 against
// 74 us on a 64-site chain at beta = 10, some spills), but an arena of 1024 such chains runs 1.47x
// faster (0.210 against 0.309 ms per sweep), 4096 of them 1.50x.
template <int Z>
__global__ void __launch_bounds__(RES_THREADS, 4) k_resident(Arena A, ResArgs R) {
  if (A.ctl->err) return;
  extern __shared__ __align__(16) unsigned char res_buf[];
  __shared__ int sw[32];
  __shared__ int fail;
  const ResLayout Ly = res_layout(R.nmax, R.nbmax, R.vcap);
  const ResSmem M = res_smem(res_buf, Ly);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int cap = iter_cap_of(A.ctl);
  for (int c = blockIdx.x; c < A.C; c += gridDim.x) {
    if (!A.all_active && !A.ch_active[c]) continue;  // a retired chain: its state is dropped
    const DChain ch = A.ch[c];
    const int N = ch.nsites, NB = ch.nbonds, so = ch.site_off;
    const size_t sbase_g = (size_t)c * R.scap;   // this chain's class-sum slots
    uint32_t sweep = A.ch_sweep[c];
    if (tid == 0) fail = 0;
    // ---- load the persistent state: spins and the off-diagonal lists, packed
    for (int i = tid; i < N; i += RES_THREADS) {
      M.spin[i] = R.spin_in[so + i];
      M.ocnt[i] = R.ocnt_in[so + i];
    }
    __syncthreads();
    const int ltot = res_scan(M.ocnt, N, M.obase, sw);
    if (ltot > Ly.s) {
      if (tid == 0) atomicExch(&A.ctl->err, ERR_OVERFLOW);
      return;
    }
    for (int i = tid; i < N; i += RES_THREADS) {
      const int src = R.obase_in[so + i], dst = M.obase[i], n = M.ocnt[i];
      for (int j = 0; j < n; ++j) { M.st[dst + j] = R.st_in[src + j]; M.sd[dst + j] = R.sd_in[src + j]; }
    }
    __syncthreads();
    for (int step = 0; step < R.m; ++step, ++sweep) {
      // ---- insertion (path_integral.C:403-577): count, place, write
      for (int b = tid; b < NB; b += RES_THREADS) M.bcnt[b] = res_insert_bond<false>(A, M, ch, sweep, b, 0);
      __syncthreads();
      const int nv = res_scan(M.bcnt, NB, M.bptr, sw);
      if (nv > Ly.v) {  // uniform: every thread sees the same total
        if (tid == 0) atomicExch(&A.ctl->err, ERR_OVERFLOW);
        return;
      }
      if (tid == 0) M.bptr[NB] = nv;
      for (int b = tid; b < NB; b += RES_THREADS) res_insert_bond<true>(A, M, ch, sweep, b, M.bptr[b]);
      __syncthreads();
      // ---- segments: 1 + incident vertices per site, then the per-site merge
      for (int i = tid; i < N; i += RES_THREADS) {
        int kk = 1;
        for (int j = A.inc_off[so + i]; j < A.inc_off[so + i + 1]; ++j) kk += M.bcnt[A.inc[j] - ch.bond_off];
        M.sbase[i] = kk;
      }
      __syncthreads();
      const int S = res_scan(M.sbase, N, M.sbase, sw);
      if (tid == 0) M.sbase[N] = S;
      __syncthreads();
      for (int i = tid; i < N; i += RES_THREADS) res_merge_site<Z>(A, M, ch, i);
      __syncthreads();
      // ---- reconnect + unify (graph_impl.h:280-295): the legs of every vertex
      bool ok = true;
      for (int x = tid; x < S; x += RES_THREADS) {
        const uint8_t info = M.si[x];
        if (!(info & SI_SRC)) continue;
        const int a = x, b = M.vslot[2 * M.sv[x] + 1], g = (info >> SI_GSHIFT) & 3;
        if (g == 1) {
          ok &= res_union(M.par, a - 1, b, cap);
          ok &= res_union(M.par, b - 1, a, cap);
        } else {
          ok &= res_union(M.par, a - 1, b - 1, cap);
          ok &= res_union(M.par, a, b, cap);
          if (g & 2) ok &= res_union(M.par, a - 1, a, cap);
        }
      }
      if (!ok) fail = 1;
      __syncthreads();
      if (fail) {
        if (tid == 0) atomicExch(&A.ctl->err, ERR_ITERCAP);
        return;
      }
      // ---- roots and class sums (path_integral.C:650-737): exact integers per root, in the
      // chain's global slots; lanes adding to the same (root, class) are summed first
      for (int x0 = 0; x0 < S; x0 += RES_THREADS) {
        const int x = x0 + tid;
        const bool in = x < S;
        int r = x;
        SegContrib sc = {0ull, 0, {0, 0, 0}};
        uint8_t info = 0;
        if (in) {
          // a read-only walk: this phase's only stores are final roots, so every parent a walk
          // reads is an ancestor (path halving here could leave a non-root parent behind)
          volatile int* V = M.par;
          int p = V[x];
          while (p != r) { r = p; p = V[r]; }
          M.par[x] = r;
          info = M.si[x];
          const bool last = info & SI_LAST;
          sc = seg_contrib(info, last ? 0 : M.si[x + 1], M.st[x], last ? 0ull : M.st[x + 1], M.sd[x],
                           last ? 0 : M.sd[x + 1]);
        }
        const unsigned grp = __match_any_sync(0xFFFFFFFFu, in ? r * 4 + sc.q : -1 - lane);
        const unsigned long long len = group_sum_u64(grp, sc.len);
        const bool leader = lane == __ffs(grp) - 1;
        const size_t slot = sbase_g + (size_t)r;
        if (in && leader && len) atomicAdd(A.cls + 4 * slot + sc.q, len);
        if (in && (info & SI_FIRST)) atomicAdd(&A.rkw[slot].K[sc.q], 1u);
#pragma unroll
        for (int d = 0; d < 3; ++d)
          if (in && sc.w[d]) atomicAdd(&A.rkw[slot].W[d], sc.w[d]);
      }
      __syncthreads();
      // ---- per cluster: flip (path_integral.C:780-803) and the record sums
      RootSums acc;
#pragma unroll
      for (int k = 0; k < NQ; ++k) acc.q[k] = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) acc.w[k] = {0, 0};
      for (int x = tid; x < S; x += RES_THREADS) {
        if (M.par[x] != x) continue;
        const size_t slot = sbase_g + (size_t)x;
        unsigned long long* cl = A.cls + 4 * slot;
        RootClass rc;
        const ulonglong2 a = __ldcg(reinterpret_cast<const ulonglong2*>(cl));
        const ulonglong2 b2 = __ldcg(reinterpret_cast<const ulonglong2*>(cl) + 1);
        const uint4 kk = __ldcg(reinterpret_cast<const uint4*>(A.rkw[slot].K));
        const int4 wd = __ldcg(reinterpret_cast<const int4*>(A.rkw[slot].W));
        rc.S[0] = a.x; rc.S[1] = a.y; rc.S[2] = b2.x; rc.S[3] = b2.y;
        rc.K[0] = kk.x; rc.K[1] = kk.y; rc.K[2] = kk.z; rc.K[3] = kk.w;
        rc.Wd[0] = wd.x; rc.Wd[1] = wd.y; rc.Wd[2] = wd.z;
        __stcg(reinterpret_cast<ulonglong2*>(cl), make_ulonglong2(0ull, 0ull));
        __stcg(reinterpret_cast<ulonglong2*>(cl) + 1, make_ulonglong2(0ull, 0ull));
        __stcg(reinterpret_cast<uint4*>(A.rkw[slot].K), make_uint4(0u, 0u, 0u, 0u));
        __stcg(reinterpret_cast<int4*>(A.rkw[slot].W), make_int4(0, 0, 0, 0));
        M.flip[x] = root_record(ch, sweep, (uint32_t)x, rc, acc);
      }
      // exact block reduction in 16-bit limbs (as k_cluster)
#pragma unroll
      for (int i = 0; i < NQ; ++i)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          const unsigned v = __reduce_add_sync(0xFFFFFFFFu, (unsigned)((acc.q[i] >> (16 * l)) & 0xFFFFull));
          if (lane == 0) M.limb[wid * NLIMB + 4 * i + l] = v;
        }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const unsigned long long wv = l < 4 ? acc.w[i].lo : acc.w[i].hi;
          const unsigned v = __reduce_add_sync(0xFFFFFFFFu, (unsigned)((wv >> (16 * (l & 3))) & 0xFFFFull));
          if (lane == 0) M.limb[wid * NLIMB + QLIMB + 8 * i + l] = v;
        }
      if (tid < REC_WORDS) M.tot[NLIMB + tid] = 0ull;
      __syncthreads();
      for (int j = tid; j < NLIMB; j += RES_THREADS) {
        unsigned long long sum = 0;
        for (int w = 0; w < RES_THREADS / 32; ++w) sum += M.limb[w * NLIMB + j];
        M.tot[j] = sum;
      }
      __syncthreads();
      if (tid < NQ) {
        unsigned long long v = 0;
        for (int l = 0; l < 4; ++l) v += M.tot[4 * tid + l] << (16 * l);
        M.tot[NLIMB + kRecQ[tid]] = v;
      } else if (tid < NQ + 8) {
        const int k = tid - NQ;
        u128 v = {0, 0};
        for (int l = 0; l < 8; ++l) {
          const unsigned long long t = M.tot[QLIMB + 8 * k + l];
          const int sh = 16 * l;
          u128 add;
          add.lo = sh < 64 ? (t << sh) : 0ull;
          add.hi = sh == 0 ? 0ull : (sh < 64 ? (t >> (64 - sh)) : (t << (sh - 64)));
          add_u128(v, add);
        }
        M.tot[NLIMB + kRecW[k]] = v.lo;
        M.tot[NLIMB + kRecW[k] + 1] = v.hi;
      } else if (tid == NQ + 8) {
        M.tot[NLIMB + R_NOP] = (unsigned long long)nv;
      }
      // ---- spin flips, vertex types, the next sweep's off-diagonal lists (path_integral.C:805-823)
      for (int i = tid; i < N; i += RES_THREADS) {
        const int base = M.sbase[i];
        const int k = M.sbase[i + 1] - base - 1;
        uint8_t fprev = M.flip[M.par[base]];
        if (fprev) M.spin[i] ^= 1u;
        int n = 0;
        for (int j = 1; j <= k; ++j) {
          const int x = base + j;
          const uint8_t fx = M.flip[M.par[x]];
          if ((((M.si[x] & SI_OFF) ? 1u : 0u) ^ fprev ^ fx) != 0) {
            M.st[base + n] = M.st[x];
            M.sd[base + n] = M.sd[x] & SD_IMASK;  // the list keeps the incidence index
            ++n;
          }
          fprev = fx;
        }
        M.obase[i] = base;
        M.ocnt[i] = n;
      }
      __syncthreads();
      if (tid < REC_WORDS)
        A.rec[((size_t)step * A.C + c) * REC_WORDS + tid] = M.tot[NLIMB + tid];
    }
    // ---- store the persistent state into the out set: spins, packed lists, sweep counter
    for (int i = tid; i < N; i += RES_THREADS) M.sv[i] = M.ocnt[i];
    __syncthreads();
    res_scan(M.sv, N, M.sv, sw);
    const size_t lbase = (size_t)c * R.lcap;
    for (int i = tid; i < N; i += RES_THREADS) {
      const int dst = (int)lbase + M.sv[i], src = M.obase[i], n = M.ocnt[i];
      for (int j = 0; j < n; ++j) { R.st_out[dst + j] = M.st[src + j]; R.sd_out[dst + j] = M.sd[src + j]; }
      R.spin_out[so + i] = M.spin[i];
      R.obase_out[so + i] = dst;
      R.ocnt_out[so + i] = n;
    }
    if (tid == 0) A.ch_sweep[c] = sweep;
    __syncthreads();
  }
}

}  // namespace lg
