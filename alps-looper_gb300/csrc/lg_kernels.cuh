// Sweep kernels of the GB300 loop-cluster engine.
//
// One sweep of every chain in the arena (path_integral.C:355-864) is this kernel sequence:
//
//   k_begin          zero this sweep's measurement records                   (:472-479 reset)
//   k_insert<0>      per bond: count vertices of the new operator string      (:403-577)
//   scan             bond vertex offsets; capacity check
//   k_insert<1>      per bond: write vertices (time, graph, type)             (:403-577)
//   k_site_count     per site: number of segments = 1 + incident vertices
//   scan             site segment offsets
//   k_merge          per site: time-ordered segment list, union-find init,
//                    temporal closure                                          (:584-589)
//   k_union          per vertex: lock-free unions of its four legs            (graph_impl.h:280-295)
//   k_compress       per segment: parent := root; roots clear accumulators    (union_find.h:324-343)
//   k_accumulate     per segment: length into the root's class sums           (:650-737)
//   k_cluster        per root: flip coin, improved / field sums -> records     (:739-803)
//   k_flip_vertex    per vertex: new diagonal/off-diagonal type               (:805-818)
//   k_site_end       per site: spin flip, compacted off-diagonal list         (:822-823)
//   k_end            per chain: operator count, sweep counter
//
// Memory layout (HBM, struct of arrays, 32-bit indices):
//   sites    spin0[N] u8, off_base[N], off_cnt[N]     persistent between sweeps
//   bonds    s0/s1[NB], chain[NB], dir0[NB] u8         static
//   vertices (bond-major CSR by bond_ptr) vtime u64 (FP64 bits), vcode u8 = g<<1|offdiag,
//            vnew u8, vslot[2] i32 (segment of the leg on source / target site)
//   segments (site-major CSR by sbase, k_s+1 per site, bottom segment first) stime u64,
//            sinfo u8, svert i32, sdir u8, parent i32, flip u8, cls[4] u64, cnt0[4] u32
//   records  rec[step][chain][32] u64 — exact integer sums (see the R_* word map)
#pragma once
#include <cstdint>

#include "lg_numerics.cuh"
#include "lg_types.h"

namespace lg {

// sinfo bits
enum : uint8_t { SI_SPIN = 1, SI_GNEG = 2, SI_FIRST = 4, SI_LAST = 8 };

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
  const int8_t* gauge;     // N
  const int* site_chain;   // N
  // per-chain mutable
  uint32_t* ch_sweep;      // C
  int* ch_slot_off;        // C+1 (this sweep)
  // persistent site state
  uint8_t* spin0;
  int* off_base;
  int* off_cnt;
  // per-sweep
  int* bond_cnt;           // NB
  int* bond_ptr;           // NB+1
  int* site_cnt;           // N
  int* sbase;              // N+1
  uint64_t* vtime;
  uint8_t* vcode;
  uint8_t* vnew;
  int* vslot;
  uint64_t* stime;
  uint8_t* sinfo;
  int* svert;
  uint8_t* sdir;
  int* parent;
  uint8_t* flip;
  unsigned long long* cls;  // 4 per segment
  unsigned int* cnt0;       // 4 per segment
  unsigned long long* rec;  // [rows][C][REC_WORDS]
  Ctl* ctl;
};

#define LG_GRID_STRIDE(i, n) \
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__device__ __forceinline__ unsigned long long* rec_row(const Arena& A, int c) {
  return A.rec + ((size_t)A.ctl->step * A.C + c) * REC_WORDS;
}

// ---------------------------------------------------------------------------------------------
__global__ void k_begin(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(i, A.C * REC_WORDS) {
    A.rec[(size_t)A.ctl->step * A.C * REC_WORDS + i] = 0ull;
  }
}

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
template <bool WRITE>
__global__ void __launch_bounds__(256) k_insert(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(b, A.NB) {
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
      const float gap = __fmul_rn(-log_open(uniform_open(wu)), ch.inv_rate);
      const uint64_t q = gap_fix52(gap, ((uint64_t)(wu & 0x1FFu) << 16) | (wg & 0xFFFFu));
      if (q >= FIX52_ONE) { more = false; return; }
      tq += q;
      if (tq >= FIX52_ONE) { more = false; return; }
      tp = fix52_bits(tq);
      gp = (uint32_t)((uint64_t)wg >= ch.T0) + (uint32_t)((uint64_t)wg >= ch.T1) +
           (uint32_t)((uint64_t)wg >= ch.T2);
    };
    next_prop();

    int out = WRITE ? A.bond_ptr[b] : 0;
    uint32_t ordinal = 0;
    rnd4 ro = {0, 0, 0, 0};
    while (true) {
      if (t0 <= t1 && t0 <= tp) {
        if (t0 == TIME_INF) break;
        p0 ^= 1u;
        if (A.sdir[i0] == own) {
          if (WRITE) {
            if ((ordinal & 3u) == 0) ro = philox(ch.seed, sweep, bl, TAG_OFFDIAG, ordinal >> 2);
            const uint32_t w = (ordinal & 3u) == 0 ? ro.x : (ordinal & 3u) == 1 ? ro.y
                             : (ordinal & 3u) == 2 ? ro.z : ro.w;
            const uint32_t g = ((uint64_t)w < ch.Poff) ? 0u : 1u;
            A.vtime[out] = t0;
            A.vcode[out] = (uint8_t)((g << 1) | 1u);
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
          }
          ++out;
        }
        next_prop();
      }
    }
    if (!WRITE) A.bond_cnt[b] = out;
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
__global__ void k_site_count(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(s, A.N) {
    int k = 1;
    for (int j = A.inc_off[s]; j < A.inc_off[s + 1]; ++j) k += A.bond_cnt[A.inc[j]];
    A.site_cnt[s] = k;
  }
}

// ---------------------------------------------------------------------------------------------
// Per site: merge the time-ordered vertex lists of its incident bonds into the site's segment
// list.  Segment j (0 <= j <= k) starts at the j-th endpoint (the bottom segment j = 0 starts at
// tau = 0) and carries the spin after that endpoint.  Ties: (time, off-diagonal first, bond).
// Also: union-find initialisation and the temporal closure (top segment hooked to the bottom,
// path_integral.C:584-589).
__global__ void __launch_bounds__(128) k_merge(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(s, A.N) {
    const int j0 = A.inc_off[s];
    const int z = A.inc_off[s + 1] - j0;
    const int base = A.sbase[s];
    const int k = A.sbase[s + 1] - base - 1;
    const uint8_t gneg = A.gauge[s] < 0 ? SI_GNEG : 0;
    int cur[MAXZ], end[MAXZ];
    uint64_t ht[MAXZ];
    uint8_t hc[MAXZ], side[MAXZ];
#pragma unroll
    for (int d = 0; d < MAXZ; ++d) {
      if (d < z) {
        const int b = A.inc[j0 + d];
        cur[d] = A.bond_ptr[b];
        end[d] = A.bond_ptr[b + 1];
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
      for (int d = 1; d < MAXZ; ++d) {
        const uint8_t dg = (uint8_t)(~hc[d] & 1u);
        if (ht[d] < bt || (ht[d] == bt && dg < bdiag)) { best = d; bt = ht[d]; bdiag = dg; }
      }
      const int x = base + j;
      int v = 0;
      uint8_t sd = 0, code = 0;
#pragma unroll
      for (int d = 0; d < MAXZ; ++d) {
        if (d == best) {
          v = cur[d]; sd = side[d]; code = hc[d];
          ++cur[d];
          ht[d] = cur[d] < end[d] ? A.vtime[cur[d]] : TIME_INF;
          hc[d] = cur[d] < end[d] ? A.vcode[cur[d]] : 0;
        }
      }
      if (code & 1u) spin ^= 1u;
      A.stime[x] = bt;
      A.sinfo[x] = (uint8_t)(spin | gneg | (j == k ? SI_LAST : 0));
      A.svert[x] = v;
      A.sdir[x] = (uint8_t)best;
      A.parent[x] = x;
      A.vslot[2 * v + sd] = x;
    }
    if (k > 0) A.parent[base + k] = base;  // closure: top segment joins the bottom one
    const int c = A.site_chain[s];
    if (s == A.ch[c].site_off) A.ch_slot_off[c] = base;
    if (s == A.N - 1) A.ch_slot_off[A.C] = base + k + 1;
  }
}

// ---------------------------------------------------------------------------------------------
// Lock-free union-find on segments.  Roots are hooked larger-index -> smaller-index with
// atomicCAS, so the root of every cluster is its smallest segment index whatever the order of
// the unions (the deterministic unify of union_find.h:231-233,270-273).  Finds halve paths with
// plain stores: a store only ever replaces a non-root's parent by one of its ancestors.
__device__ __forceinline__ int uf_find(int* P, int x) {
  while (true) {
    const int p = __ldcg(P + x);
    if (p == x) return x;
    const int gp = __ldcg(P + p);
    if (gp == p) return p;
    P[x] = gp;
    x = gp;
  }
}

__device__ __forceinline__ bool uf_union(int* P, int a, int b) {
  for (int it = 0; it < ITER_CAP; ++it) {
    a = uf_find(P, a);
    b = uf_find(P, b);
    if (a == b) return true;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int old = atomicCAS(P + hi, hi, lo);
    if (old == hi) return true;
    a = lo;
    b = old;
  }
  return false;
}

// reconnect (graph_impl.h:280-295) in segment form: g = 0 joins the two lower legs and the two
// upper legs; g = 1 joins lower-left with upper-right and lower-right with upper-left; frozen
// graphs (g & 2) join all four legs.
__global__ void __launch_bounds__(256) k_union(Arena A) {
  if (A.ctl->err) return;
  const int nv = A.ctl->nv_total;
  bool ok = true;
  LG_GRID_STRIDE(v, nv) {
    const int a = A.vslot[2 * v], b = A.vslot[2 * v + 1];
    const int g = A.vcode[v] >> 1;
    if (g & 2) {
      ok &= uf_union(A.parent, a - 1, b - 1);
      ok &= uf_union(A.parent, a, b);
      ok &= uf_union(A.parent, a - 1, a);
    } else if (g == 0) {
      ok &= uf_union(A.parent, a - 1, b - 1);
      ok &= uf_union(A.parent, a, b);
    } else {
      ok &= uf_union(A.parent, a - 1, b);
      ok &= uf_union(A.parent, b - 1, a);
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
    if (r == x) {
#pragma unroll
      for (int q = 0; q < 4; ++q) { A.cls[4 * (size_t)x + q] = 0ull; A.cnt0[4 * (size_t)x + q] = 0u; }
    }
  }
}

// Per segment: its length in 2^-40 units goes to one of four class sums of its cluster,
// class = (spin, gauge sign).  Bottom segments also count into the tau = 0 class counts.
// These eight integers per cluster determine every improved estimator of
// susceptibility.h:96-156 and the field weight of cluster.h:54-59.
__global__ void __launch_bounds__(256) k_accumulate(Arena A) {
  if (A.ctl->err) return;
  const int ns = A.ctl->ns_total;
  LG_GRID_STRIDE(x, ns) {
    const uint8_t info = A.sinfo[x];
    const int64_t ta = bits_fix40(A.stime[x]);
    const int64_t tb = (info & SI_LAST) ? ((int64_t)1 << 40) : bits_fix40(A.stime[x + 1]);
    const int q = (info & SI_SPIN) * 2 + ((info & SI_GNEG) ? 1 : 0);
    const int r = A.parent[x];
    atomicAdd(A.cls + 4 * (size_t)r + q, (unsigned long long)(tb - ta));
    if (info & SI_FIRST) atomicAdd(A.cnt0 + 4 * (size_t)r + q, 1u);
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

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
  unsigned long long s = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const unsigned limb = (unsigned)((v >> (16 * q)) & 0xFFFFull);
    s += (unsigned long long)__reduce_add_sync(0xFFFFFFFFu, limb) << (16 * q);
  }
  return s;
}

__device__ __forceinline__ u128 warp_sum_u128(u128 v) {
  u128 s = {0, 0};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const unsigned long long w = q < 4 ? v.lo : v.hi;
    const unsigned limb = (unsigned)((w >> (16 * (q & 3))) & 0xFFFFull);
    const unsigned long long t = __reduce_add_sync(0xFFFFFFFFu, limb);
    const int sh = 16 * q;
    // add t << sh into s (t < 2^21)
    unsigned long long lo_add = sh < 64 ? (t << sh) : 0ull;
    unsigned long long hi_add = sh == 0 ? 0ull : (sh < 64 ? (t >> (64 - sh)) : (t << (sh - 64)));
    const unsigned long long nlo = s.lo + lo_add;
    s.hi += hi_add + (nlo < s.lo ? 1ull : 0ull);
    s.lo = nlo;
  }
  return s;
}

// Per cluster root: flip decision (path_integral.C:780-803) and the exact per-sweep sums of the
// improved estimator collector (susceptibility.h:182-198), cluster count (:774-778), field
// energy (:852-859) and the normal time-integrated magnetisations (susceptibility.h:283-297).
__global__ void __launch_bounds__(256) k_cluster(Arena A) {
  if (A.ctl->err) return;
  const int ns = A.ctl->ns_total;
  const int lane = threadIdx.x & 31;
  const int wstride = gridDim.x * blockDim.x;
  for (int wbase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; wbase < ns; wbase += wstride) {
    const int x = wbase + lane;
    const bool is_root = x < ns && A.parent[x] == x;
    int c = 0;
    unsigned long long q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    u128 w[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) w[i] = {0, 0};
    if (is_root) {
      // chain of this segment (binary search over chain segment offsets)
      int lo = 0, hi = A.C - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.ch_slot_off[mid] <= x) lo = mid; else hi = mid - 1;
      }
      c = lo;
      const DChain ch = A.ch[c];
      const unsigned long long* S = A.cls + 4 * (size_t)x;
      const unsigned* K = A.cnt0 + 4 * (size_t)x;
      const long long s0 = (long long)S[0], s1 = (long long)S[1], s2 = (long long)S[2],
                      s3 = (long long)S[3];
      const long long k0 = K[0], k1 = K[1], k2 = K[2], k3 = K[3];
      const long long Ls = s0 + s1 + s2 + s3, Ms = s0 + s1 - s2 - s3;
      const long long SLs = s0 - s1 + s2 - s3, SMs = s0 - s1 - s2 + s3;
      const long long n0 = k0 + k1 + k2 + k3, m0 = k0 + k1 - k2 - k3;
      const long long sn0 = k0 - k1 + k2 - k3, sm0 = k0 - k1 - k2 + k3;
      const uint32_t key = (uint32_t)(x - A.ch_slot_off[c]);
      const rnd4 r = philox(ch.seed, A.ch_sweep[c], key, TAG_FLIP, 0);
      uint8_t f;
      if (!ch.field) {
        f = r.x < 0x80000000u ? 1 : 0;
      } else {
        const float xf = __fmul_rn(__ll2float_rn(Ms), ch.flip_coef);
        const float e = exp_clamped(xf);
        f = __fmul_rn(uniform_open(r.x), __fadd_rn(1.0f, e)) < 1.0f ? 1 : 0;
      }
      A.flip[x] = f;
      q[0] = 1ull;
      q[1] = (unsigned long long)m0;
      q[2] = (unsigned long long)sm0;
      q[3] = (unsigned long long)(m0 * m0);
      q[4] = (unsigned long long)(n0 * n0);
      q[5] = (unsigned long long)(sm0 * sm0);
      q[6] = (unsigned long long)(sn0 * sn0);
      q[7] = (unsigned long long)(f ? -Ms : Ms);
      q[8] = (unsigned long long)Ms;
      q[9] = (unsigned long long)SMs;
      w[0] = mul64(q[3], q[3]);
      w[1] = mul64(q[4], q[4]);
      w[2] = mul64(q[5], q[5]);
      w[3] = mul64(q[6], q[6]);
      auto ab = [](long long v) { return (unsigned long long)(v < 0 ? -v : v); };
      w[4] = mul64(ab(Ls), ab(Ls));
      w[5] = mul64(ab(Ms), ab(Ms));
      w[6] = mul64(ab(SLs), ab(SLs));
      w[7] = mul64(ab(SMs), ab(SMs));
    }
    const unsigned any = __ballot_sync(0xFFFFFFFFu, is_root);
    if (!any) continue;
    const int leader = __ffs(any) - 1;
    const int c0 = __shfl_sync(0xFFFFFFFFu, c, leader);
    const bool uniform = __all_sync(0xFFFFFFFFu, !is_root || c == c0);
    const int qw[10] = {R_NC, R_M0, R_SM0, R_M0SQ, R_N0SQ, R_SM0SQ, R_SN0SQ, R_FLD, R_MA, R_SMA};
    const int ww[8] = {R_M0Q, R_N0Q, R_SM0Q, R_SN0Q, R_LSQ, R_MSQ, R_SLSQ, R_SMSQ};
    if (uniform) {
      unsigned long long* row = rec_row(A, c0);
#pragma unroll
      for (int i = 0; i < 10; ++i) {
        const unsigned long long t = warp_sum_u64(q[i]);
        if (lane == leader && t) atomicAdd(row + qw[i], t);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const u128 t = warp_sum_u128(w[i]);
        if (lane == leader && (t.lo | t.hi)) atomic_add_u128(row + ww[i], t);
      }
    } else if (is_root) {
      unsigned long long* row = rec_row(A, c);
#pragma unroll
      for (int i = 0; i < 10; ++i) if (q[i]) atomicAdd(row + qw[i], q[i]);
#pragma unroll
      for (int i = 0; i < 8; ++i) if (w[i].lo | w[i].hi) atomic_add_u128(row + ww[i], w[i]);
    }
  }
}

// Per vertex: flip the operator type when its two clusters flip differently
// (path_integral.C:815-818; loop_0/loop_1 of graph_impl.h:489-494 in segment form).
__global__ void __launch_bounds__(256) k_flip_vertex(Arena A) {
  if (A.ctl->err) return;
  const int nv = A.ctl->nv_total;
  LG_GRID_STRIDE(v, nv) {
    const int a = A.vslot[2 * v], b = A.vslot[2 * v + 1];
    const uint8_t code = A.vcode[v];
    const int g = code >> 1;
    uint8_t t = 0;
    if (!(g & 2)) {
      const int l = A.parent[a - 1];
      const int o = (g == 0) ? A.parent[a] : A.parent[b - 1];
      t = A.flip[l] ^ A.flip[o];
    }
    A.vnew[v] = (uint8_t)((code & 1u) ^ t);
  }
}

// Per site: flip the tau = 0 spin with its bottom segment's cluster (path_integral.C:822-823)
// and compact the off-diagonal endpoints (time order kept) in place at the start of the site's
// segment range: this is the next sweep's off-diagonal list.
__global__ void __launch_bounds__(128) k_site_end(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(s, A.N) {
    const int base = A.sbase[s];
    const int k = A.sbase[s + 1] - base - 1;
    if (A.flip[A.parent[base]]) A.spin0[s] ^= 1u;
    int n = 0;
    for (int j = 1; j <= k; ++j) {
      const int x = base + j;
      if (A.vnew[A.svert[x]]) {
        A.stime[base + n] = A.stime[x];
        A.sdir[base + n] = A.sdir[x];
        ++n;
      }
    }
    A.off_base[s] = base;
    A.off_cnt[s] = n;
  }
}

__global__ void k_end(Arena A) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(c, A.C) {
    const DChain ch = A.ch[c];
    const int nv = A.bond_ptr[ch.bond_off + ch.nbonds] - A.bond_ptr[ch.bond_off];
    rec_row(A, c)[R_NOP] = (unsigned long long)nv;
    A.ch_sweep[c] += 1u;
  }
}

__global__ void k_step(Ctl* ctl) {
  if (ctl->err) return;
  ctl->step += 1u;
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
