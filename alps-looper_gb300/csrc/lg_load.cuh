// Device side of lg_load for a single chain on the grid path: the checkpoint's operators (bond
// i32 and time f64, 12 bytes each, in (time, bond) order as lg_save writes them) are decoded,
// checked and packed into the per-site endpoint lists the sweep keeps, on the GPU.
//
//   k_ld_count     per operator: range checks (first bad operator), order check against the
//                  previous operator, endpoints per site
//   k_ld_scan_*    site offsets (exclusive scan of the counts)
//   k_ld_place     per operator: its two endpoints at claimed slots of their sites' ranges
//   k_ld_sort      warp per site: the site's endpoints in operator order (= (time, bond) order),
//                  ranked by counting in shared memory; odd spin-1/2 sites reported
//   k_ld_commit_*  after the host has seen every check pass: the lists, offsets and spins
//
// Nothing persistent is written before the commit kernels, so a rejected checkpoint leaves the
// chain as it was.  Input that is not in order, or a site with more than LD_SORT_MAX endpoints,
// is flagged and packed by the host instead.
#pragma once
#include <climits>
#include <cstdint>

namespace lg {

constexpr int LD_SORT_MAX = 1024;  // endpoints per site the warp sort stages
constexpr int LD_SORT_WARPS = 8;
constexpr int LD_FLAG_UNORDERED = 1, LD_FLAG_LONG = 2;

struct LoadArgs {
  const uint8_t* spins;     // N staged spin bytes
  const uint32_t* ops;      // 3n staged words: bond, time low word, time high word
  long long n;              // operators
  int N, NB;
  const int* s0;            // sites of bond b
  const int* s1;
  const uint8_t* dir0;      // incidence index of bond b at s0 / s1
  const uint8_t* dir1;
  int* cnt;                 // N: endpoints per site (zero on entry)
  int* fill;                // N: claimed slots per site (zero on entry)
  int* off;                 // N + 1: site offsets
  int* partial;             // scan partials (one per 1024 sites)
  uint32_t* rec;            // 2n: operator index | side << 31, site by site
  int* status;              // [0] first bad operator, [1] flags, [2] first odd site
  int parity;               // spin 1/2: every site needs an even count
};

// Operator i: bond and time bits (a time of -0 read as +0); false when out of range.
__device__ __forceinline__ bool ld_op(const LoadArgs& L, long long i, int* b, uint64_t* tb) {
  const uint32_t* w = L.ops + 3 * i;
  *b = (int)w[0];
  uint64_t t = ((uint64_t)w[2] << 32) | w[1];
  if (t == 0x8000000000000000ull) t = 0;
  *tb = t;
  // 0 <= t < 1 as a double: sign clear and below the bits of 1.0 (NaN and infinities are above)
  return *b >= 0 && *b < L.NB && t < 0x3FF0000000000000ull;
}

__global__ void __launch_bounds__(256) k_ld_count(LoadArgs L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n;
       i += (long long)gridDim.x * blockDim.x) {
    int b;
    uint64_t tb;
    if (!ld_op(L, i, &b, &tb)) {
      atomicMin(&L.status[0], (int)i);
      continue;
    }
    if (i > 0) {
      int pb;
      uint64_t pt;
      ld_op(L, i - 1, &pb, &pt);
      if (!(pt < tb || (pt == tb && pb <= b))) atomicOr(&L.status[1], LD_FLAG_UNORDERED);
    }
    atomicAdd(&L.cnt[L.s0[b]], 1);
    atomicAdd(&L.cnt[L.s1[b]], 1);
  }
}

// Offsets of at most 1024 * 1024 sites: block totals, then every block scans the block totals for
// its own base and its sites; the last block writes off[N].
__global__ void __launch_bounds__(1024) k_ld_scan_blocks(LoadArgs L) {
  __shared__ int sw[32];
  const int s = blockIdx.x * 1024 + threadIdx.x;
  int tot;
  block_exclusive_scan(s < L.N ? L.cnt[s] : 0, sw, &tot);
  if (threadIdx.x == 0) L.partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_ld_scan_offsets(LoadArgs L) {
  __shared__ int sw[32];
  __shared__ int base;
  const int nparts = gridDim.x;
  int ptot;
  const int pex = block_exclusive_scan((int)threadIdx.x < nparts ? L.partial[threadIdx.x] : 0, sw, &ptot);
  if ((int)threadIdx.x == (int)blockIdx.x) base = pex;
  __syncthreads();
  const int s = blockIdx.x * 1024 + threadIdx.x;
  int tot;
  const int ex = block_exclusive_scan(s < L.N ? L.cnt[s] : 0, sw, &tot);
  if (s < L.N) L.off[s] = base + ex;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) L.off[L.N] = ptot;
}

__global__ void __launch_bounds__(256) k_ld_place(LoadArgs L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L.n;
       i += (long long)gridDim.x * blockDim.x) {
    int b;
    uint64_t tb;
    ld_op(L, i, &b, &tb);
    const int a = L.s0[b], c = L.s1[b];
    L.rec[L.off[a] + atomicAdd(&L.fill[a], 1)] = (uint32_t)i;
    L.rec[L.off[c] + atomicAdd(&L.fill[c], 1)] = (uint32_t)i | 0x80000000u;
  }
}

// Warp per site: the site's endpoints sorted by operator index (each operator reaches a site at
// most once, so the indices are distinct): each entry's rank is the number of smaller ones.
__global__ void __launch_bounds__(LD_SORT_WARPS * 32) k_ld_sort(LoadArgs L) {
  __shared__ uint32_t buf[LD_SORT_WARPS][LD_SORT_MAX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int warps = gridDim.x * LD_SORT_WARPS;
  for (int s = blockIdx.x * LD_SORT_WARPS + w; s < L.N; s += warps) {
    const int m = L.cnt[s], base = L.off[s];
    if (L.parity && (m & 1) && lane == 0) atomicMin(&L.status[2], s);
    if (m > LD_SORT_MAX) {
      if (lane == 0) atomicOr(&L.status[1], LD_FLAG_LONG);
      continue;
    }
    if (m < 2) continue;
    for (int j = lane; j < m; j += 32) buf[w][j] = L.rec[base + j];
    __syncwarp();
    for (int j = lane; j < m; j += 32) {
      const uint32_t e = buf[w][j], key = e & 0x7FFFFFFFu;
      int r = 0;
      for (int q = 0; q < m; ++q) r += (buf[w][q] & 0x7FFFFFFFu) < key;
      L.rec[base + r] = e;
    }
    __syncwarp();
  }
}

// Commit: the sorted endpoints into the site lists (time bits, incidence index) ...
__global__ void __launch_bounds__(256) k_ld_commit_lists(LoadArgs L, uint64_t* stime, uint8_t* sdir) {
  const long long n2 = 2 * L.n;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n2;
       k += (long long)gridDim.x * blockDim.x) {
    const uint32_t e = L.rec[k];
    int b;
    uint64_t tb;
    ld_op(L, e & 0x7FFFFFFFu, &b, &tb);
    stime[k] = tb;
    sdir[k] = (e >> 31) ? L.dir1[b] : L.dir0[b];
  }
}

// ... and per site its list's place and length and its spin.
__global__ void __launch_bounds__(256) k_ld_commit_sites(LoadArgs L, int* off_base, int* off_cnt,
                                                        uint8_t* spin0) {
  LG_GRID_STRIDE(s, L.N) {
    off_base[s] = L.off[s];
    off_cnt[s] = L.cnt[s];
    spin0[s] = (uint8_t)(L.spins[s] & 1u);
  }
}

}  // namespace lg
