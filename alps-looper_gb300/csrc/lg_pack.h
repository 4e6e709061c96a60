// Host-side packing of a chain's off-diagonal operators into the per-site endpoint lists the
// sweep keeps (lg_load, lg_set_state): every operator (bond b, time t) is an endpoint at both of
// b's sites; site i's endpoints are packed in (time, bond) order, the sites one after another.
//
// Input in (time, bond) order, which is how lg_save writes it, is packed on several threads in
// two cache-friendly passes: each thread appends its operators' endpoints to one record stream
// per block of consecutive sites (a few hundred write cursors instead of one per site), then each
// site block's records are counted and placed site by site.  Both passes keep the input order
// within a site, so the result is the stable counting sort by site.  Other input is sorted per site
// on one thread.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace lg {

struct PackTables {
  int N = 0, NB = 0;              // the chain's sites and bonds
  const int* s0 = nullptr;        // chain-local sites of bond b
  const int* s1 = nullptr;
  const uint8_t* dir0 = nullptr;  // incidence index of bond b at s0 / at s1
  const uint8_t* dir1 = nullptr;
  bool check_parity = true;       // spin 1/2: a world line needs an even count per site
};

struct PackResult {
  std::vector<int> oc;     // endpoints per site
  long long bad = -1;      // first operator out of range (bond, or time outside [0, 1)), or -1
  int odd_site = -1;       // first site with an odd number of endpoints (check_parity), or -1
  bool ordered = true;     // the input was in (time, bond) order
};

// One endpoint on its way to its site's list.
struct PackRec {
  uint64_t t;     // time bits
  uint32_t site;  // chain-local site
  uint32_t dir;   // incidence index
};

// Scratch of pack_site_lists: 2n records.
inline size_t pack_scratch_bytes(long long n) { return (size_t)(2 * n) * sizeof(PackRec); }

// Runs f(0..T-1), ranges 1.. on threads (on the calling thread where none can be started).
template <class F>
inline void pack_parallel(int T, const F& f) {
  std::vector<std::thread> th;
  int t = 1;
  try {
    th.reserve(T);
    for (; t < T; ++t) th.emplace_back(f, t);
  } catch (...) {
  }
  for (int u = t; u < T; ++u) f(u);
  f(0);
  for (auto& x : th) x.join();
}

// get(i, &bond, &time_bits) reads operator i of n.  t, d receive 2n endpoints; scratch holds
// pack_scratch_bytes(n) bytes (PackRec-aligned).  Stops early (with R.bad or R.odd_site set) on
// invalid input, leaving t and d undefined.  A time of -0 is read as +0.
template <class Get>
void pack_site_lists(const PackTables& P, long long n, const Get& get, uint64_t* t, uint8_t* d,
                     PackRec* scratch, PackResult& R, int max_threads) {
  const int N = P.N;
  R.oc.assign(N, 0);
  R.bad = -1;
  R.odd_site = -1;
  R.ordered = true;
  // threads: at most max_threads, about one per 64k operators
  const int T = (int)std::max<long long>(1, std::min<long long>(max_threads, n / 65536));
  const long long per = (n + T - 1) / T;
  // site blocks of 2^sh sites, at most 256 of them
  int sh = 0;
  while (((long long)(N - 1) >> sh) >= 256) ++sh;
  const int NBK = N > 0 ? ((N - 1) >> sh) + 1 : 1;
  auto read = [&](long long i, int* b, uint64_t* tb) {
    get(i, b, tb);
    double tv;
    std::memcpy(&tv, tb, 8);
    if (tv == 0.0) *tb = 0;
    return *b >= 0 && *b < P.NB && tv >= 0.0 && tv < 1.0;
  };
  // pass 1: validity, order and records per (thread, site block)
  std::vector<std::vector<long long>> cnt(T, std::vector<long long>(NBK, 0));
  std::vector<long long> bad(T, -1);
  std::vector<char> ord(T, 1);
  pack_parallel(T, [&](int k) {
    const long long i0 = k * per, i1 = std::min(n, i0 + per);
    long long* c = cnt[k].data();
    int pb = -1;
    uint64_t pt = 0;
    for (long long i = i0; i < i1; ++i) {
      int b;
      uint64_t tb;
      if (!read(i, &b, &tb)) { bad[k] = i; return; }
      ++c[P.s0[b] >> sh];
      ++c[P.s1[b] >> sh];
      if (i > i0 && !(pt < tb || (pt == tb && pb <= b))) ord[k] = 0;
      pb = b;
      pt = tb;
    }
  });
  for (int k = 0; k < T; ++k)
    if (bad[k] >= 0) { R.bad = bad[k]; return; }
  for (int k = 0; k < T; ++k) R.ordered &= ord[k] != 0;
  for (int k = 1; k < T && R.ordered; ++k) {  // across the ranges' boundaries
    const long long i = k * per;
    if (i >= n) break;
    int ba, bb;
    uint64_t ta, tb;
    read(i - 1, &ba, &ta);
    read(i, &bb, &tb);
    R.ordered = ta < tb || (ta == tb && ba <= bb);
  }
  if (!R.ordered) {
    // one thread: every site's entries, then a sort per site
    std::vector<long long> start(N + 1, 0);
    for (long long i = 0; i < n; ++i) {
      int b;
      uint64_t tb;
      read(i, &b, &tb);
      ++start[P.s0[b] + 1];
      ++start[P.s1[b] + 1];
    }
    for (int i = 0; i < N; ++i) R.oc[i] = (int)start[i + 1];
    if (P.check_parity)
      for (int i = 0; i < N; ++i)
        if (R.oc[i] & 1) { R.odd_site = i; return; }
    for (int i = 0; i < N; ++i) start[i + 1] += start[i];
    std::vector<std::pair<std::pair<uint64_t, int>, uint8_t>> ep(2 * n);  // ((time, bond), dir)
    std::vector<long long> fill(start.begin(), start.end() - 1);
    for (long long i = 0; i < n; ++i) {
      int b;
      uint64_t tb;
      read(i, &b, &tb);
      ep[fill[P.s0[b]]++] = {{tb, b}, P.dir0[b]};
      ep[fill[P.s1[b]]++] = {{tb, b}, P.dir1[b]};
    }
    for (int i = 0; i < N; ++i) {
      std::sort(ep.begin() + start[i], ep.begin() + start[i + 1]);  // the order the sweep produces
      for (long long k = start[i]; k < start[i + 1]; ++k) { t[k] = ep[k].first.first; d[k] = ep[k].second; }
    }
    return;
  }
  // record offsets: block-major, then thread, then input order (stable)
  std::vector<long long> bbase(NBK + 1, 0);
  for (int q = 0; q < NBK; ++q) {
    long long run = bbase[q];
    for (int k = 0; k < T; ++k) { const long long c = cnt[k][q]; cnt[k][q] = run; run += c; }
    bbase[q + 1] = run;
  }
  // pass 2: each thread appends its endpoints to the blocks' record streams
  pack_parallel(T, [&](int k) {
    const long long i0 = k * per, i1 = std::min(n, i0 + per);
    long long* at = cnt[k].data();
    for (long long i = i0; i < i1; ++i) {
      int b;
      uint64_t tb;
      read(i, &b, &tb);
      const int a = P.s0[b], c = P.s1[b];
      scratch[at[a >> sh]++] = PackRec{tb, (uint32_t)a, P.dir0[b]};
      scratch[at[c >> sh]++] = PackRec{tb, (uint32_t)c, P.dir1[b]};
    }
  });
  // pass 3: per site block, counts, parity and placement (the block's endpoints occupy the same
  // range [bbase[q], bbase[q+1]) in the output as in the records)
  std::vector<int> odd(T, -1);
  pack_parallel(T, [&](int k) {
    std::vector<long long> fill((size_t)1 << sh);
    for (int q = k; q < NBK; q += T) {
      const int sa = q << sh, sb = std::min(N, (q + 1) << sh);
      int* oc = R.oc.data();
      for (long long r = bbase[q]; r < bbase[q + 1]; ++r) ++oc[scratch[r].site];
      long long run = bbase[q];
      for (int s = sa; s < sb; ++s) {
        if (P.check_parity && (oc[s] & 1) && odd[k] < 0) odd[k] = s;
        fill[s - sa] = run;
        run += oc[s];
      }
      for (long long r = bbase[q]; r < bbase[q + 1]; ++r) {
        const PackRec& e = scratch[r];
        const long long pos = fill[e.site - sa]++;
        t[pos] = e.t;
        d[pos] = (uint8_t)e.dir;
      }
    }
  });
  for (int k = 0; k < T; ++k)
    if (odd[k] >= 0 && (R.odd_site < 0 || odd[k] < R.odd_site)) R.odd_site = odd[k];
}

}  // namespace lg
