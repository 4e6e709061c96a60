// Host side of the GB300 loop-cluster engine: the C ABI of include/looper_gpu.h.
//
// An Engine owns one ragged arena of independent chains (a single chain is an arena of one):
// static lattice tables, persistent per-site state, per-sweep vertex / segment buffers sized
// from the expected operator count, and a CUDA graph holding one sweep of every chain.  Sweeps
// run in chunks; after each chunk the exact per-sweep records come back to the host, which turns
// them into the reference's observables with a rebinning accumulator.
//
// Vertices are claimed from regions: every run of consecutive sites of a chain (about 4096
// expected vertices) has its own slot range and claim counter, so that claims do not contend on
// one address.  A sweep that would overflow a region is detected on the device by the insertion
// pass, before any persistent state is touched; the engine then grows the regions that
// overflowed to the demand they counted and replays that sweep with the same random numbers, so
// capacity never changes a trajectory.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/looper_gpu.h"
#include "lg_kernels.cuh"
#include "lg_pack.h"
#include "lg_load.cuh"
#include "lg_host.h"
#include "lg_resident.cuh"
#include "lg_sse.cuh"

using namespace lg;

// timed stages of one sweep, in launch order (an event is recorded after each stage)
static const int kNumStages = 7;
static const char* kStageNames[kNumStages] = {
    "k_insert", "k_site_count+scan(sites)", "k_merge", "k_union", "k_accumulate", "k_cluster",
    "k_site_end+k_end"};

static std::atomic<uint64_t> g_launches{0};
// bytes moved between host and device by this library (lg_copy_bytes, a measurement seam)
static std::atomic<uint64_t> g_h2d_bytes{0}, g_d2h_bytes{0};

static void count_copy(size_t n, cudaMemcpyKind k) {
  if (k == cudaMemcpyHostToDevice) g_h2d_bytes += n;
  else if (k == cudaMemcpyDeviceToHost) g_d2h_bytes += n;
}
static cudaError_t lg_copy(void* dst, const void* src, size_t n, cudaMemcpyKind k) {
  count_copy(n, k);
  return cudaMemcpy(dst, src, n, k);
}
static cudaError_t lg_copy_async(void* dst, const void* src, size_t n, cudaMemcpyKind k,
                                 cudaStream_t st) {
  count_copy(n, k);
  return cudaMemcpyAsync(dst, src, n, k, st);
}
static thread_local std::string g_err;

// A process-wide page-locked host buffer for the operator lists that lg_load and lg_set_state
// upload: a pinned source copies to the device at the link's rate, a pageable one goes through the
// driver's bounce buffer.  The first engine built in a process reserves it (cudaHostAlloc is slow
// enough to matter once per load), later loads grow it when they need more; a user holds the lock
// from packing until its copies have finished.  It lives until the process exits.
struct HostStage {
  std::mutex m;
  unsigned char* p = nullptr;
  size_t cap = 0;
  // (under the lock) at least n bytes; false when page-locked memory cannot be had (the caller
  // then packs into pageable memory)
  bool reserve(size_t n) {
    if (n <= cap) return true;
    const size_t want = std::max(n, 2 * cap);
    void* q = nullptr;
    if (cudaHostAlloc(&q, want, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (p) cudaFreeHost(p);
    p = static_cast<unsigned char*>(q);
    cap = want;
    return true;
  }
};
static HostStage& host_stage() {
  static HostStage* s = new HostStage();  // never destroyed: no CUDA call after the runtime is gone
  return *s;
}

int lg_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define LG_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return lg_fail(LG_EDEVICE, "%s failed: %s", #call, cudaGetErrorString(e_));            \
  } while (0)

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() { if (p) cudaFree(p); }
  void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
  void swap(DBuf& o) { std::swap(p, o.p); std::swap(n, o.n); }
  int alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) { p = nullptr; n = 0; return lg_fail(LG_ENOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e)); }
    return LG_OK;
  }
};

// Launch shape of an arena's sweep.  No choice here changes a result: every variant computes the
// same vertices, segments, clusters and exact sums.
//   insert_k  chains whose expected endpoints per site (2 beta W N_b / N) are below this insert
//             with a thread per bond, the others with a warp per site
//   narrow_k  the same split for the merge and the list compaction (thread / warp per site)
//   acc_tile  segments per block in k_accumulate (512, 1024, 2048)
//   cl_tile   segments per block in k_cluster (2048, 4096, 8192)
//   un_warps  warps per block in k_union (4, 8, 16)
//   resident  run the arena's sweeps as chain-resident launches (k_resident: one CTA per chain,
//             a chunk of sweeps per launch) where every chain fits in shared memory; the fields
//             above then wait for the arena to return to the grid path
//   union_mode  0: every union in k_union, a lane per vertex; 1: the lower-leg pairs of the
//             non-crossing vertices hooked first (k_union_pairs, spin-1/2 arenas only), the rest in
//             k_union; 2: the pairs first where allowed, the rest in k_union_bal (each warp's
//             unions balanced over its lanes)
struct Shape {
  double insert_k = 32.0;
  double narrow_k = 32.0;
  int acc_tile = 1024;
  int cl_tile = 4096;
  int un_warps = 8;
  int resident = 0;
  int union_mode = 2;
};

// Shared memory a chain-resident CTA may use by default: at most this much keeps two CTAs per SM.
constexpr size_t RES_SMEM_DEFAULT = 100 * 1024;
// The most any CTA can have (sm_103a: 227 KB of dynamic shared memory per block).
constexpr size_t RES_SMEM_MAX = 227 * 1024;

// ----------------------------------------------------------------------------------------------
struct Engine {
  std::vector<ChainSpec> spec;
  std::vector<ChainAcc> acc;
  std::vector<int> acc_of_chain;   // the accumulator chain c's measurements go to (exchange MC)
  int C = 0, N = 0, NB = 0;
  std::vector<DChain> hch;
  std::vector<int> h_bond_s0, h_bond_s1, h_inc_off, h_inc, h_inc_nbr;
  std::vector<uint8_t> h_inc_side, h_bond_dir0, h_bond_dir1, h_inc_dir;  // dir0/1: incidence index at s0/s1
  std::vector<int> h_site_chain, h_bond_chain;

  DBuf<DChain> d_ch;
  DBuf<int> d_bond_s0, d_bond_s1, d_bond_chain, d_inc_off, d_inc, d_inc_nbr, d_site_chain;
  DBuf<uint8_t> d_bond_dir0, d_inc_side, d_inc_dir;
  DBuf<int8_t> d_gauge;
  DBuf<uint32_t> d_sweep;
  DBuf<uint8_t> d_active;
  std::vector<uint8_t> h_active;
  DBuf<int> d_ch_slot_off;
  DBuf<uint8_t> d_spin0;
  DBuf<int> d_off_base, d_off_cnt;
  DBuf<int> d_bond_cnt, d_bond_ptr, d_site_cnt, d_sbase, d_partial;
  DBuf<uint64_t> d_vtime;
  DBuf<uint8_t> d_vcode;
  DBuf<int> d_vslot;
  DBuf<uint64_t> d_stime;
  DBuf<uint8_t> d_sinfo, d_sdir, d_flip;
  DBuf<int> d_svert, d_parent;
  DBuf<unsigned long long> d_cls;
  DBuf<RootKW> d_rkw;
  DBuf<unsigned long long> d_rec;
  DBuf<Ctl> d_ctl;
  // spin correlations: k_corr work tiles and the per-chunk exact sums (arena site indexed)
  int n_corr_tiles = 0, corr_smem = 0;
  bool any_spin_s = false;   // some chain has S > 1/2: k_boundary closes its sites
  // structural checks between stages (lg_validate_sweeps): the failure counter and first code;
  // never part of a captured graph
  int* val_bad = nullptr;
  bool capturing = false;
  DBuf<int2> d_corr_tiles;
  DBuf<long long> d_corr_disp, d_corr_origin;
  std::vector<long long> h_corr;

  int nv_cap = 0, ns_cap = 0;
  int rec_rows = 64;
  // vertex regions (see the file comment)
  int R = 0;
  std::vector<int> h_site_region;
  std::vector<long long> h_region_cap;
  long long region_total = 0;
  DBuf<int> d_site_region, d_region_base;
  DBuf<unsigned long long> d_region_fill;
  // site / bond classes of the current shape (nullptr list: all sites, in order)
  Shape shape;
  DBuf<int> d_wide_sites, d_narrow_sites, d_ins_sites, d_narrow_bonds;
  const int* wide_list = nullptr;   // merge / compaction, warp per site
  const int* ins_list = nullptr;    // insertion, warp per site
  int n_wide = 0, n_narrow = 0, n_ins = 0, n_narrow_b = 0;
  int sweep_launches = 0;         // kernel launches of one sweep
  int merge_cap = MERGE_CAP;      // k_merge staging capacity per warp (see set_merge_cap)
  cudaStream_t st2 = nullptr;     // the narrow kernels run beside the wide ones
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaStream_t st3 = nullptr;     // k_end runs beside the site pass
  cudaEvent_t ev_fork3 = nullptr, ev_join3 = nullptr;
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool use_graph = true;
  int nsm = 148;
  int zmax = MAXZ;                // largest number of incident bonds of a site (merge instance)
  int stream_priority = 0;   // CUDA stream priority of the arena's streams (0: the default)
  bool keep_records = false;
  std::vector<uint64_t> kept;   // raw records of chain 0 (test seam)
  // per-sweep observable values of the measurement sweeps (lg_keep_values / lg_fetch_values),
  // LG_NUM_VALUES doubles per sweep, per chain
  std::vector<uint8_t> keep_vals;
  std::vector<std::vector<double>> vals;
  std::vector<uint64_t> hrec;
  // ---- chain-resident sweeps (k_resident): the persistent state is double-buffered; d_spin0,
  // d_off_base, d_off_cnt, d_stime, d_sdir hold the current state (lists at off_base in the list
  // arrays, res_lcap entries per chain) and the rb_* set receives the next one
  bool resident = false;
  bool allow_resident = false;
  int res_vcap = 0, res_nmax = 0, res_nbmax = 0, res_lcap = 0, res_scap = 0, res_grid = 0;
  size_t res_smem = 0;
  DBuf<uint8_t> rb_spin0, rb_sdir;
  DBuf<int> rb_off_base, rb_off_cnt;
  DBuf<uint64_t> rb_stime;
  // ---- the SSE form (k_sse: one chain per warp): operator strings of sse_ocap entries per
  // chain, double-buffered with the spins (rb_spin0) like the resident path's state
  bool sse = false;
  int sse_ocap = 0, sse_fcap = 0, sse_grid = 0;
  DBuf<uint32_t> sse_ops, sse_ops_b, sse_ops_t;
  DBuf<int> sse_nop, sse_nop_b, sse_loops, sse_frag, sse_wnd, sse_cur;
  DBuf<long long> sse_est;
  DBuf<uint8_t> sse_spc, sse_flip;

  ~Engine() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_fork3) cudaEventDestroy(ev_fork3);
    if (ev_join3) cudaEventDestroy(ev_join3);
    if (st2) cudaStreamDestroy(st2);
    if (st3) cudaStreamDestroy(st3);
    if (st) cudaStreamDestroy(st);
  }

  Arena arena() {
    Arena A;
    A.ch = d_ch.p; A.C = C; A.N = N; A.NB = NB;
    A.bond_s0 = d_bond_s0.p; A.bond_s1 = d_bond_s1.p; A.bond_chain = d_bond_chain.p;
    A.bond_dir0 = d_bond_dir0.p; A.inc_off = d_inc_off.p; A.inc = d_inc.p;
    A.inc_side = d_inc_side.p; A.inc_nbr = d_inc_nbr.p; A.gauge = d_gauge.p;
    A.site_chain = d_site_chain.p;
    A.all_active = 1;
    for (uint8_t a : h_active) A.all_active &= a ? 1 : 0;
    A.ch_sweep = d_sweep.p; A.ch_slot_off = d_ch_slot_off.p; A.ch_active = d_active.p;
    A.spin0 = d_spin0.p; A.off_base = d_off_base.p; A.off_cnt = d_off_cnt.p;
    A.bond_cnt = d_bond_cnt.p; A.bond_ptr = d_bond_ptr.p; A.site_cnt = d_site_cnt.p;
    A.sbase = d_sbase.p;
    A.R = R; A.site_region = d_site_region.p; A.region_base = d_region_base.p;
    A.region_fill = d_region_fill.p;
    A.vtime = d_vtime.p; A.vcode = d_vcode.p; A.vslot = d_vslot.p;
    A.stime = d_stime.p; A.sinfo = d_sinfo.p; A.svert = d_svert.p; A.sdir = d_sdir.p;
    A.parent = d_parent.p; A.flip = d_flip.p; A.cls = d_cls.p; A.rkw = d_rkw.p; A.inc_dir = d_inc_dir.p;
    A.rec = d_rec.p; A.ctl = d_ctl.p; A.rec_rows = rec_rows;
    A.corr_tiles = d_corr_tiles.p; A.corr_disp = d_corr_disp.p; A.corr_origin = d_corr_origin.p;
    return A;
  }

  // ---- construction ----
  int build(const std::vector<ChainSpec>& specs, bool may_reside = false) {
    spec = specs;
    allow_resident = may_reside;
    C = (int)spec.size();
    acc.assign(C, ChainAcc());
    keep_vals.assign(C, 0);
    vals.assign(C, {});
    acc_of_chain.resize(C);
    for (int c = 0; c < C; ++c) acc_of_chain[c] = c;
    int dev = 0;
    LG_CUDA(cudaGetDevice(&dev));
    // one attribute, not cudaGetDeviceProperties (which queries every property, slowly)
    LG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    LG_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, stream_priority));
    LG_CUDA(cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, stream_priority));
    LG_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    LG_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    LG_CUDA(cudaStreamCreateWithPriority(&st3, cudaStreamNonBlocking, stream_priority));
    LG_CUDA(cudaEventCreateWithFlags(&ev_fork3, cudaEventDisableTiming));
    LG_CUDA(cudaEventCreateWithFlags(&ev_join3, cudaEventDisableTiming));
    LG_CUDA(cudaFuncSetAttribute(k_corr, cudaFuncAttributeMaxDynamicSharedMemorySize, CORR_SMEM));
    // static tables
    long long nsite = 0, nbond = 0;
    for (auto& s : spec) { nsite += s.N; nbond += s.NB; }
    if (nsite + 2 * 64ll > (1ll << 30) || nbond > (1ll << 30))
      return lg_fail(LG_EBUDGET, "arena too large (%lld sites, %lld bonds)", nsite, nbond);
    N = (int)nsite; NB = (int)nbond;
    hch.resize(C);
    h_bond_s0.resize(NB); h_bond_s1.resize(NB); h_bond_chain.resize(NB); h_bond_dir0.resize(NB);
    h_bond_dir1.resize(NB);
    h_site_chain.resize(N);
    std::vector<int8_t> h_gauge(N);
    h_inc_off.assign(N + 1, 0);
    int so = 0, bo = 0;
    for (int c = 0; c < C; ++c) {
      const ChainSpec& s = spec[c];
      hch[c] = s.dchain;
      hch[c].site_off = so; hch[c].nsites = s.N;
      hch[c].bond_off = bo; hch[c].nbonds = s.NB;
      for (int i = 0; i < s.N; ++i) { h_site_chain[so + i] = c; h_gauge[so + i] = (int8_t)s.gauge[i]; }
      for (int b = 0; b < s.NB; ++b) {
        h_bond_s0[bo + b] = so + s.s0[b];
        h_bond_s1[bo + b] = so + s.s1[b];
        h_bond_chain[bo + b] = c;
      }
      so += s.N; bo += s.NB;
    }
    // incident bonds per site, ascending bond id
    std::vector<int> deg(N, 0);
    for (int b = 0; b < NB; ++b) { deg[h_bond_s0[b]]++; deg[h_bond_s1[b]]++; }
    zmax = 0;
    for (int s = 0; s < N; ++s) {
      if (deg[s] > MAXZ) return lg_fail(LG_EUNSUPPORTED, "site coordination %d > %d", deg[s], MAXZ);
      h_inc_off[s + 1] = h_inc_off[s] + deg[s];
      zmax = std::max(zmax, deg[s]);
    }
    h_inc.assign(h_inc_off[N], 0);
    h_inc_side.assign(h_inc_off[N], 0);
    h_inc_nbr.assign(h_inc_off[N], 0);
    h_inc_dir.assign(h_inc_off[N], 0);
    std::vector<int> fill(N, 0);
    for (int b = 0; b < NB; ++b) {
      int a = h_bond_s0[b], t = h_bond_s1[b];
      const int c = h_bond_chain[b];
      // bond = (site*dim + d) * spin2^2 + virtual pair
      const int q = spec[c].spin2 * spec[c].spin2;
      const uint8_t dir = (uint8_t)(((b - hch[c].bond_off) / q) % spec[c].dim);
      int ia = h_inc_off[a] + fill[a]++;
      h_inc[ia] = b; h_inc_side[ia] = 0; h_inc_nbr[ia] = t; h_inc_dir[ia] = dir;
      int it = h_inc_off[t] + fill[t]++;
      h_inc[it] = b; h_inc_side[it] = 1; h_inc_nbr[it] = a; h_inc_dir[it] = dir;
    }
    // bonds were visited in ascending order, so each site's list is ascending already
    for (int b = 0; b < NB; ++b) {
      int a = h_bond_s0[b];
      for (int j = h_inc_off[a]; j < h_inc_off[a + 1]; ++j)
        if (h_inc[j] == b && h_inc_side[j] == 0) { h_bond_dir0[b] = (uint8_t)(j - h_inc_off[a]); break; }
      const int t = h_bond_s1[b];
      for (int j = h_inc_off[t]; j < h_inc_off[t + 1]; ++j)
        if (h_inc[j] == b) { h_bond_dir1[b] = (uint8_t)(j - h_inc_off[t]); break; }
    }
    int rc;
    if ((rc = d_ch.alloc(C)) || (rc = d_bond_s0.alloc(NB)) || (rc = d_bond_s1.alloc(NB)) ||
        (rc = d_bond_chain.alloc(NB)) || (rc = d_bond_dir0.alloc(NB)) ||
        (rc = d_inc_off.alloc(N + 1)) || (rc = d_inc.alloc(h_inc.size())) ||
        (rc = d_inc_nbr.alloc(h_inc.size())) || (rc = d_inc_dir.alloc(h_inc.size())) ||
        (rc = d_inc_side.alloc(h_inc.size())) || (rc = d_gauge.alloc(N)) ||
        (rc = d_site_chain.alloc(N)) || (rc = d_sweep.alloc(C)) || (rc = d_active.alloc(C)) ||
        (rc = d_ch_slot_off.alloc(C + 1)) || (rc = d_spin0.alloc(N)) ||
        (rc = d_off_base.alloc(N)) || (rc = d_off_cnt.alloc(N)) || (rc = d_bond_cnt.alloc(NB)) ||
        (rc = d_bond_ptr.alloc(NB + 1)) || (rc = d_site_cnt.alloc(N)) ||
        (rc = d_sbase.alloc(N + 1)) || (rc = d_ctl.alloc(1)))
      return rc;
    int maxparts = std::max((NB + SCAN_TILE - 1) / SCAN_TILE, (N + SCAN_TILE - 1) / SCAN_TILE);
    maxparts = std::max(maxparts, (N + SITE_SCAN_BLOCK - 1) / SITE_SCAN_BLOCK);  // k_site_blocks
    if ((rc = d_partial.alloc(maxparts + 1))) return rc;
    LG_CUDA(lg_copy(d_ch.p, hch.data(), C * sizeof(DChain), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_bond_s0.p, h_bond_s0.data(), NB * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_bond_s1.p, h_bond_s1.data(), NB * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_bond_chain.p, h_bond_chain.data(), NB * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_bond_dir0.p, h_bond_dir0.data(), NB, cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_inc_off.p, h_inc_off.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_inc.p, h_inc.data(), h_inc.size() * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_inc_side.p, h_inc_side.data(), h_inc_side.size(), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_inc_nbr.p, h_inc_nbr.data(), h_inc_nbr.size() * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_inc_dir.p, h_inc_dir.data(), h_inc_dir.size(), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_gauge.p, h_gauge.data(), N, cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_site_chain.p, h_site_chain.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    h_active.assign(C, 1);
    LG_CUDA(lg_copy(d_active.p, h_active.data(), C, cudaMemcpyHostToDevice));
    std::vector<uint32_t> sw(C);
    for (int c = 0; c < C; ++c) sw[c] = (uint32_t)spec[c].mcs;
    LG_CUDA(lg_copy(d_sweep.p, sw.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice));
    // vertex regions and per-sweep buffers from the expected operator count
    LG_CUDA(cudaMemset(d_ctl.p, 0, sizeof(Ctl)));
    if ((rc = build_corr())) return rc;
    any_spin_s = false;
    for (int c = 0; c < C; ++c) {
      any_spin_s |= spec[c].spin2 > 1;
    }
    bool any_sse = false, all_sse = true;
    for (auto& s : spec) { any_sse |= s.sse; all_sse &= s.sse; }
    if (any_sse && !all_sse)
      return lg_fail(LG_EINVAL, "an arena holds either path-integral or SSE chains, not both");
    sse = any_sse;
    if (!sse) {  // the pinned buffer of lg_load / lg_set_state, once per process (32 MiB: 670k operators)
      HostStage& hs = host_stage();
      std::lock_guard<std::mutex> lock(hs.m);
      hs.reserve(32u << 20);
    }
    if (sse) {
      if ((rc = setup_sse(res_vcap_for(1.0), false))) return rc;
    } else if (allow_resident && C >= nsm && res_fits(res_vcap_for(1.0), RES_SMEM_DEFAULT)) {
      // chain-resident by default from one chain per SM on (1024 64-site chains at beta = 10:
      // 0.21 against 0.33 ms per sweep); a few chains would leave most SMs idle while one CTA
      // walks each chain's serial phases, and the grid path spreads them over the GPU (a lone
      // such chain: 39 against 86 us).  The autotuner times both either way.
      if ((rc = setup_resident(res_vcap_for(1.0)))) return rc;
      shape = default_shape();
      shape.resident = 1;
    } else {
      if ((rc = setup_grid())) return rc;
    }
    // initial spins (one launch per distinct init mode)
    Arena A = arena();
    int random = spec.empty() ? 0 : spec[0].init_spins;
    k_init_spins<<<std::max(1, std::min((N + 255) / 256, nsm * 8)), 256, 0, st>>>(A, random);
    ++g_launches;
    LG_CUDA(cudaGetLastError());
    for (int c = 0; c < C; ++c)
      if (spec[c].init_spins != random) {
        std::vector<uint8_t> sp(spec[c].N);
        for (int i = 0; i < spec[c].N; ++i)
          sp[i] = spec[c].init_spins ? (uint8_t)(philox(spec[c].dchain.seed, 0xFFFFFFFFu, (uint32_t)i, TAG_SPIN, 0).x & 1u) : 0;
        LG_CUDA(lg_copy_async(d_spin0.p + hch[c].site_off, sp.data(), sp.size(), cudaMemcpyHostToDevice, st));
      }
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
  }

  // ---- the SSE form ----
  // Buffers for ocap operators per chain.  With keep, the current strings, counts and spins
  // survive (an overflow grows the capacity and replays the chunk).
  int setup_sse(int ocap, bool keep) {
    std::vector<uint32_t> ops;
    std::vector<int> nops;
    if (keep) {
      ops.resize((size_t)C * sse_ocap);
      nops.resize(C);
      LG_CUDA(lg_copy(ops.data(), sse_ops.p, ops.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
      LG_CUDA(lg_copy(nops.data(), sse_nop.p, C * sizeof(int), cudaMemcpyDeviceToHost));
    }
    int nmax = 0;
    for (auto& s : spec) nmax = std::max(nmax, s.N);
    const long long fc = (long long)nmax + ocap;
    if ((long long)C * fc * 8 > (1ll << 34))
      return lg_fail(LG_EBUDGET, "SSE arena too large (%d chains of %lld fragments)", C, fc);
    const int old_ocap = sse_ocap;
    sse_ocap = ocap;
    sse_fcap = (int)fc;
    const size_t oc = (size_t)C * ocap, fcn = (size_t)C * fc;
    int rc;
    if ((rc = sse_ops.alloc(oc)) || (rc = sse_ops_b.alloc(oc)) || (rc = sse_ops_t.alloc(oc)) ||
        (rc = sse_nop.alloc(C)) || (rc = sse_nop_b.alloc(C)) || (rc = sse_loops.alloc(2 * oc)) ||
        (rc = sse_frag.alloc(fcn)) || (rc = sse_est.alloc(8 * fcn)) || (rc = sse_wnd.alloc(3 * fcn)) ||
        (rc = sse_cur.alloc(N)) || (rc = sse_spc.alloc(N)) || (rc = sse_flip.alloc(fcn)) ||
        (rc = rb_spin0.alloc(N)) || (rc = d_rec.alloc((size_t)rec_rows * C * REC_WORDS)))
      return rc;
    if (keep) {
      std::vector<uint32_t> nw(oc, 0u);
      for (int c = 0; c < C; ++c)
        for (int i = 0; i < nops[c] && i < ocap; ++i) nw[(size_t)c * ocap + i] = ops[(size_t)c * old_ocap + i];
      LG_CUDA(lg_copy(sse_ops.p, nw.data(), oc * sizeof(uint32_t), cudaMemcpyHostToDevice));
      LG_CUDA(lg_copy(sse_nop.p, nops.data(), C * sizeof(int), cudaMemcpyHostToDevice));
    } else {
      LG_CUDA(cudaMemset(sse_nop.p, 0, C * sizeof(int)));
    }
    sse_grid = std::max(1, std::min((C + SSE_WARPS - 1) / SSE_WARPS, nsm * 16));
    return LG_OK;
  }

  // run() on the SSE form: chunks of up to rec_rows sweeps, one k_sse launch each; a chunk in
  // which a string outgrows its capacity is dropped and replayed after the capacity grows.
  int run_sse(long long n, float* ms, size_t flush_bytes) {
    DBuf<uint8_t> flushbuf;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
      if (flush_bytes) { int rc = flushbuf.alloc(flush_bytes); if (rc) return rc; }
      LG_CUDA(cudaEventCreate(&e0));
      LG_CUDA(cudaEventCreate(&e1));
    }
    struct EvG { cudaEvent_t a, b; ~EvG() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); } } eg{e0, e1};
    long long done_total = 0;
    while (n > 0) {
      const int m = (int)std::min<long long>(n, rec_rows);
      SseArgs S;
      S.m = m; S.ocap = sse_ocap; S.fcap = sse_fcap;
      S.spin_in = d_spin0.p; S.spin_out = rb_spin0.p;
      S.ops_in = sse_ops.p; S.ops_out = sse_ops_b.p; S.ops_tmp = sse_ops_t.p;
      S.nop_in = sse_nop.p; S.nop_out = sse_nop_b.p;
      S.loops = sse_loops.p; S.frag = sse_frag.p; S.est = sse_est.p; S.wnd = sse_wnd.p;
      S.cur = sse_cur.p; S.spc = sse_spc.p; S.flipf = sse_flip.p;
      if (ms) {
        if (flush_bytes) LG_CUDA(cudaMemsetAsync(flushbuf.p, (int)(done_total & 0xFF), flush_bytes, st));
        LG_CUDA(cudaEventRecord(e0, st));
      }
      k_sse<<<sse_grid, SSE_THREADS, 0, st>>>(arena(), S);
      ++g_launches;
      if (ms) LG_CUDA(cudaEventRecord(e1, st));
      LG_CUDA(cudaGetLastError());
      Ctl hc;
      LG_CUDA(lg_copy_async(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      LG_CUDA(cudaStreamSynchronize(st));
      if (hc.err) {
        std::vector<uint32_t> sw(C);
        for (int c = 0; c < C; ++c) sw[c] = (uint32_t)spec[c].mcs;
        LG_CUDA(lg_copy(d_sweep.p, sw.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice));
        Ctl z0 = hc;
        z0.err = 0;
        LG_CUDA(lg_copy(d_ctl.p, &z0, sizeof(Ctl), cudaMemcpyHostToDevice));
        if (hc.err == ERR_BOUNDARY)
          return lg_fail(LG_EINVAL, "spin-S configuration not periodic in imaginary time");
        if (hc.err != ERR_OVERFLOW) return lg_fail(LG_EDEVICE, "SSE sweep failed (%d)", hc.err);
        const long long o2 = std::min<long long>(1ll << 28, ((long long)sse_ocap * 3 / 2 + 63) & ~31ll);
        if (o2 <= sse_ocap) return lg_fail(LG_EBUDGET, "SSE operator string too long");
        int rc = setup_sse((int)o2, true);
        if (rc) return rc;
        continue;
      }
      d_spin0.swap(rb_spin0);
      sse_ops.swap(sse_ops_b);
      sse_nop.swap(sse_nop_b);
      hrec.resize((size_t)m * C * REC_WORDS);
      LG_CUDA(lg_copy(hrec.data(), d_rec.p, hrec.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      int rc = consume(m);
      if (rc) return rc;
      if (ms) {
        float t = 0;
        LG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        for (int i = 0; i < m; ++i) ms[done_total + i] = t / m;
      }
      done_total += m;
      n -= m;
    }
    return LG_OK;
  }

  // The SSE state of chain c: spins and the whole operator string (bond << 1 | off-diagonal).
  int sse_get(int c, std::vector<int32_t>& spins, std::vector<uint32_t>& ops) {
    const ChainSpec& s = spec[c];
    std::vector<uint8_t> sp(s.N);
    LG_CUDA(lg_copy(sp.data(), d_spin0.p + hch[c].site_off, s.N, cudaMemcpyDeviceToHost));
    spins.assign(sp.begin(), sp.end());
    int n = 0;
    LG_CUDA(lg_copy(&n, sse_nop.p + c, sizeof(int), cudaMemcpyDeviceToHost));
    ops.resize(n);
    if (n) LG_CUDA(lg_copy(ops.data(), sse_ops.p + (size_t)c * sse_ocap, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return LG_OK;
  }

  // Replace chain c's SSE state (checked first: bonds in range, and every site's spin periodic
  // through the string; for S > 1/2 every real site's number of up virtual spins).
  int sse_set(int c, const int32_t* spins, const std::vector<uint32_t>& ops, uint64_t sweep) {
    const ChainSpec& s = spec[c];
    std::vector<uint8_t> sp(s.N), cur(s.N);
    for (int i = 0; i < s.N; ++i) cur[i] = sp[i] = (uint8_t)(spins[i] & 1);
    for (size_t i = 0; i < ops.size(); ++i) {
      const uint32_t b = ops[i] >> 1;
      if ((int)b >= s.NB) return lg_fail(LG_EINVAL, "operator %zu out of range", i);
      if (ops[i] & 1u) { cur[s.s0[b]] ^= 1u; cur[s.s1[b]] ^= 1u; }
    }
    const int q = std::max(1, s.spin2);
    for (int i = 0; i < s.N; i += q) {
      int a = 0, b = 0;
      for (int k = 0; k < q; ++k) { a += cur[i + k]; b += sp[i + k]; }
      if (a != b) return lg_fail(LG_EINVAL, "site %d: the string is not periodic in imaginary time", i / q);
    }
    if ((long long)ops.size() > sse_ocap) {
      int rc = setup_sse((int)std::min<long long>(1ll << 28, ((long long)ops.size() * 3 / 2 + 63) & ~31ll), true);
      if (rc) return rc;
    }
    const int n = (int)ops.size();
    LG_CUDA(lg_copy(sse_nop.p + c, &n, sizeof(int), cudaMemcpyHostToDevice));
    if (n) LG_CUDA(lg_copy(sse_ops.p + (size_t)c * sse_ocap, ops.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_spin0.p + hch[c].site_off, sp.data(), s.N, cudaMemcpyHostToDevice));
    const uint32_t sw = (uint32_t)sweep;
    LG_CUDA(lg_copy(d_sweep.p + c, &sw, sizeof(uint32_t), cudaMemcpyHostToDevice));
    spec[c].mcs = sweep;
    return LG_OK;
  }

  // ---- grid path buffers: vertex regions, per-sweep arrays, merge staging, launch shape
  int setup_grid() {
    int rc;
    if ((rc = build_regions())) return rc;
    if ((rc = alloc_dynamic(region_total, false))) return rc;
    set_merge_cap();
    return set_shape(default_shape());
  }

  // ---- chain-resident sweeps ----
  // Vertex capacity per chain for a margin factor f: the largest expected operator count of the
  // arena's chains (ChainSpec::expected_vertices: 1.6 beta W N_b + 8 sqrt + 64) times f.
  int res_vcap_for(double f) const {
    double v = 0;
    for (auto& s : spec) v = std::max(v, s.expected_vertices());
    return (int)std::min(1e9, std::ceil(f * v / 32.0) * 32.0);
  }
  // Every chain qualifies (spin 1/2, no correlation measurement) and a chain of vcap vertices
  // fits in `limit` bytes of shared memory.
  bool res_fits(int vcap, size_t limit) const {
    if (n_corr_tiles || any_spin_s || C == 0 || zmax > 6) return false;
    int nmax = 0, nbmax = 0;
    for (auto& s : spec) { nmax = std::max(nmax, s.N); nbmax = std::max(nbmax, s.NB); }
    if ((long long)nmax + 2ll * vcap > (1ll << 24)) return false;
    return res_layout(nmax, nbmax, vcap).bytes + 256 <= limit;
  }
  // Buffers of the resident path for vertex capacity vcap per chain (the state arrays keep their
  // contents only through download_lists / upload_lists, which the callers do).
  int setup_resident(int vcap) {
    res_nmax = res_nbmax = 0;
    for (auto& s : spec) { res_nmax = std::max(res_nmax, s.N); res_nbmax = std::max(res_nbmax, s.NB); }
    res_vcap = vcap;
    res_lcap = 2 * vcap;
    res_scap = res_nmax + 2 * vcap;
    const ResLayout Ly = res_layout(res_nmax, res_nbmax, vcap);
    res_smem = Ly.bytes;
    const int z = merge_z(zmax);
    const void* fn = z == 2 ? (const void*)k_resident<2> : z == 4 ? (const void*)k_resident<4>
                                                                   : (const void*)k_resident<6>;
    LG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res_smem));
    int per_sm = 0;
    LG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, RES_THREADS, res_smem));
    if (per_sm < 1) return lg_fail(LG_EBUDGET, "chain-resident sweep does not fit an SM");
    res_grid = (int)std::min<long long>(C, (long long)nsm * per_sm);
    const size_t lt = (size_t)C * res_lcap, sc = (size_t)C * res_scap;
    int rc;
    if ((rc = d_stime.alloc(lt)) || (rc = d_sdir.alloc(lt)) || (rc = rb_stime.alloc(lt)) ||
        (rc = rb_sdir.alloc(lt)) || (rc = rb_spin0.alloc(N)) || (rc = rb_off_base.alloc(N)) ||
        (rc = rb_off_cnt.alloc(N)) || (rc = d_cls.alloc(4 * sc)) || (rc = d_rkw.alloc(sc)) ||
        (rc = d_rec.alloc((size_t)rec_rows * C * REC_WORDS)))
      return rc;
    LG_CUDA(cudaMemset(d_cls.p, 0, 4 * sc * sizeof(unsigned long long)));
    LG_CUDA(cudaMemset(d_rkw.p, 0, sc * sizeof(RootKW)));
    // the grid path's per-sweep arrays are not used here
    d_vtime.release(); d_vcode.release(); d_vslot.release(); d_sinfo.release(); d_svert.release();
    d_parent.release(); d_flip.release();
    drop_graph();
    resident = true;
    return LG_OK;
  }

  // Move the arena between the two paths, keeping its state (spins, off-diagonal lists, sweep
  // counters, accumulators): every result is the same on both.
  int to_grid() {
    if (!resident) return LG_OK;
    SiteLists L;
    int rc = download_lists(L);
    if (rc) return rc;
    rb_stime.release(); rb_sdir.release(); rb_spin0.release(); rb_off_base.release(); rb_off_cnt.release();
    resident = false;
    if ((rc = setup_grid())) return rc;
    return upload_lists(L);
  }
  int to_resident(size_t limit = RES_SMEM_MAX - 1024) {
    if (resident) return LG_OK;
    if (!res_fits(res_vcap_for(1.0), limit)) return lg_fail(LG_EUNSUPPORTED, "the arena's chains do not fit the chain-resident path");
    SiteLists L;
    int rc = download_lists(L);
    if (rc) return rc;
    if ((rc = setup_resident(res_vcap_for(1.0)))) return rc;
    return upload_lists(L);
  }

  // run() on the resident path: chunks of up to rec_rows sweeps, one k_resident launch each.
  // A chunk that fails leaves the state it started from in place: on an overflow the capacity
  // grows (or the arena moves to the grid path) and the chunk runs again with the same random
  // numbers, so capacity never changes a trajectory.
  int run_resident(long long n, float* ms, size_t flush_bytes) {
    DBuf<uint8_t> flushbuf;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
      if (flush_bytes) { int rc = flushbuf.alloc(flush_bytes); if (rc) return rc; }
      LG_CUDA(cudaEventCreate(&e0));
      LG_CUDA(cudaEventCreate(&e1));
    }
    struct EvG { cudaEvent_t a, b; ~EvG() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); } } eg{e0, e1};
    long long done_total = 0;
    while (n > 0) {
      if (!resident) {  // moved to the grid path by an overflow: the rest runs there
        return run(n, ms ? ms + done_total : nullptr, flush_bytes);
      }
      const int m = (int)std::min<long long>(n, rec_rows);
      ResArgs R;
      R.m = m; R.nmax = res_nmax; R.nbmax = res_nbmax; R.vcap = res_vcap; R.lcap = res_lcap;
      R.scap = res_scap;
      R.spin_in = d_spin0.p; R.obase_in = d_off_base.p; R.ocnt_in = d_off_cnt.p;
      R.st_in = d_stime.p; R.sd_in = d_sdir.p;
      R.spin_out = rb_spin0.p; R.obase_out = rb_off_base.p; R.ocnt_out = rb_off_cnt.p;
      R.st_out = rb_stime.p; R.sd_out = rb_sdir.p;
      Arena A = arena();
      if (ms) {
        if (flush_bytes) LG_CUDA(cudaMemsetAsync(flushbuf.p, (int)(done_total & 0xFF), flush_bytes, st));
        LG_CUDA(cudaEventRecord(e0, st));
      }
      const int z = merge_z(zmax);
      if (z == 2) k_resident<2><<<res_grid, RES_THREADS, res_smem, st>>>(A, R);
      else if (z == 4) k_resident<4><<<res_grid, RES_THREADS, res_smem, st>>>(A, R);
      else k_resident<6><<<res_grid, RES_THREADS, res_smem, st>>>(A, R);
      ++g_launches;
      if (ms) LG_CUDA(cudaEventRecord(e1, st));
      LG_CUDA(cudaGetLastError());
      Ctl hc;
      LG_CUDA(lg_copy_async(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      LG_CUDA(cudaStreamSynchronize(st));
      if (hc.err) {
        // the chunk is dropped: sweep counters back to the host's count
        std::vector<uint32_t> sw(C);
        for (int c = 0; c < C; ++c) sw[c] = (uint32_t)spec[c].mcs;
        LG_CUDA(lg_copy(d_sweep.p, sw.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice));
        if (hc.err == ERR_ITERCAP) {
          return lg_fail(LG_EITERCAP, "union-find iteration cap hit; the chain state is lost "
                                      "(load a checkpoint to continue)");
        }
        Ctl z0 = hc;
        z0.err = 0;
        LG_CUDA(lg_copy(d_ctl.p, &z0, sizeof(Ctl), cudaMemcpyHostToDevice));
        // overflow: more capacity, or the grid path when a CTA cannot hold it
        const int v2 = (int)std::min<long long>(1ll << 24, ((long long)res_vcap * 3 / 2 + 63) & ~31ll);
        SiteLists L;
        int rc = download_lists(L);
        if (rc) return rc;
        if (res_fits(v2, RES_SMEM_MAX - 1024)) {
          if ((rc = setup_resident(v2))) return rc;
        } else {
          rb_stime.release(); rb_sdir.release(); rb_spin0.release(); rb_off_base.release();
          rb_off_cnt.release();
          resident = false;
          shape.resident = 0;
          if ((rc = setup_grid())) return rc;
        }
        if ((rc = upload_lists(L))) return rc;
        continue;
      }
      d_spin0.swap(rb_spin0); d_off_base.swap(rb_off_base); d_off_cnt.swap(rb_off_cnt);
      d_stime.swap(rb_stime); d_sdir.swap(rb_sdir);
      hrec.resize((size_t)m * C * REC_WORDS);
      LG_CUDA(lg_copy(hrec.data(), d_rec.p, hrec.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      int rc = consume(m);
      if (rc) return rc;
      if (ms) {
        float t = 0;
        LG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        for (int i = 0; i < m; ++i) ms[done_total + i] = t / m;
      }
      done_total += m;
      n -= m;
    }
    return LG_OK;
  }

  // Spin correlation work (k_corr): one tile per CORR_THREADS entries of every chain that
  // measures correlations or the structure factor; zeroed sum arrays.
  int build_corr() {
    std::vector<int2> tiles;
    bool disp = false, orig = false;
    int maxn = 0;
    for (int c = 0; c < C; ++c) {
      const DChain& d = hch[c];
      if (!d.corr_disp && d.corr_origin < 0) continue;
      disp |= d.corr_disp != 0;
      orig |= d.corr_origin >= 0;
      maxn = std::max(maxn, d.nsites);
      for (int r0 = 0; r0 < d.nsites; r0 += CORR_THREADS) tiles.push_back(make_int2(c, r0));
    }
    n_corr_tiles = (int)tiles.size();
    corr_smem = maxn <= CORR_SMEM ? maxn : 0;
    if (!n_corr_tiles) return LG_OK;
    int rc;
    if ((rc = d_corr_tiles.alloc(tiles.size())) || (rc = d_corr_disp.alloc(disp ? N : 0)) ||
        (rc = d_corr_origin.alloc(orig ? N : 0)))
      return rc;
    LG_CUDA(lg_copy(d_corr_tiles.p, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
    if (disp) LG_CUDA(cudaMemset(d_corr_disp.p, 0, (size_t)N * sizeof(long long)));
    if (orig) LG_CUDA(cudaMemset(d_corr_origin.p, 0, (size_t)N * sizeof(long long)));
    if (!disp) d_corr_disp.n = 0;
    if (!orig) d_corr_origin.n = 0;
    return LG_OK;
  }

  // Vertex regions: each chain's sites in runs of S consecutive sites, S chosen so that a region
  // expects about 4096 vertices; a region's capacity is 1.3 times its expectation plus slack.
  int build_regions() {
    h_site_region.assign(N, 0);
    h_region_cap.clear();
    for (int c = 0; c < C; ++c) {
      const int n = spec[c].N;
      const double per_site = n ? spec[c].expected_vertices() / n : 0.0;
      int S = per_site > 0 ? (int)std::ceil(4096.0 / per_site) : 1024;
      S = std::min(std::max(S, 8), 1024);
      for (int i0 = 0; i0 < n; i0 += S) {
        const int m = std::min(S, n - i0);
        const double e = per_site * m;
        long long cap = (long long)std::ceil(1.3 * e + 8.0 * std::sqrt(e)) + 32;
        cap = (cap + 7) & ~7ll;
        for (int i = 0; i < m; ++i) h_site_region[hch[c].site_off + i0 + i] = (int)h_region_cap.size();
        h_region_cap.push_back(cap);
      }
    }
    R = (int)h_region_cap.size();
    int rc;
    if ((rc = d_site_region.alloc(N)) || (rc = d_region_fill.alloc(R))) return rc;
    LG_CUDA(lg_copy(d_site_region.p, h_site_region.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    return layout_regions();
  }

  // Region slot ranges from the capacities.
  int layout_regions() {
    std::vector<int> base(R + 1, 0);
    long long tot = 0;
    for (int r = 0; r < R; ++r) {
      base[r] = (int)tot;
      tot += h_region_cap[r];
      if (tot > (1ll << 30) - N) return lg_fail(LG_EBUDGET, "vertex capacity %lld too large", tot);
    }
    base[R] = (int)tot;
    region_total = tot;
    int rc = d_region_base.alloc(R + 1);
    if (rc) return rc;
    LG_CUDA(lg_copy(d_region_base.p, base.data(), (R + 1) * sizeof(int), cudaMemcpyHostToDevice));
    drop_graph();
    return LG_OK;
  }

  // A sweep starts with its record row and the region claim counters at zero; k_end leaves them
  // so for the next sweep.  This sets them up for the record row the host resets the counter to
  // (row 0), after a chunk, a failed sweep or a reallocation.
  int clear_sweep_state() {
    if (d_rec.p) LG_CUDA(cudaMemsetAsync(d_rec.p, 0, (size_t)C * REC_WORDS * sizeof(unsigned long long), st));
    if (R) LG_CUDA(cudaMemsetAsync(d_region_fill.p, 0, (size_t)R * sizeof(unsigned long long), st));
    return LG_OK;
  }

  // After an overflowing sweep: grow every region whose demand passed its capacity.
  int grow_regions() {
    std::vector<unsigned long long> fill(R);
    LG_CUDA(lg_copy(fill.data(), d_region_fill.p, R * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    bool grew = false;
    for (int r = 0; r < R; ++r) {
      if ((long long)fill[r] <= h_region_cap[r]) continue;
      const long long need = (long long)std::min<unsigned long long>(fill[r], 1ull << 40);
      h_region_cap[r] = ((long long)(1.25 * need) + 64 + 7) & ~7ll;
      grew = true;
    }
    if (!grew)  // no region reported a shortage: grow them all, so that the replay progresses
      for (auto& c : h_region_cap) c = ((long long)(1.25 * c) + 64 + 7) & ~7ll;
    int rc = layout_regions();
    if (rc) return rc;
    return alloc_dynamic(region_total, true);
  }

  // (Re)allocate the per-sweep buffers for cap vertices (at least the regions' total); with keep,
  // preserve the persistent off-diagonal lists that live at the front of each site's segment
  // range.
  int alloc_dynamic(long long cap, bool keep) {
    cap = std::max(cap, region_total);
    if (cap > (1ll << 30) - N) return lg_fail(LG_EBUDGET, "vertex capacity %lld too large", cap);
    int new_nv = (int)cap;
    int new_ns = 2 * new_nv + N;
    DBuf<uint64_t> old_t;
    DBuf<uint8_t> old_d;
    size_t keep_n = 0;
    if (keep) {
      std::swap(old_t.p, d_stime.p); std::swap(old_t.n, d_stime.n);
      std::swap(old_d.p, d_sdir.p); std::swap(old_d.n, d_sdir.n);
      keep_n = (size_t)ns_cap;
    }
    int rc;
    if ((rc = d_vtime.alloc(new_nv)) || (rc = d_vcode.alloc(new_nv)) ||
        (rc = d_vslot.alloc(2 * (size_t)new_nv)) || (rc = d_stime.alloc(new_ns)) ||
        (rc = d_sinfo.alloc(new_ns)) || (rc = d_svert.alloc(new_ns)) || (rc = d_sdir.alloc(new_ns)) ||
        (rc = d_parent.alloc(new_ns)) || (rc = d_flip.alloc(new_ns)) ||
        (rc = d_cls.alloc(4 * (size_t)new_ns)) || (rc = d_rkw.alloc((size_t)new_ns)) ||
        (rc = d_rec.alloc((size_t)rec_rows * C * REC_WORDS)))
      return rc;
    // cluster class sums must start at zero (k_cluster clears what it consumes)
    LG_CUDA(cudaMemset(d_cls.p, 0, 4 * (size_t)new_ns * sizeof(unsigned long long)));
    LG_CUDA(cudaMemset(d_rkw.p, 0, (size_t)new_ns * sizeof(RootKW)));
    if (keep) {
      LG_CUDA(lg_copy(d_stime.p, old_t.p, keep_n * sizeof(uint64_t), cudaMemcpyDeviceToDevice));
      LG_CUDA(lg_copy(d_sdir.p, old_d.p, keep_n, cudaMemcpyDeviceToDevice));
    }
    nv_cap = new_nv;
    ns_cap = new_ns;
    if ((rc = clear_sweep_state())) return rc;
    Ctl hc;
    LG_CUDA(lg_copy(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost));
    hc.nv_cap = nv_cap; hc.ns_cap = ns_cap;
    LG_CUDA(lg_copy(d_ctl.p, &hc, sizeof(Ctl), cudaMemcpyHostToDevice));
    drop_graph();
    return LG_OK;
  }

  // Starting shape before any tuning.  An arena of few sites is latency-bound: a warp per site
  // gives the shortest critical path there, whatever the temperature.  A large arena fills the
  // GPU either way, and its low-temperature-density chains do better with a thread per bond or
  // site (thresholds from autotuning the 512-chain mixed arena).  Tiles shrink until the grid
  // has at least two blocks per SM.
  Shape default_shape() const {
    Shape s;
    if (N < 131072) {
      s.insert_k = 0.0;
      s.narrow_k = 0.0;
    } else {
      s.insert_k = 64.0;
      s.narrow_k = 16.0;
    }
    const long long goal = 2ll * nsm;
    s.acc_tile = ns_cap / 2048 >= goal ? 2048 : (ns_cap / 1024 >= goal ? 1024 : 512);
    s.cl_tile = ns_cap / 4096 >= goal ? 4096 : 2048;
    s.un_warps = 8;
    return s;
  }

  // k_merge stages a site's endpoints in shared memory up to merge_cap of them (larger sites take
  // the one-thread merge).  The capacity follows the arena's largest expected endpoint count per
  // site with a wide margin, so that small arenas keep k_merge's shared memory (and so its
  // occupancy) small.
  void set_merge_cap() {
    double mu = 0;
    for (int c = 0; c < C; ++c) mu = std::max(mu, endpoints_per_site(c));
    int cap = (int)std::ceil(1.6 * mu + 6.0 * std::sqrt(mu) + 32.0);
    cap = (cap + 31) & ~31;
    merge_cap = std::min(std::max(cap, 64), MERGE_CAP);
    drop_graph();
  }

  // Expected endpoints per site of chain c: the narrow / wide criterion.
  double endpoints_per_site(int c) const {
    const ChainSpec& s = spec[c];
    return s.N ? 2.0 * s.beta * s.W * s.NB / s.N : 0.0;
  }

  // Adopt a launch shape: classify chains as narrow or wide and upload the class lists.
  int set_shape(const Shape& sh) {
    if (sse) { shape = sh; return LG_OK; }  // the SSE form has no launch shape
    if (!(sh.acc_tile == 512 || sh.acc_tile == 1024 || sh.acc_tile == 2048) ||
        !(sh.cl_tile == 2048 || sh.cl_tile == 4096 || sh.cl_tile == 8192) ||
        !(sh.un_warps == 4 || sh.un_warps == 8 || sh.un_warps == 16) || !(sh.narrow_k >= 0) ||
        !(sh.insert_k >= 0) || !(sh.resident == 0 || sh.resident == 1) ||
        !(sh.union_mode >= 0 && sh.union_mode <= 2))
      return lg_fail(LG_EINVAL, "bad launch shape");
    if (sh.resident && !resident) {
      int rc = to_resident();
      if (rc) return rc;
    } else if (!sh.resident && resident) {
      int rc = to_grid();
      if (rc) return rc;
    }
    if (resident) {  // the grid fields are kept for when the arena returns to the grid path
      shape = sh;
      return LG_OK;
    }
    std::vector<int> ws, nsl, is, nbl;
    for (int c = 0; c < C; ++c) {
      const double mu = endpoints_per_site(c);
      const bool narrow = mu < sh.narrow_k, narrow_ins = mu < sh.insert_k;
      for (int i = 0; i < spec[c].N; ++i) {
        (narrow ? nsl : ws).push_back(hch[c].site_off + i);
        if (!narrow_ins) is.push_back(hch[c].site_off + i);
      }
      if (narrow_ins)
        for (int b = 0; b < spec[c].NB; ++b) nbl.push_back(hch[c].bond_off + b);
    }
    int rc;
    auto upload = [&](DBuf<int>& d, const std::vector<int>& h) -> int {
      int r = d.alloc(std::max<size_t>(h.size(), 1));
      if (r) return r;
      if (!h.empty())
        LG_CUDA(lg_copy(d.p, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
      return LG_OK;
    };
    n_wide = (int)ws.size();
    n_narrow = (int)nsl.size();
    n_ins = (int)is.size();
    n_narrow_b = (int)nbl.size();
    // a list covering every site in order is passed as nullptr (no indirection)
    wide_list = nullptr;
    ins_list = nullptr;
    if (n_wide > 0 && n_wide < N) {
      if ((rc = upload(d_wide_sites, ws))) return rc;
      wide_list = d_wide_sites.p;
    }
    if (n_ins > 0 && n_ins < N) {
      if ((rc = upload(d_ins_sites, is))) return rc;
      ins_list = d_ins_sites.p;
    }
    if ((rc = upload(d_narrow_sites, nsl)) || (rc = upload(d_narrow_bonds, nbl))) return rc;
    shape = sh;
    drop_graph();
    return LG_OK;
  }

  void drop_graph() {
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
  }

  int grid_for(long long n, int threads, int per_sm = 8) {
    long long g = (n + threads - 1) / threads;
    long long m = (long long)nsm * per_sm;
    if (g > m) g = m;
    if (g < 1) g = 1;
    return (int)g;
  }

  // Three-kernel exclusive scan on the engine's stream (launches are counted by the caller).
  void scan(const int* in, int* out, int n, int* total, int cap, int per_item, int extra,
            cudaEvent_t* ev = nullptr) {
    int parts = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (parts < 1) parts = 1;
    k_scan_reduce<<<parts, SCAN_THREADS, 0, st>>>(in, n, d_partial.p, d_ctl.p);
    k_scan_partials<<<1, 1024, 0, st>>>(d_partial.p, parts, total, cap, per_item, extra, d_ctl.p);
    k_scan_apply<<<parts, SCAN_THREADS, 0, st>>>(in, out, n, d_partial.p, d_ctl.p);
    if (ev) cudaEventRecord(*ev, st);
  }

  // The sweep of every chain, as a fixed sequence of launches (capturable).  With ev != nullptr
  // an event is recorded after each stage (kNumStages events) for per-kernel timing.  When an
  // arena has both narrow and wide chains, the narrow kernels of a stage run on a second stream
  // beside the wide ones (a fork and a join in the captured graph).
  void enqueue_sweep(cudaEvent_t* ev = nullptr) {
    Arena A = arena();
    int launches = 0;
    auto mark = [&](int k) {
      if (ev) cudaEventRecord(ev[k], st);
      if (val_bad && !capturing && (k == 0 || k == 2 || k == 4 || k == 6))
        k_validate<<<grid_for(std::max(std::max(NB, N), ns_cap), 256, 16), 256, 0, st>>>(arena(), k, val_bad);
    };
    bool both = false;
    auto fork = [&](bool b) { both = b; if (b) { cudaEventRecord(ev_fork, st); cudaStreamWaitEvent(st2, ev_fork, 0); } };
    auto join = [&]() { if (both) { cudaEventRecord(ev_join, st2); cudaStreamWaitEvent(st, ev_join, 0); } };
    fork(n_ins > 0 && n_narrow_b > 0);
    if (n_ins) {
      k_insert<<<grid_for((long long)n_ins * 32, INS_WARPS * 32, 16), INS_WARPS * 32, 0, st>>>(A, ins_list, n_ins);
      ++launches;
    }
    if (n_narrow_b) {
      k_insert_narrow<<<grid_for(n_narrow_b, 256, 16), 256, 0, both ? st2 : st>>>(A, d_narrow_bonds.p, n_narrow_b);
      ++launches;
    }
    join();
    mark(0);
    if (N <= SITE_SCAN_MAX) {
      const int g = (N + SITE_SCAN_BLOCK - 1) / SITE_SCAN_BLOCK;
      k_site_blocks<<<g, SITE_SCAN_BLOCK, 0, st>>>(A, d_partial.p);
      k_site_offsets<<<g, SITE_SCAN_BLOCK, 0, st>>>(A, d_partial.p);
      launches += 2;
    } else {
      k_site_count<<<grid_for(N, 256, 16), 256, 0, st>>>(A);
      scan(d_site_cnt.p, d_sbase.p, N, &d_ctl.p->ns_total, ns_cap, 1, 0);
      launches += 4;
    }
    mark(1);
    fork(n_wide > 0 && n_narrow > 0);
    if (n_wide) {
      launch_merge(zmax, grid_for((long long)n_wide * 32, MERGE_WARPS * 32, 16),
                   MERGE_WARPS * merge_smem_per_warp(merge_cap), st, A, wide_list, n_wide, merge_cap);
      ++launches;
    }
    if (n_narrow) {
      launch_merge_narrow(zmax, grid_for(n_narrow, 256, 16), both ? st2 : st, A, d_narrow_sites.p, n_narrow);
      ++launches;
    }
    join();
    if (any_spin_s) {
      k_boundary<<<grid_for(N, 256, 16), 256, 0, st>>>(A);
      ++launches;
    }
    mark(2);
    {
      const int w = shape.un_warps, per = w * UN_CHUNK;
      const int g = (ns_cap + per - 1) / per;  // one chunk per warp: no straggler tail
      const bool pairs = shape.union_mode >= 1 && !any_spin_s;
      if (pairs) {
        k_union_pairs<<<grid_for((ns_cap + UP_PER - 1) / UP_PER, 256, 16), 256, 0, st>>>(A);
        ++launches;
      }
      if (shape.union_mode == 2) {
        // persistent: at most eight CTAs per SM, no more warps than chunks
        const int gb = (int)std::max<long long>(1, std::min<long long>(
            (long long)nsm * 8, ((long long)ns_cap + UB_WARPS * UN_CHUNK - 1) / (UB_WARPS * UN_CHUNK)));
        if (pairs) k_union_bal<true><<<gb, UB_WARPS * 32, 0, st>>>(A);
        else k_union_bal<false><<<gb, UB_WARPS * 32, 0, st>>>(A);
      } else if (pairs) {
        if (w == 4) k_union<4, true><<<g, 4 * 32, 0, st>>>(A);
        else if (w == 16) k_union<16, true><<<g, 16 * 32, 0, st>>>(A);
        else k_union<8, true><<<g, 8 * 32, 0, st>>>(A);
      } else {
        if (w == 4) k_union<4><<<g, 4 * 32, 0, st>>>(A);
        else if (w == 16) k_union<16><<<g, 16 * 32, 0, st>>>(A);
        else k_union<8><<<g, 8 * 32, 0, st>>>(A);
      }
    }
    mark(3);
    {
      const int t = shape.acc_tile, g = (ns_cap + t - 1) / t;  // one tile per block
      if (t == 512) k_accumulate<512><<<g, 256, 0, st>>>(A);
      else if (t == 2048) k_accumulate<2048><<<g, 256, 0, st>>>(A);
      else k_accumulate<1024><<<g, 256, 0, st>>>(A);
    }
    mark(4);
    launches += 2;
    {
      const int t = shape.cl_tile, g = (ns_cap + t - 1) / t;  // one tile per block
      if (t == 2048) k_cluster<2048><<<g, CL_THREADS, 0, st>>>(A);
      else if (t == 8192) k_cluster<8192><<<g, CL_THREADS, 0, st>>>(A);
      else k_cluster<4096><<<g, CL_THREADS, 0, st>>>(A);
    }
    mark(5);
    launches += 1;
    // k_end (counters, the next record row, claim counters) needs nothing of the site pass, so
    // it runs beside it on a third stream; k_corr reads the sweep counter before k_end advances
    // it, so with correlations the order stays sequential
    const bool end_beside = n_corr_tiles == 0;
    if (end_beside) {
      cudaEventRecord(ev_fork3, st);
      cudaStreamWaitEvent(st3, ev_fork3, 0);
      k_end<<<1, 1024, 0, st3>>>(A);
    }
    fork(n_wide > 0 && n_narrow > 0);
    if (n_wide) {
      k_site_end<<<grid_for((long long)n_wide * 32, 256, 16), 256, 0, st>>>(A, wide_list, n_wide);
      ++launches;
    }
    if (n_narrow) {
      k_site_end_narrow<<<grid_for(n_narrow, 256, 16), 256, 0, both ? st2 : st>>>(A, d_narrow_sites.p, n_narrow);
      ++launches;
    }
    join();
    if (n_corr_tiles) {
      k_corr<<<n_corr_tiles, CORR_THREADS, corr_smem, st>>>(A);
      ++launches;
    }
    if (end_beside) {
      cudaEventRecord(ev_join3, st3);
      cudaStreamWaitEvent(st, ev_join3, 0);
    } else {
      k_end<<<1, 1024, 0, st>>>(A);
    }
    mark(6);
    launches += 1;
    sweep_launches = launches;
    g_launches += launches;
  }

  int ensure_graph() {
    if (!use_graph || gexec) return LG_OK;
    LG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    uint64_t before = g_launches.load();
    capturing = true;
    enqueue_sweep();
    capturing = false;
    g_launches = before;  // counted when the graph is launched
    LG_CUDA(cudaStreamEndCapture(st, &graph));
    LG_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
    return LG_OK;
  }

  // Run n sweeps of every chain.  With ms != nullptr every sweep is bracketed by events and
  // preceded by an L2 flush of flush_bytes (outside the brackets).
  int run(long long n, float* ms = nullptr, size_t flush_bytes = 0) {
    if (sse) return run_sse(n, ms, flush_bytes);
    if (resident) return run_resident(n, ms, flush_bytes);
    DBuf<uint8_t> flushbuf;
    std::vector<cudaEvent_t> ev;
    if (ms) {
      if (flush_bytes) { int rc = flushbuf.alloc(flush_bytes); if (rc) return rc; }
      ev.resize(2 * rec_rows);
      for (auto& e : ev) LG_CUDA(cudaEventCreate(&e));
    }
    struct EvGuard { std::vector<cudaEvent_t>& v; ~EvGuard() { for (auto e : v) cudaEventDestroy(e); } } guard{ev};
    long long done_total = 0;
    while (n > 0) {
      int m = (int)std::min<long long>(n, rec_rows);
      int rc = ensure_graph();
      if (rc) return rc;
      for (int i = 0; i < m; ++i) {
        if (ms) {
          if (flush_bytes) LG_CUDA(cudaMemsetAsync(flushbuf.p, i & 0xFF, flush_bytes, st));
          LG_CUDA(cudaEventRecord(ev[2 * i], st));
        }
        if (gexec) {
          LG_CUDA(cudaGraphLaunch(gexec, st));
          g_launches += sweep_launches;
        } else {
          enqueue_sweep();
        }
        if (ms) LG_CUDA(cudaEventRecord(ev[2 * i + 1], st));
      }
      LG_CUDA(cudaGetLastError());
      Ctl hc;
      LG_CUDA(lg_copy_async(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      LG_CUDA(cudaStreamSynchronize(st));
      int done = (int)hc.step;
      if (done > 0) {
        hrec.resize((size_t)done * C * REC_WORDS);
        LG_CUDA(lg_copy(hrec.data(), d_rec.p, hrec.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        if ((rc = consume(done))) return rc;
        if (ms)
          for (int i = 0; i < done; ++i)
            LG_CUDA(cudaEventElapsedTime(&ms[done_total + i], ev[2 * i], ev[2 * i + 1]));
      }
      done_total += done;
      Ctl z = hc;
      z.step = 0;
      z.err = 0;
      if (hc.err == ERR_ITERCAP) {
        // the sweep stopped after the merge had overwritten the persistent operator lists, so
        // the arena's state is lost: the error stays set (every later run reports it) until a
        // checkpoint is loaded (set_state on a single-chain engine)
        Ctl zk = hc;
        zk.step = 0;
        LG_CUDA(lg_copy(d_ctl.p, &zk, sizeof(Ctl), cudaMemcpyHostToDevice));
        clear_sweep_state();
        return lg_fail(LG_EITERCAP, "union-find iteration cap hit; the chain state is lost "
                                    "(load a checkpoint to continue)");
      }
      if (hc.err == ERR_BOUNDARY) {
        LG_CUDA(lg_copy(d_ctl.p, &z, sizeof(Ctl), cudaMemcpyHostToDevice));
        clear_sweep_state();
        return lg_fail(LG_EINVAL, "spin-S configuration not periodic in imaginary time");
      }
      if (hc.err == ERR_OVERFLOW) {
        LG_CUDA(lg_copy(d_ctl.p, &z, sizeof(Ctl), cudaMemcpyHostToDevice));
        rc = grow_regions();
        if (rc) return rc;
      } else {
        LG_CUDA(lg_copy(d_ctl.p, &z, sizeof(Ctl), cudaMemcpyHostToDevice));
      }
      if ((rc = clear_sweep_state())) return rc;
      n -= done;
    }
    return LG_OK;
  }

  // n sweeps launched kernel by kernel with events between stages (no graph).
  int profile(long long n, size_t flush_bytes, double* kernel_ms, long long* vertices) {
    if (sse) return lg_fail(LG_EUNSUPPORTED, "the per-kernel profile is a path-integral measurement");
    if (resident) {  // the per-kernel profile is a grid-path measurement
      int rc = to_grid();
      if (rc) return rc;
      shape.resident = 0;
    }
    DBuf<uint8_t> flushbuf;
    if (flush_bytes) { int rc = flushbuf.alloc(flush_bytes); if (rc) return rc; }
    cudaEvent_t ev[kNumStages + 1];
    for (auto& e : ev) LG_CUDA(cudaEventCreate(&e));
    struct G { cudaEvent_t* e; ~G() { for (int i = 0; i <= kNumStages; ++i) cudaEventDestroy(e[i]); } } g{ev};
    for (int k = 0; k < kNumStages; ++k) kernel_ms[k] = 0;
    long long verts = 0;
    while (n > 0) {
      if (flush_bytes) LG_CUDA(cudaMemsetAsync(flushbuf.p, (int)(n & 0xFF), flush_bytes, st));
      LG_CUDA(cudaEventRecord(ev[kNumStages], st));
      enqueue_sweep(ev);
      LG_CUDA(cudaGetLastError());
      Ctl hc;
      LG_CUDA(lg_copy_async(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      LG_CUDA(cudaStreamSynchronize(st));
      if (hc.err) {
        long long left = n;
        int rc = run(1);  // resolves an overflow (grows, replays) like lg_run
        if (rc) return rc;
        n = left - 1;
        continue;
      }
      float t;
      LG_CUDA(cudaEventElapsedTime(&t, ev[kNumStages], ev[0]));
      kernel_ms[0] += t;
      for (int k = 1; k < kNumStages; ++k) {
        LG_CUDA(cudaEventElapsedTime(&t, ev[k - 1], ev[k]));
        kernel_ms[k] += t;
      }
      verts += (hc.ns_total - N) / 2;  // every vertex adds a segment at each of its two sites
      hrec.resize((size_t)C * REC_WORDS);
      LG_CUDA(lg_copy(hrec.data(), d_rec.p, hrec.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      if (int rc = consume(1)) return rc;
      Ctl z = hc;
      z.step = 0;
      LG_CUDA(lg_copy(d_ctl.p, &z, sizeof(Ctl), cudaMemcpyHostToDevice));
      if (int rc = clear_sweep_state()) return rc;
      --n;
    }
    *vertices = verts;
    return LG_OK;
  }

  // Launch-shape autotuner.  Each candidate shape is timed over `trial` sweeps (per-stage events,
  // L2 flushed before each sweep); the candidates are searched one coordinate at a time, starting
  // with the narrow / wide split, and the fastest shape is kept.  The timed sweeps are the
  // chains' own sweeps: no shape changes a result, so tuning costs no extra sweeps.
  int autotune(int trial, size_t flush_bytes, std::string& report) {
    if (sse) {  // one chain per warp: nothing to choose
      report = "chosen: SSE form (one chain per warp)\n";
      return run(trial);
    }
    if (trial < 1) trial = 1;
    char line[224];
    report.clear();
    // the chain-resident path, where the arena qualifies: timed first, over whole chunks
    const int trial2 = std::max(trial, 8);
    double res_ms = -1;
    const bool can_res = allow_resident && res_fits(res_vcap_for(1.0), RES_SMEM_DEFAULT);
    if (can_res) {
      Shape r = shape;
      r.resident = 1;
      int rc = set_shape(r);
      if (rc) return rc;
      std::vector<float> t(trial2);
      if ((rc = run(1))) return rc;
      if ((rc = run(trial2, t.data(), flush_bytes))) return rc;
      if (resident) {
        res_ms = 0;
        for (float x : t) res_ms += x;
        res_ms /= trial2;
        std::snprintf(line, sizeof(line), "resident (one CTA per chain, %d sweeps per launch): %.4f ms\n",
                      trial2, res_ms);
        report += line;
      }
      Shape g = shape;
      g.resident = 0;
      if ((rc = set_shape(g))) return rc;
    }
    auto time_shape = [&](const Shape& sh, double* ms) -> int {
      int rc = set_shape(sh);
      if (rc) return rc;
      std::vector<double> km(kNumStages);
      long long v = 0;
      if ((rc = profile(1, flush_bytes, km.data(), &v))) return rc;  // first launches: untimed
      if ((rc = profile(trial, flush_bytes, km.data(), &v))) return rc;
      double t = 0;
      for (double x : km) t += x;
      *ms = t / trial;
      std::snprintf(line, sizeof(line), "insert_k=%g narrow_k=%g acc_tile=%d cl_tile=%d union_warps=%d union_mode=%d: %.4f ms\n",
                    sh.insert_k, sh.narrow_k, sh.acc_tile, sh.cl_tile, sh.un_warps, sh.union_mode, *ms);
      report += line;
      return LG_OK;
    };
    Shape best = shape;
    double best_ms = 0;
    int rc = time_shape(best, &best_ms);
    if (rc) return rc;
    // a candidate must beat the kept shape by 2%, so that timing noise does not move the shape
    auto consider = [&](Shape cand) -> int {
      double ms = 0;
      int r = time_shape(cand, &ms);
      if (r) return r;
      if (ms < 0.98 * best_ms) { best_ms = ms; best = cand; }
      return LG_OK;
    };
    // narrow / wide split: one candidate per distinct set of narrow chains
    std::vector<double> mu(C);
    for (int c = 0; c < C; ++c) mu[c] = endpoints_per_site(c);
    std::vector<int> seen;
    auto n_below = [&](double k) { int n = 0; for (double m : mu) n += m < k; return n; };
    const double ks[] = {0.0, 4.0, 8.0, 16.0, 32.0, 64.0, 128.0, 256.0, 1e300};
    seen.push_back(n_below(best.narrow_k));
    for (double k : ks) {
      const int nb = n_below(k);
      if (std::find(seen.begin(), seen.end(), nb) != seen.end()) continue;
      seen.push_back(nb);
      Shape c = best;
      c.narrow_k = k;
      if ((rc = consider(c))) return rc;
    }
    seen.assign(1, n_below(best.insert_k));
    for (double k : ks) {
      const int nb = n_below(k);
      if (std::find(seen.begin(), seen.end(), nb) != seen.end()) continue;
      seen.push_back(nb);
      Shape c = best;
      c.insert_k = k;
      if ((rc = consider(c))) return rc;
    }
    for (int t : {512, 1024, 2048}) {
      if (t == best.acc_tile) continue;
      Shape c = best; c.acc_tile = t;
      if ((rc = consider(c))) return rc;
    }
    for (int t : {2048, 4096, 8192}) {
      if (t == best.cl_tile) continue;
      Shape c = best; c.cl_tile = t;
      if ((rc = consider(c))) return rc;
    }
    for (int w : {4, 8, 16}) {
      if (w == best.un_warps) continue;
      Shape c = best; c.un_warps = w;
      if ((rc = consider(c))) return rc;
    }
    for (int m : {0, 1, 2}) {
      if (m == best.union_mode || (m == 1 && any_spin_s)) continue;
      Shape c = best; c.union_mode = m;
      if ((rc = consider(c))) return rc;
    }
    if ((rc = set_shape(best))) return rc;
    if (res_ms > 0) {
      // the best grid shape timed as it runs (CUDA graph), against the resident time
      std::vector<float> t(trial2);
      if ((rc = run(trial2, t.data(), flush_bytes))) return rc;
      double g = 0;
      for (float x : t) g += x;
      g /= trial2;
      std::snprintf(line, sizeof(line), "grid (CUDA graph, best shape): %.4f ms\n", g);
      report += line;
      if (res_ms < 0.98 * g) {
        best.resident = 1;
        best_ms = res_ms;
      }
    }
    std::snprintf(line, sizeof(line), "chosen: %sinsert_k=%g narrow_k=%g acc_tile=%d cl_tile=%d union_warps=%d union_mode=%d (%.4f ms)\n",
                  best.resident ? "resident; " : "", best.insert_k, best.narrow_k, best.acc_tile,
                  best.cl_tile, best.un_warps, best.union_mode, best_ms);
    report += line;
    return set_shape(best);
  }

  // Host side of a finished chunk of `rows` sweeps: records into the accumulators, then the
  // chunk's correlation sums (k_corr adds only measurement sweeps) into the vector accumulators.
  int consume(int rows) {
    std::vector<int64_t> measured(n_corr_tiles ? C : 0, 0);
    for (int r = 0; r < rows; ++r) {
      for (int c = 0; c < C; ++c) {
        const uint64_t* rec = hrec.data() + ((size_t)r * C + c) * REC_WORDS;
        ChainSpec& s = spec[c];
        if (keep_records && c == 0) kept.insert(kept.end(), rec, rec + REC_WORDS);
        s.last_nop = rec[R_NOP];
        if (s.mcs >= (uint64_t)s.therm && s.mcs < (uint64_t)(s.therm + s.sweeps)) {
          acc[acc_of_chain[c]].push(s, rec);
          if (keep_vals[c]) {
            const size_t o = vals[c].size();
            vals[c].resize(o + LG_NUM_VALUES);
            record_scalars(s, rec, vals[c].data() + o);
          }
          if (n_corr_tiles) ++measured[c];
        }
        ++s.mcs;
      }
    }
    if (!n_corr_tiles) return LG_OK;
    bool any = false;
    for (int64_t m : measured) any |= m > 0;
    if (!any) return LG_OK;
    for (int which = 0; which < 2; ++which) {
      DBuf<long long>& d = which ? d_corr_origin : d_corr_disp;
      if (!d.n) continue;
      h_corr.resize(N);
      LG_CUDA(lg_copy(h_corr.data(), d.p, (size_t)N * sizeof(long long), cudaMemcpyDeviceToHost));
      LG_CUDA(cudaMemsetAsync(d.p, 0, (size_t)N * sizeof(long long), st));
      for (int c = 0; c < C; ++c) {
        const bool on = which ? hch[c].corr_origin >= 0 : hch[c].corr_disp != 0;
        if (!on || !measured[c]) continue;
        ChainAcc& a = acc[acc_of_chain[c]];
        (which ? a.corr_origin : a.corr_disp)
            .add_chunk(reinterpret_cast<const int64_t*>(h_corr.data()) + hch[c].site_off, hch[c].nsites,
                       measured[c]);
      }
    }
    return LG_OK;
  }

  // ---- state access (test seams, checkpoints) ----
  int get_state(int c, std::vector<int32_t>& spins, std::vector<int32_t>& bonds,
                std::vector<double>& times) {
    if (sse) {  // the off-diagonal operators, with (index + 1/2) / n as their time (the order)
      std::vector<uint32_t> ops;
      int rc = sse_get(c, spins, ops);
      if (rc) return rc;
      bonds.clear(); times.clear();
      for (size_t i = 0; i < ops.size(); ++i)
        if (ops[i] & 1u) { bonds.push_back((int32_t)(ops[i] >> 1)); times.push_back((i + 0.5) / ops.size()); }
      return LG_OK;
    }
    const ChainSpec& s = spec[c];
    int so = hch[c].site_off;
    std::vector<uint8_t> sp(s.N);
    std::vector<int> ob(s.N), oc(s.N);
    LG_CUDA(lg_copy(sp.data(), d_spin0.p + so, s.N, cudaMemcpyDeviceToHost));
    LG_CUDA(lg_copy(ob.data(), d_off_base.p + so, s.N * sizeof(int), cudaMemcpyDeviceToHost));
    LG_CUDA(lg_copy(oc.data(), d_off_cnt.p + so, s.N * sizeof(int), cudaMemcpyDeviceToHost));
    spins.assign(sp.begin(), sp.end());
    std::vector<std::pair<uint64_t, int>> ops;
    // one copy of each list array over the span the chain's lists occupy
    long long lo = -1, hi = 0;
    for (int i = 0; i < s.N; ++i)
      if (oc[i]) { lo = lo < 0 ? ob[i] : std::min<long long>(lo, ob[i]); hi = std::max<long long>(hi, (long long)ob[i] + oc[i]); }
    std::vector<uint64_t> t(lo < 0 ? 0 : hi - lo);
    std::vector<uint8_t> d(t.size());
    if (!t.empty()) {
      LG_CUDA(lg_copy(t.data(), d_stime.p + lo, t.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      LG_CUDA(lg_copy(d.data(), d_sdir.p + lo, d.size(), cudaMemcpyDeviceToHost));
    }
    for (int i = 0; i < s.N; ++i) {
      const int gs = so + i;
      for (int j = 0; j < oc[i]; ++j) {
        const int idx = h_inc_off[gs] + d[ob[i] - lo + j];
        if (h_inc_side[idx] != 0) continue;  // take each operator once, from its source site
        ops.push_back({t[ob[i] - lo + j], h_inc[idx] - hch[c].bond_off});
      }
    }
    std::sort(ops.begin(), ops.end());
    bonds.resize(ops.size()); times.resize(ops.size());
    for (size_t i = 0; i < ops.size(); ++i) {
      bonds[i] = ops[i].second;
      double t; std::memcpy(&t, &ops[i].first, 8); times[i] = t;
    }
    return LG_OK;
  }

  // Off-diagonal lists of every site as (time bits, incident-bond index) pairs.
  typedef std::vector<std::vector<std::pair<uint64_t, uint8_t>>> SiteLists;

  int download_lists(SiteLists& L) {
    std::vector<int> ob(N), oc(N);
    LG_CUDA(lg_copy(ob.data(), d_off_base.p, N * sizeof(int), cudaMemcpyDeviceToHost));
    LG_CUDA(lg_copy(oc.data(), d_off_cnt.p, N * sizeof(int), cudaMemcpyDeviceToHost));
    L.assign(N, {});
    // one copy of each list array over the span the lists occupy
    long long lo = -1, hi = 0;
    for (int i = 0; i < N; ++i)
      if (oc[i]) { lo = lo < 0 ? ob[i] : std::min<long long>(lo, ob[i]); hi = std::max<long long>(hi, (long long)ob[i] + oc[i]); }
    if (lo < 0) return LG_OK;
    std::vector<uint64_t> t(hi - lo);
    std::vector<uint8_t> d(hi - lo);
    LG_CUDA(lg_copy(t.data(), d_stime.p + lo, t.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    LG_CUDA(lg_copy(d.data(), d_sdir.p + lo, d.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < N; ++i) {
      L[i].resize(oc[i]);
      for (int j = 0; j < oc[i]; ++j) L[i][j] = {t[ob[i] - lo + j], d[ob[i] - lo + j]};
    }
    return LG_OK;
  }

  // Lay the lists out contiguously from segment 0 and upload them.
  int upload_lists(const SiteLists& L) {
    std::vector<int> oc(N);
    long long total = 0;
    for (int i = 0; i < N; ++i) { oc[i] = (int)L[i].size(); total += oc[i]; }
    std::vector<uint64_t> t(total);
    std::vector<uint8_t> d(total);
    for (long long i = 0, k = 0; i < N; ++i)
      for (const auto& e : L[i]) { t[k] = e.first; d[k] = e.second; ++k; }
    return upload_flat(oc, t.data(), d.data());
  }

  // The same from the lists of every site packed in site order (oc[i] entries for site i).
  int upload_flat(const std::vector<int>& oc, const uint64_t* t, const uint8_t* d) {
    std::vector<int> ob(N);
    long long total = 0;
    for (int i = 0; i < N; ++i) { ob[i] = (int)total; total += oc[i]; }
    if (resident) {
      // the list arrays hold res_lcap entries per chain; a chain with more grows the capacity
      long long need = 0;
      for (int c = 0; c < C; ++c) {
        long long n = 0;
        for (int i = 0; i < spec[c].N; ++i) n += oc[hch[c].site_off + i];
        need = std::max(need, n);
      }
      if (need > res_lcap || total > (long long)d_stime.n) {
        const int v2 = (int)std::min<long long>(1ll << 24, ((std::max<long long>(need, res_lcap) * 3 / 4) + 63) & ~31ll);
        if (!res_fits(v2, RES_SMEM_MAX - 1024)) {
          resident = false;
          shape.resident = 0;
          rb_stime.release(); rb_sdir.release(); rb_spin0.release(); rb_off_base.release();
          rb_off_cnt.release();
          int rc = setup_grid();
          if (rc) return rc;
          return upload_flat(oc, t, d);
        }
        int rc = setup_resident(v2);
        if (rc) return rc;
      }
    } else if (total > ns_cap) {
      int rc = alloc_dynamic(total + 4096, false);
      if (rc) return rc;
    }
    LG_CUDA(lg_copy(d_off_base.p, ob.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_off_cnt.p, oc.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    if (total) {
      LG_CUDA(lg_copy(d_stime.p, t, total * sizeof(uint64_t), cudaMemcpyHostToDevice));
      LG_CUDA(lg_copy(d_sdir.p, d, total, cudaMemcpyHostToDevice));
    }
    return LG_OK;
  }

  // n sweeps kernel by kernel with the structural checks of k_validate after insertion, merge,
  // cluster sums and the end of the sweep.  LG_EDEVICE names the first failed check.
  int validate(long long n) {
    if (sse) return lg_fail(LG_EUNSUPPORTED, "the structural checks are of the path-integral form");
    if (resident) {  // the structural checks are of the grid path's arrays
      int rc = to_grid();
      if (rc) return rc;
      shape.resident = 0;
    }
    DBuf<int> bad;
    int rc = bad.alloc(2);
    if (rc) return rc;
    LG_CUDA(cudaMemset(bad.p, 0, 2 * sizeof(int)));
    std::vector<double> km(kNumStages);
    long long v = 0;
    val_bad = bad.p;
    rc = profile(n, 0, km.data(), &v);
    val_bad = nullptr;
    if (rc) return rc;
    int hb[2];
    LG_CUDA(lg_copy(hb, bad.p, sizeof(hb), cudaMemcpyDeviceToHost));
    if (hb[0]) return lg_fail(LG_EDEVICE, "structural check %d failed (%d failures)", hb[1], hb[0]);
    return LG_OK;
  }

  // Union-find retries per union (Ctl::iter_cap): a test seam for the LG_EITERCAP path.
  int set_iter_cap(int cap) {
    Ctl hc;
    LG_CUDA(lg_copy(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost));
    hc.iter_cap = cap;
    LG_CUDA(lg_copy(d_ctl.p, &hc, sizeof(Ctl), cudaMemcpyHostToDevice));
    return LG_OK;
  }

  // A chain's off-diagonal operators as the sweep keeps them: per site, its endpoints in (time,
  // bond) order as (time bits, incidence index), packed in site order (R.oc[i] entries of site i).
  struct Packed {
    PackResult R;
    uint64_t* t = nullptr;  // 2n endpoints: time bits
    uint8_t* d = nullptr;   // and incidence index
    std::unique_ptr<unsigned char[]> own;  // when they are not in the pinned stage
  };

  // Packs n operators of chain c (operator i given by get(i, &bond, &time bits)) with
  // pack_site_lists, into the pinned stage when `stage` (held under its lock) can hold them.
  template <class Get>
  void pack_ops(int c, long long n, const Get& get, Packed& P, HostStage* stage) {
    const ChainSpec& s = spec[c];
    const int bo = hch[c].bond_off;
    PackTables tab;
    tab.N = s.N;
    tab.NB = s.NB;
    tab.s0 = s.s0.data();
    tab.s1 = s.s1.data();
    tab.dir0 = h_bond_dir0.data() + bo;
    tab.dir1 = h_bond_dir1.data() + bo;
    tab.check_parity = s.spin2 <= 1;  // spin-S chains close through the matching, which checks its sectors
    const size_t td = ((size_t)n * 18 + 63) & ~(size_t)63;  // 2n time words and 2n incidence bytes
    const size_t need = td + pack_scratch_bytes(n) + 64;
    unsigned char* base = nullptr;
    if (stage && stage->reserve(need)) {
      base = stage->p;
    } else {
      P.own.reset(new unsigned char[need]);  // no zero fill: every byte used is written
      base = P.own.get();
    }
    P.t = reinterpret_cast<uint64_t*>(base);
    P.d = base + (size_t)n * 16;
    PackRec* scratch = reinterpret_cast<PackRec*>(base + td);
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    pack_site_lists(tab, n, get, P.t, P.d, scratch, P.R, std::min(8, hw));
  }

  // Makes a packed, checked state chain c's state (spins sp[i] in {0, 1}, sweeps done).
  int commit_state(int c, const Packed& P, const std::vector<uint8_t>& sp, uint64_t sweep) {
    const ChainSpec& s = spec[c];
    const int so = hch[c].site_off;
    int rc;
    if (C > 1) {  // the other chains' lists stay as they are
      SiteLists L;
      if ((rc = download_lists(L))) return rc;
      for (int i = 0, k = 0; i < s.N; ++i) {
        auto& Li = L[so + i];
        Li.clear();
        for (int j = 0; j < P.R.oc[i]; ++j, ++k) Li.push_back({P.t[k], P.d[k]});
      }
      if ((rc = upload_lists(L))) return rc;
    } else {
      // a complete, valid state: a union-find failure (LG_EITERCAP) no longer applies
      const int zero = 0;
      LG_CUDA(lg_copy(&d_ctl.p->err, &zero, sizeof(int), cudaMemcpyHostToDevice));
      LG_CUDA(lg_copy(&d_ctl.p->step, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice));
      if ((rc = upload_flat(P.R.oc, P.t, P.d))) return rc;
    }
    LG_CUDA(lg_copy(d_spin0.p + so, sp.data(), s.N, cudaMemcpyHostToDevice));
    uint32_t sw = (uint32_t)sweep;
    LG_CUDA(lg_copy(d_sweep.p + c, &sw, sizeof(uint32_t), cudaMemcpyHostToDevice));
    spec[c].mcs = sweep;
    return LG_OK;
  }

  int set_state(int c, const int32_t* spins, const int32_t* bonds, const double* times, long long n,
                uint64_t sweep) {
    if (sse) return lg_fail(LG_EUNSUPPORTED, "an SSE chain takes its state from lg_load (diagonal operators included)");
    const ChainSpec& s = spec[c];
    HostStage& hs = host_stage();
    std::lock_guard<std::mutex> lock(hs.m);
    Packed P;
    pack_ops(c, n, [&](long long i, int* b, uint64_t* tb) { *b = bonds[i]; std::memcpy(tb, &times[i], 8); }, P, &hs);
    if (P.R.bad >= 0) return lg_fail(LG_EINVAL, "operator %lld out of range", P.R.bad);
    if (P.R.odd_site >= 0)
      return lg_fail(LG_EINVAL, "site %d has an odd number of off-diagonal operators "
                                "(not periodic in imaginary time)", P.R.odd_site);
    std::vector<uint8_t> sp(s.N);
    for (int i = 0; i < s.N; ++i) sp[i] = (uint8_t)(spins[i] & 1);
    return commit_state(c, P, sp, sweep);
  }

  // lg_load of a path-integral checkpoint: the operators are read in place from the blob, packed
  // by pack_ops while a second thread checks the checksum; nothing reaches the device before
  // both are done.
  // Whether lg_load of n operators can pack on the device: a single chain on the grid path, the
  // path-integral form, site offsets in one two-level scan, operator indices below 2^31.
  bool device_load_ok(long long n) const {
    return C == 1 && !sse && !resident && N <= SITE_SCAN_MAX && n > 0 && n < (1ll << 30);
  }

  // The device pass of lg_load (lg_load.cuh).  Stages the spins, operators and the bonds' target
  // incidence indices into the pinned buffer (held by the caller), copies them into the class-sum
  // array (scratch between sweeps, cleared again before returning), runs the checks and the
  // packing, and reads back the status.  *bad, *flags, *odd receive the device checks.  The lists
  // are written only by device_load_commit.
  int device_load_pack(const uint8_t* buf, long long n, HostStage& hs, LoadArgs& L, int* bad,
                       int* flags, int* odd, size_t* scratch_used) {
    if (n > nv_cap) {  // the lists and the scratch need room for 2n endpoints; keep the current ones
      int rc = alloc_dynamic(n + 4096, true);
      if (rc) return rc;
    }
    const size_t npad = ((size_t)N + 15) & ~(size_t)15;
    const size_t ops_b = (size_t)n * 12, dir_b = ((size_t)NB + 15) & ~(size_t)15;
    const size_t stage_b = npad + ops_b + dir_b + 16;  // spins, operators, target incidences, status
    const size_t rec_b = ((size_t)(2 * n) * 4 + 15) & ~(size_t)15;
    const size_t fill_b = ((size_t)N * 4 + 15) & ~(size_t)15;
    const size_t used = stage_b + rec_b + fill_b;
    if (used > (size_t)ns_cap * 4 * sizeof(unsigned long long) || !hs.reserve(stage_b)) {
      *bad = INT_MAX;  // no room: the host packs instead
      *flags = LD_FLAG_LONG;
      *odd = INT_MAX;
      return LG_OK;
    }
    unsigned char* h = hs.p;
    // staging: spins, operator records (4-byte aligned), then dir1; several threads copy the
    // operators
    std::memcpy(h, buf + CHECKPOINT_HEAD, N);
    const unsigned char* ops = buf + CHECKPOINT_HEAD + N;
    const int T = (int)std::max<size_t>(1, std::min<size_t>(4, ops_b >> 20));
    pack_parallel(T, [&](int k) {
      const size_t a = ops_b * k / T, b = ops_b * (k + 1) / T;
      std::memcpy(h + npad + a, ops + a, b - a);
    });
    std::memcpy(h + npad + ops_b, h_bond_dir1.data(), NB);
    int* hstat = reinterpret_cast<int*>(h + npad + ops_b + dir_b);
    hstat[0] = INT_MAX; hstat[1] = 0; hstat[2] = INT_MAX; hstat[3] = 0;
    unsigned char* d = reinterpret_cast<unsigned char*>(d_cls.p);
    LG_CUDA(lg_copy_async(d, h, stage_b, cudaMemcpyHostToDevice, st));
    *scratch_used = used;
    L.spins = d;
    L.ops = reinterpret_cast<const uint32_t*>(d + npad);
    L.n = n;
    L.N = N;
    L.NB = NB;
    L.s0 = d_bond_s0.p;
    L.s1 = d_bond_s1.p;
    L.dir0 = d_bond_dir0.p;
    L.dir1 = d + npad + ops_b;
    L.status = reinterpret_cast<int*>(d + npad + ops_b + dir_b);
    L.rec = reinterpret_cast<uint32_t*>(d + stage_b);
    L.fill = reinterpret_cast<int*>(d + stage_b + rec_b);
    L.cnt = d_site_cnt.p;
    L.off = d_sbase.p;
    L.partial = d_partial.p;
    L.parity = spec[0].spin2 <= 1;
    LG_CUDA(cudaMemsetAsync(L.cnt, 0, (size_t)N * sizeof(int), st));
    LG_CUDA(cudaMemsetAsync(L.fill, 0, (size_t)N * sizeof(int), st));
    const int gops = grid_for(n, 256, 8);
    const int gsites = (N + 1023) / 1024;
    k_ld_count<<<gops, 256, 0, st>>>(L);
    k_ld_scan_blocks<<<gsites, 1024, 0, st>>>(L);
    k_ld_scan_offsets<<<gsites, 1024, 0, st>>>(L);
    k_ld_place<<<gops, 256, 0, st>>>(L);
    k_ld_sort<<<grid_for(N, LD_SORT_WARPS, 8), LD_SORT_WARPS * 32, 0, st>>>(L);
    g_launches += 5;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(lg_copy_async(hstat, L.status, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    LG_CUDA(cudaStreamSynchronize(st));
    *bad = hstat[0];
    *flags = hstat[1];
    *odd = hstat[2];
    return LG_OK;
  }

  // The checked, packed state becomes the chain's (device_load_pack ran and every check passed).
  int device_load_commit(const LoadArgs& L, uint64_t mcs) {
    k_ld_commit_lists<<<grid_for(2 * L.n, 256, 8), 256, 0, st>>>(L, d_stime.p, d_sdir.p);
    k_ld_commit_sites<<<grid_for(N, 256, 8), 256, 0, st>>>(L, d_off_base.p, d_off_cnt.p, d_spin0.p);
    g_launches += 2;
    LG_CUDA(cudaGetLastError());
    // a complete, valid state: a union-find failure (LG_EITERCAP) no longer applies
    LG_CUDA(cudaMemsetAsync(&d_ctl.p->err, 0, sizeof(int), st));
    LG_CUDA(cudaMemsetAsync(&d_ctl.p->step, 0, sizeof(uint32_t), st));
    const uint32_t sw = (uint32_t)mcs;
    LG_CUDA(lg_copy_async(d_sweep.p, &sw, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    LG_CUDA(cudaStreamSynchronize(st));
    spec[0].mcs = mcs;
    return LG_OK;
  }

  // lg_load of a path-integral checkpoint.  The checksum's blocks are hashed on host threads
  // while the operators are checked and packed: on the device (device_load_ok), else by
  // pack_site_lists on host threads.  Nothing reaches the chain's state before every check has
  // passed.
  int load_checkpoint(int c, const uint8_t* buf, size_t size) {
    const ChainSpec& s = spec[c];
    if (!buf || size < CHECKPOINT_HEAD + 8) return lg_fail(LG_ECORRUPT, "checkpoint too short");
    // the checksum's blocks on up to four threads beside the packing
    const size_t nblk = checkpoint_blocks(size);
    std::vector<uint64_t> bh(nblk, 0);
    const int K = (int)std::min<size_t>(4, nblk);
    std::vector<std::thread> sum;
    auto hash_blocks = [&](int k) {
      for (size_t b = (size_t)k; b < nblk; b += (size_t)K) bh[b] = checkpoint_block_hash(buf, size, b);
    };
    int started = 0;
    try {
      sum.reserve(K);
      for (; started < K; ++started) sum.emplace_back(hash_blocks, started);
    } catch (...) {
    }
    auto join_sum = [&]() {
      for (auto& t : sum) t.join();
      sum.clear();
      for (int k = started; k < K; ++k) hash_blocks(k);  // blocks no thread could be started for
    };
    uint64_t n = 0, mcs = 0;
    int hrc = LG_OK;
    HostStage& hs = host_stage();
    std::unique_lock<std::mutex> lock(hs.m);
    Packed P;
    std::vector<uint8_t> sp;
    bool on_device = false, device_flags = false;
    int dbad = INT_MAX, dflags = 0, dodd = INT_MAX;
    LoadArgs L{};
    size_t scratch = 0;
    int drc = LG_OK;
    try {
      hrc = checkpoint_header(s, buf, size, &n, &mcs);
      if (hrc == LG_OK && device_load_ok((long long)n)) {
        on_device = true;
        drc = device_load_pack(buf, (long long)n, hs, L, &dbad, &dflags, &dodd, &scratch);
        device_flags = drc == LG_OK && dbad == INT_MAX && dflags != 0;
      }
      if (hrc == LG_OK && (!on_device || device_flags)) {  // unordered input or a very long list
        const uint8_t* ops = buf + CHECKPOINT_HEAD + s.N;
        pack_ops(c, (long long)n, [&](long long i, int* b, uint64_t* tb) {
          std::memcpy(b, ops + 12 * i, 4);
          std::memcpy(tb, ops + 12 * i + 4, 8);
        }, P, &hs);
        sp.resize(s.N);
        for (int i = 0; i < s.N; ++i) sp[i] = (uint8_t)(buf[CHECKPOINT_HEAD + i] & 1);
      }
    } catch (...) {
      join_sum();
      if (scratch) cudaMemsetAsync(d_cls.p, 0, scratch, st);
      throw;
    }
    join_sum();
    const bool sum_ok = checkpoint_combine(bh.data(), nblk) == checkpoint_stored_checksum(buf, size);
    auto finish = [&](int rc) {  // the class sums were scratch: zero again for the next sweep
      if (scratch && cudaMemsetAsync(d_cls.p, 0, scratch, st) != cudaSuccess && rc == LG_OK)
        rc = lg_fail(LG_EDEVICE, "cudaMemsetAsync failed");
      return rc;
    };
    // the checksum is reported first, then the header (its message is already set), then the rest
    if (!sum_ok) return finish(lg_fail(LG_ECORRUPT, "checkpoint checksum mismatch"));
    if (hrc) return finish(checkpoint_header(s, buf, size, &n, &mcs));
    if (drc) return finish(drc);
    if (on_device && !device_flags) {
      if (dbad != INT_MAX) return finish(lg_fail(LG_ECORRUPT, "checkpoint operator %d out of range", dbad));
      if (dodd != INT_MAX)
        return finish(lg_fail(LG_EINVAL, "site %d has an odd number of off-diagonal operators "
                                         "(not periodic in imaginary time)", dodd));
      return finish(device_load_commit(L, mcs));
    }
    if (P.R.bad >= 0) return finish(lg_fail(LG_ECORRUPT, "checkpoint operator %lld out of range", P.R.bad));
    if (P.R.odd_site >= 0)
      return finish(lg_fail(LG_EINVAL, "site %d has an odd number of off-diagonal operators "
                                       "(not periodic in imaginary time)", P.R.odd_site));
    return finish(commit_state(c, P, sp, mcs));
  }

  // Cluster labels of an explicit configuration (single-chain engine): fills the bond vertex
  // lists from the given time order and runs the segment merge + union-find kernels.
  int uf_label(long long nops, const int32_t* bonds, const int32_t* graphs, std::vector<int32_t>& labels,
               long long* nc) {
    const ChainSpec& s = spec[0];
    std::vector<int> cnt(NB, 0);
    for (long long i = 0; i < nops; ++i) {
      if (bonds[i] < 0 || bonds[i] >= NB || graphs[i] < 0 || graphs[i] > 3)
        return lg_fail(LG_EINVAL, "vertex %lld out of range", i);
      cnt[bonds[i]]++;
    }
    std::vector<int> ptr(NB + 1, 0);
    for (int b = 0; b < NB; ++b) ptr[b + 1] = ptr[b] + cnt[b];
    if (nops > nv_cap) { int rc = alloc_dynamic(nops + 1024, false); if (rc) return rc; }
    std::vector<uint64_t> vt(nops);
    std::vector<uint8_t> vc(nops);
    std::vector<int> fillp(ptr.begin(), ptr.end() - 1);
    std::vector<int> vidx(nops);
    for (long long i = 0; i < nops; ++i) {
      int b = bonds[i];
      int v = fillp[b]++;
      vt[v] = (uint64_t)(i + 1);  // strictly increasing keys reproduce the given order
      vc[v] = (uint8_t)(graphs[i] << 1);
      vidx[i] = v;
    }
    LG_CUDA(lg_copy(d_bond_cnt.p, cnt.data(), NB * sizeof(int), cudaMemcpyHostToDevice));
    LG_CUDA(lg_copy(d_bond_ptr.p, ptr.data(), (NB + 1) * sizeof(int), cudaMemcpyHostToDevice));
    if (nops) {
      LG_CUDA(lg_copy(d_vtime.p, vt.data(), nops * sizeof(uint64_t), cudaMemcpyHostToDevice));
      LG_CUDA(lg_copy(d_vcode.p, vc.data(), nops, cudaMemcpyHostToDevice));
    }
    Ctl hc{};
    hc.nv_total = (int)nops; hc.nv_cap = nv_cap; hc.ns_cap = ns_cap;
    LG_CUDA(lg_copy(d_ctl.p, &hc, sizeof(Ctl), cudaMemcpyHostToDevice));
    Arena A = arena();
    k_site_count<<<grid_for(N, 256, 16), 256, 0, st>>>(A);
    scan(d_site_cnt.p, d_sbase.p, N, &d_ctl.p->ns_total, ns_cap, 1, 0);
    launch_merge(zmax, grid_for((long long)N * 32, MERGE_WARPS * 32, 16),
                 MERGE_WARPS * merge_smem_per_warp(MERGE_CAP), st, A, nullptr, N, MERGE_CAP);
    k_union<><<<grid_for(2 * nops + N, UN_WARPS * UN_CHUNK), UN_WARPS * 32, 0, st>>>(A);
    k_compress<<<grid_for(2 * nops + N, 256), 256, 0, st>>>(A);
    g_launches += 7;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaStreamSynchronize(st));
    LG_CUDA(lg_copy(&hc, d_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost));
    if (hc.err) return lg_fail(LG_EITERCAP, "union-find failed (%d)", hc.err);
    long long ns = 2 * nops + N;
    std::vector<int> par(ns), sb(N + 1), vs(2 * std::max<long long>(nops, 1));
    LG_CUDA(lg_copy(par.data(), d_parent.p, ns * sizeof(int), cudaMemcpyDeviceToHost));
    LG_CUDA(lg_copy(sb.data(), d_sbase.p, (N + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    if (nops) LG_CUDA(lg_copy(vs.data(), d_vslot.p, 2 * nops * sizeof(int), cudaMemcpyDeviceToHost));
    // fragments: site bottoms, then graph-0 vertices in the given order
    std::vector<int> froot;
    froot.reserve(N + nops);
    for (int i = 0; i < N; ++i) froot.push_back(par[sb[i]]);
    for (long long i = 0; i < nops; ++i)
      if (graphs[i] == 0) froot.push_back(par[vs[2 * (size_t)vidx[i]]]);
    std::vector<int> minfrag(ns, -1);
    for (size_t f = 0; f < froot.size(); ++f)
      if (minfrag[froot[f]] < 0) minfrag[froot[f]] = (int)f;  // fragments visited in index order
    std::vector<int> id(froot.size(), -1);
    long long n_c = 0;
    for (size_t f = 0; f < froot.size(); ++f)
      if (minfrag[froot[f]] == (int)f) id[f] = (int)n_c++;
    labels.resize(froot.size());
    for (size_t f = 0; f < froot.size(); ++f) labels[f] = id[minfrag[froot[f]]];
    *nc = n_c;
    (void)s;
    return LG_OK;
  }

  // Retire (or re-enable) a chain: a retired chain inserts no operators and costs almost nothing.
  int set_active(int c, bool on) {
    const bool was_all = std::all_of(h_active.begin(), h_active.end(), [](uint8_t a) { return a != 0; });
    h_active[c] = on ? 1 : 0;
    const bool all = std::all_of(h_active.begin(), h_active.end(), [](uint8_t a) { return a != 0; });
    if (all != was_all) drop_graph();  // the arena's all_active flag is a launch parameter
    LG_CUDA(lg_copy_async(d_active.p + c, &h_active[c], 1, cudaMemcpyHostToDevice, st));
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
  }

  // Take over chains of another arena on the same device: from[c] is the index of new chain c
  // in `old` (or -1 for a new chain).  Spins, off-diagonal lists, sweep counters, schedule and
  // observable accumulators move; the old arena must not be used afterwards.
  int adopt(Engine& old, const std::vector<int>& from) {
    std::vector<int> map(N, -1);
    std::vector<uint32_t> sw(C);
    LG_CUDA(lg_copy(sw.data(), d_sweep.p, C * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (int c = 0; c < C; ++c) {
      const int o = from[c];
      if (o < 0) continue;
      if (old.spec[o].N != spec[c].N) return lg_fail(LG_EINVAL, "adopt: size mismatch");
      for (int i = 0; i < spec[c].N; ++i) map[hch[c].site_off + i] = old.hch[o].site_off + i;
      spec[c].mcs = old.spec[o].mcs;
      spec[c].last_nop = old.spec[o].last_nop;
      acc[c] = old.acc[o];
      sw[c] = (uint32_t)old.spec[o].mcs;
    }
    LG_CUDA(lg_copy(d_sweep.p, sw.data(), C * sizeof(uint32_t), cudaMemcpyHostToDevice));
    DBuf<int> dmap, dcnt, dbase;
    int rc;
    if ((rc = dmap.alloc(N)) || (rc = dcnt.alloc(N)) || (rc = dbase.alloc(N + 1))) return rc;
    LG_CUDA(lg_copy(dmap.p, map.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    Arena A = arena();
    k_repack_count<<<grid_for(N, 256), 256, 0, st>>>(A, dmap.p, old.d_off_cnt.p, dcnt.p);
    LG_CUDA(cudaMemsetAsync(d_ctl.p, 0, sizeof(int), st));
    scan(dcnt.p, dbase.p, N, &d_ctl.p->ns_total, 0x7FFFFFFF, 0, 0);
    g_launches += 3;
    LG_CUDA(lg_copy_async(d_off_cnt.p, dcnt.p, N * sizeof(int), cudaMemcpyDeviceToDevice, st));
    int total = 0;
    LG_CUDA(lg_copy_async(&total, dbase.p + N, sizeof(int), cudaMemcpyDeviceToHost, st));
    LG_CUDA(cudaStreamSynchronize(st));
    if (resident) {
      // the lists land packed in the list array; a chain longer than its slots grows them on
      // its first sweep (overflow), as any other
      if (total > (long long)d_stime.n) {
        if ((rc = d_stime.alloc(total)) || (rc = d_sdir.alloc(total))) return rc;
        A = arena();
      }
    } else if (total > ns_cap) {
      if ((rc = alloc_dynamic(total + 4096, false))) return rc;
      A = arena();
    }
    k_repack_copy<<<grid_for((long long)N * 32, 256), 256, 0, st>>>(A, dmap.p, old.d_spin0.p,
        old.d_off_base.p, old.d_stime.p, old.d_sdir.p, dbase.p);
    g_launches += 2;
    LG_CUDA(cudaGetLastError());
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
  }

  // Exchange of temperatures between chains c1 and c2 (same model): their inverse temperatures
  // and the device parameters that depend on them trade places.  The launch shape, the graph and
  // the accumulators stay (the caller re-points acc_of_chain); a region that then overflows
  // grows on the next sweep as usual.
  int swap_beta(int c1, int c2) {
    const double b1 = spec[c1].beta, b2 = spec[c2].beta;
    int rc;
    if ((rc = spec[c1].set_beta(b2)) || (rc = spec[c2].set_beta(b1))) return rc;
    for (int c : {c1, c2}) {
      hch[c].inv_rate = spec[c].dchain.inv_rate;
      hch[c].flip_coef = spec[c].dchain.flip_coef;
      hch[c].sse_bw = spec[c].dchain.sse_bw;
      LG_CUDA(lg_copy_async(d_ch.p + c, &hch[c], sizeof(DChain), cudaMemcpyHostToDevice, st));
    }
    LG_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
  }

  int set_beta(int c, double beta) {
    int rc = spec[c].set_beta(beta);
    if (rc) return rc;
    hch[c].inv_rate = spec[c].dchain.inv_rate;
    hch[c].flip_coef = spec[c].dchain.flip_coef;
    hch[c].sse_bw = spec[c].dchain.sse_bw;
    LG_CUDA(lg_copy(d_ch.p + c, &hch[c], sizeof(DChain), cudaMemcpyHostToDevice));
    acc[c] = ChainAcc();
    if (resident || sse) return LG_OK;  // a grown operator count grows the capacity on overflow
    set_merge_cap();
    return set_shape(shape);  // the chain's narrow / wide class depends on beta
  }
};

// ================================================================================================
// C ABI
// ================================================================================================
struct lg_chain {
  std::shared_ptr<Engine> eng;
  int index = 0;
};
struct lg_batch {
  std::shared_ptr<Engine> eng;
  std::vector<lg_chain> views;
};

extern "C" {

int lg_last_error(char* buf, size_t n) {
  return lg_guard([&]() -> int {
    if (buf && n) { std::snprintf(buf, n, "%s", g_err.c_str()); }
    return (int)g_err.size();
  });
}

uint64_t lg_kernel_launches(void) { return g_launches.load(); }

void lg_copy_bytes(uint64_t* h2d, uint64_t* d2h) {
  if (h2d) *h2d = g_h2d_bytes.load();
  if (d2h) *d2h = g_d2h_bytes.load();
}

const char* lg_version(void) {
  static std::string v;
  if (v.empty()) {
    int rt = 0; cudaRuntimeGetVersion(&rt);
    v = "looper_gb300 1.0 (sm_103a; CUDA runtime " + std::to_string(rt) + ")";
  }
  return v.c_str();
}

int lg_create(const lg_params* p, lg_chain** out) {
  return lg_guard([&]() -> int {
    if (!p || !out) return lg_fail(LG_EINVAL, "null argument");
    ChainSpec s;
    int rc = s.init(*p);
    if (rc) return rc;
    auto e = std::make_shared<Engine>();
    rc = e->build({s}, true);
    if (rc) return rc;
    lg_chain* c = new lg_chain();
    c->eng = e;
    *out = c;
    return LG_OK;
  });
}

int lg_destroy(lg_chain* c) {
  return lg_guard([&]() -> int {
    delete c; return LG_OK;
  });
}

int lg_run(lg_chain* c, int64_t n) {
  return lg_guard([&]() -> int {
    if (!c || n < 0) return lg_fail(LG_EINVAL, "bad argument");
    if (c->eng->C != 1) return lg_fail(LG_EINVAL, "lg_run on a batch member; use lg_batch_run");
    return c->eng->run(n);
  });
}

int lg_is_thermalized(const lg_chain* c) {
  return lg_guard([&]() -> int {
    const ChainSpec& s = c->eng->spec[c->index];
    return s.mcs >= (uint64_t)s.therm ? 1 : 0;
  });
}

double lg_progress(const lg_chain* c) {
  const ChainSpec& s = c->eng->spec[c->index];
  double tot = (double)(s.therm + s.sweeps);
  return tot > 0 ? std::min(1.0, (double)s.mcs / tot) : 1.0;
}

int lg_observables(lg_chain* c, lg_obs* out) {
  return lg_guard([&]() -> int {
    if (!c || !out) return lg_fail(LG_EINVAL, "null argument");
    c->eng->acc[c->index].report(c->eng->spec[c->index], out);
    return LG_OK;
  });
}

// Real part of the discrete Fourier transform sum_r e^{i k.r} f(r) over a periodic L^dim grid
// (site order x fastest), one dimension at a time: O(N L dim).
static void grid_dft(int dim, int L, const std::vector<double>& f, std::vector<double>& out) {
  const int N = (int)f.size();
  std::vector<double> re(f), im(N, 0.0), tr(N), ti(N);
  std::vector<double> cs(L), sn(L);
  for (int t = 0; t < L; ++t) {
    const double a = 2.0 * M_PI * (double)t / (double)L;
    cs[t] = std::cos(a);
    sn[t] = std::sin(a);
  }
  int stride = 1;
  for (int d = 0; d < dim; ++d) {
    for (int i = 0; i < N; ++i) {
      const int x = (i / stride) % L, base = i - x * stride;
      double sr = 0, si = 0;
      for (int y = 0; y < L; ++y) {  // k_x = x, r_x = y: phase 2 pi x y / L
        const int t = (int)(((long long)x * y) % L);
        const double vr = re[base + y * stride], vi = im[base + y * stride];
        sr += vr * cs[t] - vi * sn[t];
        si += vr * sn[t] + vi * cs[t];
      }
      tr[i] = sr;
      ti[i] = si;
    }
    re.swap(tr);
    im.swap(ti);
    stride *= L;
  }
  out = re;
}

int lg_correlations(lg_chain* c, int kind, double* mean, double* err) {
  return lg_guard([&]() -> int {
    if (!c || !mean) return lg_fail(LG_EINVAL, "null argument");
    const Engine& e = *c->eng;
    const ChainSpec& s = e.spec[c->index];
    const ChainAcc& a = e.acc[c->index];
    const int N = s.N;
    std::vector<double> m, er;
    if (kind == LG_CORR_SPIN || kind == LG_CORR_STAGGERED) {
      if (!s.measure_corr) return lg_fail(LG_EINVAL, "the chain does not measure correlations");
      if (kind == LG_CORR_STAGGERED && !s.bipartite)
        return lg_fail(LG_EINVAL, "staggered correlations need a bipartite lattice");
      const bool origin = s.corr_origin >= 0;
      (origin ? a.corr_origin : a.corr_disp).mean_err(m, er);
      if ((int)m.size() != N) { m.assign(N, NAN); er.assign(N, NAN); }
      // correlation.h:243-264: 1/4 (1-2s)(1-2s'), times 1/N pairs per displacement without origin
      const double f = origin ? 0.25 : 0.25 / N;
      for (int i = 0; i < N; ++i) {
        double g = 1.0;
        if (kind == LG_CORR_STAGGERED)
          g = origin ? (double)(s.gauge[s.corr_origin] * s.gauge[i]) : (double)s.gauge[i] * s.gauge[0];
        mean[i] = f * g * m[i];
        if (err) err[i] = f * er[i];
      }
      return LG_OK;
    }
    if (kind == LG_SFAC) {
      if (!s.measure_sfac) return lg_fail(LG_EINVAL, "the chain does not measure the structure factor");
      // S(k) = 1/N |sum_s (1/2 - s_s) e^{ik.r_s}|^2 (correlation.h:268-281) = sum_r e^{ik.r} C(r)
      // with C(r) = 1/(4N) sum_i m_i m_{i+r}: the transform of the all-pairs sums, per sweep and so
      // for the mean and for every bin mean
      const VecAcc& v = a.corr_disp;
      if ((int)v.sum.size() != N || v.count <= 0) {
        for (int i = 0; i < N; ++i) { mean[i] = NAN; if (err) err[i] = NAN; }
        return LG_OK;
      }
      std::vector<double> f(N), out;
      for (int i = 0; i < N; ++i) f[i] = 0.25 * (double)v.sum[i] / (double)v.count / N;
      grid_dft(s.dim, s.L, f, out);
      for (int i = 0; i < N; ++i) mean[i] = out[i];
      if (err) {
        // bins merged into at most 32 groups for the error
        const size_t B = v.bins.size();
        const size_t G = std::min<size_t>(B, 32);
        std::vector<double> var(N, 0.0);
        int64_t tot = 0;
        if (G >= 2) {
          for (size_t g = 0; g < G; ++g) {
            const size_t k0 = g * B / G, k1 = (g + 1) * B / G;
            int64_t cnt = 0;
            std::vector<double> fb(N, 0.0);
            for (size_t k = k0; k < k1; ++k) {
              cnt += v.bin_count[k];
              for (int i = 0; i < N; ++i) fb[i] += (double)v.bins[k][i];
            }
            for (int i = 0; i < N; ++i) fb[i] = 0.25 * fb[i] / (double)cnt / N;
            grid_dft(s.dim, s.L, fb, out);
            for (int i = 0; i < N; ++i) var[i] += (double)cnt * (out[i] - mean[i]) * (out[i] - mean[i]);
            tot += cnt;
          }
          for (int i = 0; i < N; ++i) err[i] = std::sqrt(var[i] / (double)tot / (double)(G - 1));
        } else {
          for (int i = 0; i < N; ++i) err[i] = NAN;
        }
      }
      return LG_OK;
    }
    return lg_fail(LG_EINVAL, "unknown correlation kind %d", kind);
  });
}

int lg_correlation_sums(lg_chain* c, int which, int64_t* sums, int64_t* nsweeps) {
  return lg_guard([&]() -> int {
    if (!c || !sums) return lg_fail(LG_EINVAL, "null argument");
    const Engine& e = *c->eng;
    const ChainSpec& s = e.spec[c->index];
    const ChainAcc& a = e.acc[c->index];
    const bool on = which == 0 ? e.hch[c->index].corr_disp != 0 : e.hch[c->index].corr_origin >= 0;
    if (which < 0 || which > 1 || !on) return lg_fail(LG_EINVAL, "the chain does not keep these sums");
    const VecAcc& v = which ? a.corr_origin : a.corr_disp;
    for (int i = 0; i < s.N; ++i) sums[i] = (int)v.sum.size() == s.N ? v.sum[i] : 0;
    if (nsweeps) *nsweeps = v.count;
    return LG_OK;
  });
}

int lg_set_beta(lg_chain* c, double beta) {
  return lg_guard([&]() -> int {
    return c->eng->set_beta(c->index, beta);
  });
}

double lg_weight_parameter(lg_chain* c) { return (double)c->eng->spec[c->index].last_nop; }

double lg_log_weight(double gw, double beta) { return std::log(beta) * gw; }

int lg_get_state(lg_chain* c, int32_t* spins, int32_t* bonds, double* times, int64_t cap,
                 int64_t* n) {
  return lg_guard([&]() -> int {
    std::vector<int32_t> sp, bd;
    std::vector<double> tm;
    int rc = c->eng->get_state(c->index, sp, bd, tm);
    if (rc) return rc;
    if (spins) std::memcpy(spins, sp.data(), sp.size() * sizeof(int32_t));
    int64_t m = std::min<int64_t>(cap, (int64_t)bd.size());
    if (bonds && m > 0) std::memcpy(bonds, bd.data(), m * sizeof(int32_t));
    if (times && m > 0) std::memcpy(times, tm.data(), m * sizeof(double));
    if (n) *n = (int64_t)bd.size();
    return LG_OK;
  });
}

int lg_set_state(lg_chain* c, const int32_t* spins, const int32_t* bonds, const double* times,
                 int64_t n, uint64_t sweep) {
  return lg_guard([&]() -> int {
    return c->eng->set_state(c->index, spins, bonds, times, n, sweep);
  });
}

int lg_keep_records(lg_chain* c, int on) {
  return lg_guard([&]() -> int {
    if (c->index != 0) return lg_fail(LG_EINVAL, "records are kept for chain 0 only");
    c->eng->keep_records = on != 0;
    return LG_OK;
  });
}

int lg_fetch_records(lg_chain* c, uint64_t* out, int64_t cap, int64_t* n) {
  return lg_guard([&]() -> int {
    auto& k = c->eng->kept;
    int64_t rows = (int64_t)(k.size() / LG_RECORD_WORDS);
    int64_t m = std::min(rows, cap);
    if (out && m > 0) std::memcpy(out, k.data(), m * LG_RECORD_WORDS * sizeof(uint64_t));
    k.erase(k.begin(), k.begin() + m * LG_RECORD_WORDS);
    if (n) *n = m;
    return LG_OK;
  });
}

int lg_value_mask(const lg_chain* c, uint64_t* mask) {
  return lg_guard([&]() -> int {
    if (!c || !mask) return lg_fail(LG_EINVAL, "null argument");
    *mask = value_mask(c->eng->spec[c->index]);
    return LG_OK;
  });
}

int lg_keep_values(lg_chain* c, int on) {
  return lg_guard([&]() -> int {
    if (!c) return lg_fail(LG_EINVAL, "null argument");
    c->eng->keep_vals[c->index] = on ? 1 : 0;
    if (!on) c->eng->vals[c->index].clear();
    return LG_OK;
  });
}

int lg_fetch_values(lg_chain* c, double* out, int64_t cap, int64_t* n) {
  return lg_guard([&]() -> int {
    if (!c || cap < 0 || (cap > 0 && !out)) return lg_fail(LG_EINVAL, "bad argument");
    auto& k = c->eng->vals[c->index];
    const int64_t rows = (int64_t)(k.size() / LG_NUM_VALUES);
    const int64_t m = std::min(rows, cap);
    if (m > 0) std::memcpy(out, k.data(), (size_t)m * LG_NUM_VALUES * sizeof(double));
    k.erase(k.begin(), k.begin() + (size_t)m * LG_NUM_VALUES);
    if (n) *n = m;
    return LG_OK;
  });
}

int lg_save(lg_chain* c, void* buf, size_t* size) {
  return lg_guard([&]() -> int {
    std::vector<int32_t> sp, bd;
    std::vector<double> tm;
    int rc;
    if (c->eng->sse) {  // the whole string: bond << 1 | type, in order
      std::vector<uint32_t> ops;
      if ((rc = c->eng->sse_get(c->index, sp, ops))) return rc;
      for (size_t i = 0; i < ops.size(); ++i) { bd.push_back((int32_t)ops[i]); tm.push_back((i + 0.5) / ops.size()); }
    } else if ((rc = c->eng->get_state(c->index, sp, bd, tm))) {
      return rc;
    }
    std::vector<uint8_t> blob;
    checkpoint_encode(c->eng->spec[c->index], sp, bd, tm, blob);
    if (!buf) { *size = blob.size(); return LG_OK; }
    if (*size < blob.size()) { *size = blob.size(); return lg_fail(LG_EINVAL, "buffer too small"); }
    std::memcpy(buf, blob.data(), blob.size());
    *size = blob.size();
    return LG_OK;
  });
}

int lg_validate_sweeps(lg_chain* c, int64_t n) {
  return lg_guard([&]() -> int {
    if (!c || n < 0) return lg_fail(LG_EINVAL, "bad argument");
    if (c->eng->C != 1) return lg_fail(LG_EINVAL, "lg_validate_sweeps on a batch member; use lg_batch_validate_sweeps");
    return c->eng->validate(n);
  });
}

int lg_batch_validate_sweeps(lg_batch* b, int64_t n) {
  return lg_guard([&]() -> int {
    if (!b || n < 0) return lg_fail(LG_EINVAL, "bad argument");
    return b->eng->validate(n);
  });
}

int lg_set_iteration_cap(lg_chain* c, int cap) {
  return lg_guard([&]() -> int {
    if (!c) return lg_fail(LG_EINVAL, "null argument");
    return c->eng->set_iter_cap(cap);
  });
}

int lg_load(lg_chain* c, const void* buf, size_t size) {
  return lg_guard([&]() -> int {
    if (!c) return lg_fail(LG_EINVAL, "null argument");
    if (!c->eng->sse) return c->eng->load_checkpoint(c->index, (const uint8_t*)buf, size);
    std::vector<int32_t> sp, bd;
    std::vector<double> tm;
    uint64_t mcs = 0;
    int rc = checkpoint_decode(c->eng->spec[c->index], (const uint8_t*)buf, size, sp, bd, tm, &mcs);
    if (rc) return rc;
    if (c->eng->sse) {
      for (size_t i = 1; i < tm.size(); ++i)
        if (!(tm[i] > tm[i - 1])) return lg_fail(LG_ECORRUPT, "checkpoint operators out of order");
      std::vector<uint32_t> ops(bd.begin(), bd.end());
      return c->eng->sse_set(c->index, sp.data(), ops, mcs);
    }
    return c->eng->set_state(c->index, sp.data(), bd.data(), tm.data(), (int64_t)bd.size(), mcs);
  });
}

int lg_uf_label(int lattice, int L, int64_t nops, const int32_t* bonds, const int32_t* graphs,
                int32_t* labels, int64_t cap, int64_t* nfrag, int64_t* nc) {
  return lg_guard([&]() -> int {
    lg_params p;
    lg_params_default(&p);
    p.lattice = lattice; p.L = L; p.T = 1.0; p.Jxy = 0.0; p.Jz = 1.0;  // no sign check needed
    ChainSpec s;
    int rc = s.init(p);
    if (rc) return rc;
    Engine e;
    rc = e.build({s});
    if (rc) return rc;
    std::vector<int32_t> lab;
    long long n_c = 0;
    rc = e.uf_label(nops, bonds, graphs, lab, &n_c);
    if (rc) return rc;
    if (nfrag) *nfrag = (int64_t)lab.size();
    if (nc) *nc = n_c;
    if (labels) std::memcpy(labels, lab.data(), std::min<int64_t>(cap, (int64_t)lab.size()) * sizeof(int32_t));
    return (int64_t)lab.size() > cap ? lg_fail(LG_EINVAL, "labels buffer too small") : LG_OK;
  });
}

int lg_batch_create(int n, const lg_params* p, lg_batch** out) {
  return lg_guard([&]() -> int {
    if (n <= 0 || !p || !out) return lg_fail(LG_EINVAL, "bad argument");
    std::vector<ChainSpec> specs(n);
    for (int i = 0; i < n; ++i) {
      int rc = specs[i].init(p[i]);
      if (rc) return rc;
    }
    auto e = std::make_shared<Engine>();
    int rc = e->build(specs, true);
    if (rc) return rc;
    lg_batch* b = new lg_batch();
    b->eng = e;
    b->views.resize(n);
    for (int i = 0; i < n; ++i) { b->views[i].eng = e; b->views[i].index = i; }
    *out = b;
    return LG_OK;
  });
}

int lg_batch_destroy(lg_batch* b) {
  return lg_guard([&]() -> int {
    delete b; return LG_OK;
  });
}
int lg_batch_run(lg_batch* b, int64_t n) {
  return lg_guard([&]() -> int {
    return b->eng->run(n);
  });
}
int lg_batch_size(const lg_batch* b) {
  return lg_guard([&]() -> int {
    return b->eng->C;
  });
}
lg_chain* lg_batch_chain(lg_batch* b, int i) {
  return (i >= 0 && i < (int)b->views.size()) ? &b->views[i] : nullptr;
}
int lg_batch_observables(lg_batch* b, int chain, lg_obs* out) {
  return lg_guard([&]() -> int {
    if (chain < 0 || chain >= b->eng->C) return lg_fail(LG_EINVAL, "chain index");
    b->eng->acc[chain].report(b->eng->spec[chain], out);
    return LG_OK;
  });
}
int lg_batch_stats(const lg_batch* b, int64_t* total_sites, int64_t* site_sweeps) {
  return lg_guard([&]() -> int {
    long long ts = 0, ss = 0;
    for (auto& s : b->eng->spec) { ts += s.volume; ss += (long long)s.volume * (long long)s.mcs; }
    if (total_sites) *total_sites = ts;
    if (site_sweeps) *site_sweeps = ss;
    return LG_OK;
  });
}


static void shape_out(const Shape& s, lg_shape* out) {
  if (!out) return;
  out->insert_k = s.insert_k;
  out->narrow_k = s.narrow_k;
  out->acc_tile = s.acc_tile;
  out->cl_tile = s.cl_tile;
  out->union_warps = s.un_warps;
  out->resident = s.resident;
  out->union_mode = s.union_mode;
}

static int autotune_engine(Engine& e, int trial, size_t flush_bytes, lg_shape* chosen, char* report,
                           size_t report_len) {
  std::string rep;
  int rc = e.autotune(trial, flush_bytes, rep);
  if (report && report_len) std::snprintf(report, report_len, "%s", rep.c_str());
  if (rc) return rc;
  shape_out(e.shape, chosen);
  return LG_OK;
}

int lg_autotune(lg_chain* c, int trial_sweeps, size_t flush_bytes, lg_shape* chosen, char* report,
                size_t report_len) {
  return lg_guard([&]() -> int {
    if (!c || trial_sweeps < 1) return lg_fail(LG_EINVAL, "bad argument");
    if (c->eng->C != 1) return lg_fail(LG_EINVAL, "lg_autotune on a batch member; use lg_batch_autotune");
    return autotune_engine(*c->eng, trial_sweeps, flush_bytes, chosen, report, report_len);
  });
}

int lg_batch_autotune(lg_batch* b, int trial_sweeps, size_t flush_bytes, lg_shape* chosen,
                      char* report, size_t report_len) {
  return lg_guard([&]() -> int {
    if (!b || trial_sweeps < 1) return lg_fail(LG_EINVAL, "bad argument");
    return autotune_engine(*b->eng, trial_sweeps, flush_bytes, chosen, report, report_len);
  });
}

static int set_shape_engine(Engine& e, const lg_shape* in) {
  Shape s;
  s.insert_k = in->insert_k;
  s.narrow_k = in->narrow_k;
  s.acc_tile = in->acc_tile;
  s.cl_tile = in->cl_tile;
  s.un_warps = in->union_warps;
  s.resident = in->resident;
  s.union_mode = in->union_mode;
  return e.set_shape(s);
}

int lg_get_shape(const lg_chain* c, lg_shape* out) {
  return lg_guard([&]() -> int {
    if (!c || !out) return lg_fail(LG_EINVAL, "null argument");
    shape_out(c->eng->shape, out);
    return LG_OK;
  });
}

int lg_set_shape(lg_chain* c, const lg_shape* in) {
  return lg_guard([&]() -> int {
    if (!c || !in) return lg_fail(LG_EINVAL, "null argument");
    if (c->eng->C != 1) return lg_fail(LG_EINVAL, "lg_set_shape on a batch member; use lg_batch_set_shape");
    return set_shape_engine(*c->eng, in);
  });
}

int lg_batch_get_shape(const lg_batch* b, lg_shape* out) {
  return lg_guard([&]() -> int {
    if (!b || !out) return lg_fail(LG_EINVAL, "null argument");
    shape_out(b->eng->shape, out);
    return LG_OK;
  });
}

int lg_batch_set_shape(lg_batch* b, const lg_shape* in) {
  return lg_guard([&]() -> int {
    if (!b || !in) return lg_fail(LG_EINVAL, "null argument");
    return set_shape_engine(*b->eng, in);
  });
}

int lg_time_sweeps(lg_chain* c, int64_t n, size_t flush_bytes, float* ms) {
  return lg_guard([&]() -> int {
    if (!c || n < 0 || !ms) return lg_fail(LG_EINVAL, "bad argument");
    return c->eng->run(n, ms, flush_bytes);
  });
}

int lg_batch_time_sweeps(lg_batch* b, int64_t n, size_t flush_bytes, float* ms) {
  return lg_guard([&]() -> int {
    if (!b || n < 0 || !ms) return lg_fail(LG_EINVAL, "bad argument");
    return b->eng->run(n, ms, flush_bytes);
  });
}

int lg_profile_sweeps(lg_chain* c, int64_t n, size_t flush_bytes, double* kernel_ms,
                      int64_t* vertices) {
  return lg_guard([&]() -> int {
    long long v = 0;
    int rc = c->eng->profile(n, flush_bytes, kernel_ms, &v);
    if (vertices) *vertices = v;
    return rc;
  });
}

int lg_batch_profile_sweeps(lg_batch* b, int64_t n, size_t flush_bytes, double* kernel_ms,
                            int64_t* vertices) {
  return lg_guard([&]() -> int {
    long long v = 0;
    int rc = b->eng->profile(n, flush_bytes, kernel_ms, &v);
    if (vertices) *vertices = v;
    return rc;
  });
}

int lg_num_kernels(void) {
  return lg_guard([&]() -> int {
    return kNumStages;
  });
}
const char* lg_kernel_name(int k) { return (k >= 0 && k < kNumStages) ? kStageNames[k] : ""; }

}  // extern "C"

// Allocation-free variant of lg_uf_label (same translation unit: it launches these kernels).
#include "lg_static.cu"

// Request server with continuous batching over one arena.
#include "lg_server.cu"

// Exchange Monte Carlo over a ladder of temperatures in one arena.
#include "lg_exchange.cu"
