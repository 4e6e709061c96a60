// lg_uf_label_static: the cluster labelling of lg_uf_label without any allocation.
//
// Some callers of this library cannot call cudaMalloc.
// - A plug-in whose host framework owns every device allocation through its own pool, where a
//   library allocation outside that pool is forbidden or would defeat its memory budgeting.
// - Code on a latency-critical path that cannot take the device-wide synchronisation of
//   cudaFree.  (This call synchronises only its own stream, once, to return the counts.)
//
// For them this entry point takes device pointers for its inputs and outputs.  It keeps every
// intermediate array (bond lists, segments, the union-find forest, fragment ids) in one
// file-scope static device array of LG_STATIC_SCRATCH_BYTES, which every GPU that loads this
// library holds until the process exits.  The work is the one lg_uf_label does with allocated
// buffers: the same segment merge and lock-free union-find kernels, with the reference-numbered
// labels assigned on the device.  Vertices are placed into their bonds' lists by a stable
// two-pass radix sort on the bond index (linear work, so a lattice of two sites with 2^18
// vertices is as cheap as any other input of that size).
//
// Limits: at most LG_STATIC_MAX_SITES sites and LG_STATIC_MAX_OPS vertices per call; larger
// inputs are rejected with LG_EBUDGET before any device work.
//
// Set-up: the first call on each device, with that device current, looks up the array's device
// address with cudaGetSymbolAddress and keeps it for the life of the process.  Make that first
// call before opening any stream capture.  cudaDeviceReset unloads the array, so the kept address
// is stale after a reset: do not call this entry point on a device that was reset.
//
// Sharing: every call uses the same array, and the array keeps what the last call left.  The
// call clears everything that must start at zero.  Calls whose device work overlaps (for
// example, calls on two streams at once) race on the array and give wrong labels; serialise
// them.
//
// This translation unit is included at the end of lg_engine.cu so that it launches the very
// kernels of the sweep.

#include <mutex>

namespace {

constexpr size_t LG_STATIC_SCRATCH_BYTES = 32ull << 20;  // 32 MiB per device
constexpr int LG_STATIC_MAX_SITES = 16384;
constexpr int LG_STATIC_MAX_OPS = 1 << 18;

static __device__ __align__(256) unsigned char g_label_scratch[LG_STATIC_SCRATCH_BYTES];

std::mutex g_scratch_mu;
void* g_scratch_addr[64] = {nullptr};

// Device address of g_label_scratch on the current device (looked up once per device).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return lg_fail(LG_EDEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return lg_fail(LG_EDEVICE, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_label_scratch);
    if (e != cudaSuccess || !p)
      return lg_fail(LG_EDEVICE, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return LG_OK;
}

// Bump layout of the scratch array (256-byte aligned pieces).
struct Carve {
  unsigned char* base;
  size_t used = 0;
  template <class T>
  T* take(size_t n) {
    used = (used + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + used);
    used += n * sizeof(T);
    return p;
  }
};

// Incident bonds of a periodic hypercubic lattice, ascending bond id, as the engine builds them.
__global__ void ks_lattice(Arena A, int dim, int L) {
  LG_GRID_STRIDE(s, A.N) {
    int x[3] = {0, 0, 0}, r = s, par = 0;
    for (int i = 0; i < dim; ++i) { x[i] = r % L; r /= L; par += x[i]; }
    int b[2 * MAXZ];
    uint8_t sd[2 * MAXZ];
    int n = 0;
    for (int d = 0; d < dim; ++d) {
      b[n] = s * dim + d; sd[n] = 0; ++n;                       // s is the source
      int y[3] = {x[0], x[1], x[2]};
      y[d] = (y[d] + L - 1) % L;
      int t = 0;
      for (int j = dim - 1; j >= 0; --j) t = t * L + y[j];
      b[n] = t * dim + d; sd[n] = 1; ++n;                       // s is the target
    }
    for (int i = 1; i < n; ++i)
      for (int j = i; j > 0 && b[j - 1] > b[j]; --j) {
        const int tb = b[j]; b[j] = b[j - 1]; b[j - 1] = tb;
        const uint8_t ts = sd[j]; sd[j] = sd[j - 1]; sd[j - 1] = ts;
      }
    const int o = s * 2 * dim;
    for (int i = 0; i < n; ++i) { const_cast<int*>(A.inc)[o + i] = b[i]; const_cast<uint8_t*>(A.inc_side)[o + i] = sd[i]; }
    const_cast<int*>(A.inc_off)[s] = o;
    if (s == A.N - 1) const_cast<int*>(A.inc_off)[A.N] = A.N * 2 * dim;
    const_cast<int8_t*>(A.gauge)[s] = (par % 2 == 0) ? 1 : -1;
    const_cast<int*>(A.site_chain)[s] = 0;
    A.spin0[s] = 0;
  }
}

// Count vertices per bond and flag graph-0 vertices; reject malformed input.
__global__ void ks_count(Arena A, const int32_t* bonds, const int32_t* graphs, int nops, int* g0flag) {
  LG_GRID_STRIDE(i, nops) {
    const int b = bonds[i], g = graphs[i];
    if (b < 0 || b >= A.NB || g < 0 || g > 3) { atomicExch(&A.ctl->err, 3); continue; }
    atomicAdd(A.bond_cnt + b, 1);
    g0flag[i] = (g == 0) ? 1 : 0;
  }
}

// Stable LSD radix sort of the vertices by bond index (two 8-bit digits: bonds < 2^16), so that
// each bond's vertices come out in input (time) order.  Tiles of RS_TILE entries; the digit
// counts of every tile are stored digit-major, hist[d * ntiles + t], so that their exclusive
// scan gives each (digit, tile) its first output position in stable order.
constexpr int RS_THREADS = 256;
constexpr int RS_PER = 8;
constexpr int RS_TILE = RS_THREADS * RS_PER;

__global__ void __launch_bounds__(RS_THREADS) ks_radix_hist(const int32_t* key, int n, int shift,
                                                            int* hist, int ntiles, const Ctl* ctl) {
  if (ctl->err) return;
  __shared__ int h[256];
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    for (int i = threadIdx.x; i < 256; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    for (int j = 0; j < RS_PER; ++j) {
      const int e = t * RS_TILE + j * RS_THREADS + threadIdx.x;
      if (e < n) atomicAdd(&h[(key[e] >> shift) & 255], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += RS_THREADS) hist[i * ntiles + t] = h[i];
    __syncthreads();
  }
}

// Scatter of one digit pass.  A tile's entries are placed in order: chunk by chunk, and within a
// chunk warp by warp, each lane after the lanes of its warp with the same digit (match_any) and
// after everything placed before with that digit (base[d]).  val == nullptr: the value of entry e
// is e (the input index).
__global__ void __launch_bounds__(RS_THREADS) ks_radix_scatter(const int32_t* key, const int* val,
                                                               int n, int shift, const int* hoff,
                                                               int ntiles, int32_t* kout, int* vout,
                                                               const Ctl* ctl) {
  if (ctl->err) return;
  __shared__ int base[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    for (int i = threadIdx.x; i < 256; i += RS_THREADS) base[i] = hoff[i * ntiles + t];
    __syncthreads();
    for (int c = 0; c < RS_PER; ++c) {
      const int e = t * RS_TILE + c * RS_THREADS + threadIdx.x;
      const bool ok = e < n;
      const int k = ok ? key[e] : 0;
      const int d = ok ? (k >> shift) & 255 : 256 + lane;  // lanes past the end: no group
      const unsigned grp = __match_any_sync(0xFFFFFFFFu, d);
      const int r = __popc(grp & ((1u << lane) - 1u));
      const bool last = (grp >> lane) == 1u;                // highest lane of its group
      for (int ww = 0; ww < RS_THREADS / 32; ++ww) {
        if (w == ww) {
          const int pos = ok ? base[d] + r : 0;
          __syncwarp();
          if (ok && last) base[d] += __popc(grp);
          if (ok) { kout[pos] = k; vout[pos] = val ? val[e] : e; }
        }
        __syncthreads();
      }
    }
  }
}

// Vertex slots from the sorted order: position p holds input idx[p]; its key is idx + 1 (the
// given time order) and its code the input graph.
__global__ void ks_place(Arena A, const int* idx, const int32_t* graphs, int nops, int* v_of_input) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(p, nops) {
    const int i = idx[p];
    v_of_input[i] = p;
    A.vtime[p] = (uint64_t)i + 1;
    A.vcode[p] = (uint8_t)(graphs[i] << 1);
  }
}

__global__ void ks_compress(Arena A) {
  if (A.ctl->err) return;
  const int ns = A.ctl->ns_total;
  LG_GRID_STRIDE(x, ns) {
    int r = x, p = A.parent[x];
    while (p != r) { r = p; p = A.parent[r]; }
    A.parent[x] = r;
  }
}

// Fragment f: f < N is the bottom segment of site f; N + k the upper segments of the k-th
// graph-0 vertex in time order.  froot[f] = its cluster root; minfrag[root] = min f.
__global__ void ks_fragments(Arena A, int nops, const int* g0flag, const int* g0ord,
                             const int* v_of_input, int* g0_input, int* froot, unsigned* minfrag) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(i, nops) {
    if (g0flag[i]) g0_input[g0ord[i]] = i;
  }
  LG_GRID_STRIDE(s, A.N) {
    const int r = A.parent[A.sbase[s]];
    froot[s] = r;
    atomicMin(minfrag + r, (unsigned)s);
  }
}

__global__ void ks_fragments_g0(Arena A, int ng0, const int* g0_input, const int* v_of_input,
                                int* froot, unsigned* minfrag) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(k, ng0) {
    const int v = v_of_input[g0_input[k]];
    const int r = A.parent[A.vslot[2 * v]];
    froot[A.N + k] = r;
    atomicMin(minfrag + r, (unsigned)(A.N + k));
  }
}

__global__ void ks_repflag(Arena A, int nfrag, const int* froot, const unsigned* minfrag, int* flag) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(f, nfrag) flag[f] = (minfrag[froot[f]] == (unsigned)f) ? 1 : 0;
}

__global__ void ks_label(Arena A, int nfrag, const int* froot, const unsigned* minfrag,
                         const int* id, int32_t* labels) {
  if (A.ctl->err) return;
  LG_GRID_STRIDE(f, nfrag) labels[f] = id[minfrag[froot[f]]];
}

void static_scan(const int* in, int* out, int n, int* total, int* partial, Ctl* ctl,
                 cudaStream_t st) {
  int parts = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (parts < 1) parts = 1;
  k_scan_reduce<<<parts, SCAN_THREADS, 0, st>>>(in, n, partial, ctl);
  k_scan_partials<<<1, 1024, 0, st>>>(partial, parts, total, 0x7FFFFFFF, 0, 0, ctl);
  k_scan_apply<<<parts, SCAN_THREADS, 0, st>>>(in, out, n, partial, ctl);
  g_launches += 3;
}

int grid_of(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g > 4096) g = 4096;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

extern "C" int lg_uf_label_static(int lattice, int L, int64_t nops, const int32_t* d_bonds,
                                  const int32_t* d_graphs, int32_t* d_labels, int64_t* nfrag,
                                  int64_t* nc, void* stream) {
  return lg_guard([&]() -> int {
    if (lattice < LG_CHAIN || lattice > LG_CUBIC || L < 2)
      return lg_fail(LG_EINVAL, "lg_uf_label_static: bad lattice");
    const int dim = lattice;
    long long N = 1;
    for (int i = 0; i < dim; ++i) { N *= L; if (N > LG_STATIC_MAX_SITES) break; }
    if (N > LG_STATIC_MAX_SITES)
      return lg_fail(LG_EBUDGET, "lg_uf_label_static: %lld sites exceed the static limit of %d",
                     N, LG_STATIC_MAX_SITES);
    if (nops < 0 || nops > LG_STATIC_MAX_OPS)
      return lg_fail(LG_EBUDGET, "lg_uf_label_static: %lld vertices exceed the static limit of %d",
                     (long long)nops, LG_STATIC_MAX_OPS);
    if (nops > 0 && (!d_bonds || !d_graphs)) return lg_fail(LG_EINVAL, "null input");
    if (!d_labels) return lg_fail(LG_EINVAL, "null output");
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)N, nb = n * dim, nv = (int)nops, ns = 2 * nv + n, nf = n + nv;

    Carve cv{static_cast<unsigned char*>(base)};
    Arena A{};
    A.C = 1; A.N = n; A.NB = nb;
    DChain* ch = cv.take<DChain>(1);
    A.ch = ch;
    A.inc_off = cv.take<int>(n + 1);
    A.inc = cv.take<int>((size_t)2 * dim * n);
    A.inc_side = cv.take<uint8_t>((size_t)2 * dim * n);
    A.gauge = cv.take<int8_t>(n);
    A.site_chain = cv.take<int>(n);
    A.ch_slot_off = cv.take<int>(2);
    A.spin0 = cv.take<uint8_t>(n);
    A.bond_cnt = cv.take<int>(nb);
    A.bond_ptr = cv.take<int>(nb + 1);
    A.site_cnt = cv.take<int>(n);
    A.sbase = cv.take<int>(n + 1);
    A.vtime = cv.take<uint64_t>(nv + 1);
    A.vcode = cv.take<uint8_t>(nv + 1);
    A.vslot = cv.take<int>(2 * (size_t)nv + 2);
    A.stime = cv.take<uint64_t>(ns);
    A.sinfo = cv.take<uint8_t>(ns);
    A.svert = cv.take<int>(ns);
    A.sdir = cv.take<uint8_t>(ns);
    A.parent = cv.take<int>(ns);
    Ctl* ctl = cv.take<Ctl>(1);
    A.ctl = ctl;
    int* g0flag = cv.take<int>(nv + 1);
    int* g0ord = cv.take<int>(nv + 1);
    int* g0_input = cv.take<int>(nv + 1);
    int* v_of_input = cv.take<int>(nv + 1);
    int* froot = cv.take<int>(nf);
    unsigned* minfrag = cv.take<unsigned>(ns);
    int* flag = cv.take<int>(nf);
    int* id = cv.take<int>(nf + 1);
    int* totals = cv.take<int>(4);
    const int ntiles = nv > 0 ? (nv + RS_TILE - 1) / RS_TILE : 1;
    int* hist = cv.take<int>((size_t)256 * ntiles);
    int* hoff = cv.take<int>((size_t)256 * ntiles + 1);
    // the radix sort's key / value buffers reuse arrays that are filled only after it
    int32_t* keyA = froot;
    int* valA = flag;
    int32_t* keyB = id;
    int* valB = g0_input;
    const int maxn = std::max(std::max(std::max(nb, ns), nf), 256 * ntiles) + 1;
    int* partial = cv.take<int>(maxn / SCAN_TILE + 2);
    if (cv.used > LG_STATIC_SCRATCH_BYTES)
      return lg_fail(LG_EBUDGET, "lg_uf_label_static: %zu bytes of scratch needed, %zu available",
                     cv.used, LG_STATIC_SCRATCH_BYTES);

    // everything that must start at zero (or at the atomicMin identity)
    DChain hch{};
    LG_CUDA(lg_copy_async(ch, &hch, sizeof(DChain), cudaMemcpyHostToDevice, st));
    LG_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    LG_CUDA(cudaMemsetAsync(A.bond_cnt, 0, nb * sizeof(int), st));
    LG_CUDA(cudaMemsetAsync(minfrag, 0xFF, (size_t)ns * sizeof(unsigned), st));
    LG_CUDA(cudaMemsetAsync(totals, 0, 4 * sizeof(int), st));

    ks_lattice<<<grid_of(n, 128), 128, 0, st>>>(A, dim, L);
    if (nv > 0) ks_count<<<grid_of(nv, 256), 256, 0, st>>>(A, d_bonds, d_graphs, nv, g0flag);
    static_scan(A.bond_cnt, A.bond_ptr, nb, &ctl->nv_total, partial, ctl, st);
    if (nv > 0) {
      const int g = std::min(ntiles, 4096);
      ks_radix_hist<<<g, RS_THREADS, 0, st>>>(d_bonds, nv, 0, hist, ntiles, ctl);
      static_scan(hist, hoff, 256 * ntiles, totals + 2, partial, ctl, st);
      ks_radix_scatter<<<g, RS_THREADS, 0, st>>>(d_bonds, nullptr, nv, 0, hoff, ntiles, keyA, valA, ctl);
      ks_radix_hist<<<g, RS_THREADS, 0, st>>>(keyA, nv, 8, hist, ntiles, ctl);
      static_scan(hist, hoff, 256 * ntiles, totals + 3, partial, ctl, st);
      ks_radix_scatter<<<g, RS_THREADS, 0, st>>>(keyA, valA, nv, 8, hoff, ntiles, keyB, valB, ctl);
      ks_place<<<grid_of(nv, 256), 256, 0, st>>>(A, valB, d_graphs, nv, v_of_input);
      g_launches += 5;
    }
    k_site_count<<<grid_of(n, 256), 256, 0, st>>>(A);
    static_scan(A.site_cnt, A.sbase, n, &ctl->ns_total, partial, ctl, st);
    launch_merge(2 * dim, grid_of((long long)n * 32, MERGE_WARPS * 32),
                 MERGE_WARPS * merge_smem_per_warp(MERGE_CAP), st, A, nullptr, n, MERGE_CAP);
    if (nv > 0) k_union<><<<grid_of(ns, UN_WARPS * UN_CHUNK), UN_WARPS * 32, 0, st>>>(A);
    ks_compress<<<grid_of(ns, 256), 256, 0, st>>>(A);
    static_scan(g0flag, g0ord, nv, totals, partial, ctl, st);
    g_launches += nv > 0 ? 6 : 4;  // the scans and the sort count their own
    LG_CUDA(cudaGetLastError());
    int ng0 = 0, err = 0;
    LG_CUDA(lg_copy_async(&ng0, totals, sizeof(int), cudaMemcpyDeviceToHost, st));
    LG_CUDA(lg_copy_async(&err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    LG_CUDA(cudaStreamSynchronize(st));
    if (err == 3) return lg_fail(LG_EINVAL, "lg_uf_label_static: bond or graph out of range");
    if (err) return lg_fail(LG_EITERCAP, "lg_uf_label_static: union-find failed (%d)", err);
    const int nfrag_ = n + ng0;
    ks_fragments<<<grid_of(std::max(n, nv), 256), 256, 0, st>>>(A, nv, g0flag, g0ord, v_of_input,
                                                              g0_input, froot, minfrag);
    if (ng0 > 0)
      ks_fragments_g0<<<grid_of(ng0, 256), 256, 0, st>>>(A, ng0, g0_input, v_of_input, froot, minfrag);
    ks_repflag<<<grid_of(nfrag_, 256), 256, 0, st>>>(A, nfrag_, froot, minfrag, flag);
    static_scan(flag, id, nfrag_, totals + 1, partial, ctl, st);
    ks_label<<<grid_of(nfrag_, 256), 256, 0, st>>>(A, nfrag_, froot, minfrag, id, d_labels);
    g_launches += ng0 > 0 ? 4 : 3;
    LG_CUDA(cudaGetLastError());
    int ncl = 0;
    LG_CUDA(lg_copy_async(&ncl, totals + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    LG_CUDA(cudaStreamSynchronize(st));
    if (nfrag) *nfrag = nfrag_;
    if (nc) *nc = ncl;
    return LG_OK;
  });
}
