// Host-side model setup, observables and checkpoints of the GB300 loop-cluster engine.
#pragma once
#include <cstdint>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/looper_gpu.h"
#include "lg_types.h"

int lg_fail(int code, const char* fmt, ...);

// Every int entry point of the C ABI runs its body through lg_guard, so that no C++ exception
// crosses the ABI: a failed host allocation becomes LG_ENOMEM, anything else LG_EDEVICE, each
// with its message in lg_last_error.
template <class F>
inline int lg_guard(F&& body) {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    return lg_fail(LG_ENOMEM, "host memory allocation failed");
  } catch (const std::length_error& e) {
    return lg_fail(LG_ENOMEM, "host allocation too large (%s)", e.what());
  } catch (const std::exception& e) {
    return lg_fail(LG_EDEVICE, "unexpected exception: %s", e.what());
  } catch (...) {
    return lg_fail(LG_EDEVICE, "unexpected exception");
  }
}

// One chain's model, lattice and Monte Carlo schedule, validated from lg_params.
struct ChainSpec {
  int dim = 1, L = 0, N = 0, NB = 0;   // N, NB: (virtual) sites and bonds of the simulation
  int spin2 = 1, volume = 0;           // 2S; real sites
  std::vector<int> s0, s1, gauge;
  bool bipartite = true;
  double beta = 1, jxy = 1, jz = 1, h = 0, force_scatter = 0;
  double v[4] = {0, 0, 0, 0};   // graph weights of one bond (xxz graphs 0..3)
  double W = 0;                 // sum of v
  double energy_offset = 0;     // sum over bonds of W/2 (weight_impl.h:187,199)
  int64_t therm = 0, sweeps = 0;
  uint64_t mcs = 0;             // sweeps done
  uint64_t last_nop = 0;
  int init_spins = 0;
  bool field = false, improved = true;
  bool measure_corr = false, measure_sfac = false;
  bool sse = false;              // ALGORITHM "loop; sse" (the SSE worker, k_sse)
  int corr_origin = -1;
  lg::DChain dchain{};

  int init(const lg_params& p);
  int set_beta(double b);
  double expected_vertices() const;
};

// Rebinning accumulator: up to 128 bin means, bin size doubling as data come in.
struct BinAcc {
  std::vector<double> bins;
  int64_t bin_size = 1, fill = 0, count = 0;
  double cur = 0, sum = 0, sum2 = 0;
  void push(double x);
  double mean() const { return count ? sum / count : 0.0; }
  double error() const;
  double tau() const;
};

enum {
  RAW_E = 0, RAW_E2, RAW_M, RAW_ABSM, RAW_M2, RAW_M4, RAW_CHI, RAW_SM2, RAW_SM4, RAW_SCHI,
  RAW_GM2, RAW_GCHI, RAW_NC, RAW_NOP, RAW_STIFF, NUM_RAW
};

// Exact integer sums of a vector observable over chunks of sweeps, kept as up to 128 bins
// (neighbouring bins merge when full).
struct VecAcc {
  std::vector<int64_t> sum;
  int64_t count = 0;
  std::vector<std::vector<int64_t>> bins;
  std::vector<int64_t> bin_count;
  void add_chunk(const int64_t* s, int n, int64_t sweeps);
  void mean_err(std::vector<double>& mean, std::vector<double>& err) const;
};

struct ChainAcc {
  BinAcc raw[NUM_RAW];
  VecAcc corr_disp;    // sum_i m_i m_{i+r} per displacement r
  VecAcc corr_origin;  // m_o m_j per site j
  void push(const ChainSpec& s, const uint64_t* rec);
  void report(const ChainSpec& s, lg_obs* out) const;
};

// Observable values of one sweep record (path_integral.C:827-862).
void record_values(const ChainSpec& s, const uint64_t* rec, double* v);

// The LG_NUM_VALUES per-sweep values loop_worker::run pushes (LG_VAL_*), NaN where the chain's
// estimator / lattice pushes no such entry; value_mask has bit i set for the pushed ones.
void record_scalars(const ChainSpec& s, const uint64_t* rec, double* v);
uint64_t value_mask(const ChainSpec& s);

// Checkpoint blob (path_integral.C:111-124 save/load content): a 32-byte header ("LGCK", version,
// dim, L, mcs, operator count), the spins, 12 bytes per operator, a trailing checksum: FNV-1a of
// each CHECKPOINT_BLOCK bytes before it, then FNV-1a of those block hashes.
constexpr size_t CHECKPOINT_HEAD = 32;
constexpr size_t CHECKPOINT_BLOCK = 1u << 20;
constexpr uint32_t CHECKPOINT_VERSION_PI = 3;   // path integral: off-diagonal operators and times
constexpr uint32_t CHECKPOINT_VERSION_SSE = 4;  // SSE: the whole operator string
size_t checkpoint_blocks(size_t size);
uint64_t checkpoint_block_hash(const uint8_t* buf, size_t size, size_t block);
uint64_t checkpoint_combine(const uint64_t* block_hash, size_t nblocks);
uint64_t checkpoint_checksum(const uint8_t* buf, size_t size);
uint64_t checkpoint_stored_checksum(const uint8_t* buf, size_t size);
bool checkpoint_checksum_ok(const uint8_t* buf, size_t size);
// The header and size of a blob for chain s (no checksum): operator count and sweeps done.
int checkpoint_header(const ChainSpec& s, const uint8_t* buf, size_t size, uint64_t* nops,
                      uint64_t* mcs);
void checkpoint_encode(const ChainSpec& s, const std::vector<int32_t>& spins,
                       const std::vector<int32_t>& bonds, const std::vector<double>& times,
                       std::vector<uint8_t>& blob);
int checkpoint_decode(const ChainSpec& s, const uint8_t* buf, size_t size,
                      std::vector<int32_t>& spins, std::vector<int32_t>& bonds,
                      std::vector<double>& times, uint64_t* mcs);
