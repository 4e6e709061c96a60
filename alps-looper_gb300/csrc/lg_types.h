// Plain types shared by the host engine and the device kernels.
#pragma once
#include <cstdint>

namespace lg {

constexpr int MAXZ = 24;                // largest number of (virtual) bonds at a (virtual) site:
                                        // 2 dim 2S, e.g. S = 2 on the simple-cubic lattice
// segment direction byte (sdir): the incidence index of the segment's vertex at its site in
// bits 0-4, the bond's lattice direction in bits 5-6
constexpr int SD_DSHIFT = 5;
constexpr int SD_IMASK = 31;
constexpr int REC_WORDS = 32;           // uint64 words per sweep record
constexpr int ITER_CAP = 1 << 22;       // union-find retry cap per union

enum : int { ERR_OVERFLOW = 1, ERR_ITERCAP = 2, ERR_BOUNDARY = 3 };

// Per-sweep record words: exact integer sums over the clusters of one chain.
//   NOP  operator count                      NC   cluster count
//   M0   sum (1-2c) at tau=0 (2 x M)         SM0  staggered version
//   *SQ  sum over clusters of squares        *Q   sum of 4th powers (u128: lo, hi)
//   LSQ/MSQ/SLSQ/SMSQ  sum of squared time-integrated size / magnetisation (2^-40 units, u128)
//   FLD  sum_c (flipped ? -M_c : M_c)        MA / SMA  sum of time-integrated (staggered) M
//   WSQ  sum over clusters and directions of the cluster winding squared
//   W0..W2  total winding per direction (signed)
enum : int {
  R_NOP = 0, R_NC, R_M0, R_SM0, R_M0SQ, R_N0SQ, R_SM0SQ, R_SN0SQ,
  R_M0Q = 8, R_N0Q = 10, R_SM0Q = 12, R_SN0Q = 14, R_LSQ = 16, R_MSQ = 18, R_SLSQ = 20,
  R_SMSQ = 22, R_FLD = 24, R_MA = 25, R_SMA = 26, R_WSQ = 27, R_W0 = 28, R_W1 = 29, R_W2 = 30
};

struct DChain {
  uint64_t seed;
  uint64_t T0, T1, T2, Poff;   // graph-choice thresholds on the 2^32 scale
  float inv_rate;              // 1 / (beta W_b) rounded to float; 0 when W_b == 0
  float flip_coef;             // beta * h * 2^-40 rounded to float
  int field;
  int site_off, nsites;
  int bond_off, nbonds;
  // spin correlations (correlation.h): all-pairs sums per displacement (corr_disp) and/or the
  // products with site corr_origin (>= 0), added for sweeps in [corr_from, corr_to)
  int dim, L;
  int corr_disp, corr_origin;
  uint32_t corr_from, corr_to;
  int spin2;                   // 2S: virtual sites per real site (their boundary: k_boundary)
  // the SSE worker (k_sse): beta times the total bond weight, and the diagonal graph choice of
  // graph_impl.h:297-312 on the 2^32 scale (antiparallel: graph 0 below Pd0, else 2; parallel:
  // graph 1 below Pd1, else 3)
  double sse_bw;
  uint64_t Pd0, Pd1;
};

struct Ctl {
  int err;
  int nv_total;      // vertices this sweep
  int ns_total;      // segments this sweep
  uint32_t step;     // record row of the current sweep
  int nv_cap;
  int ns_cap;
  int iter_cap;      // union-find retries per union: 0 = ITER_CAP; < 0 = none (test seam)
  int pad;
};

}  // namespace lg
