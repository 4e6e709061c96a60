// Device numerics of the loop-cluster sweep: counter-based random numbers, the float formulas
// that turn them into imaginary-time gaps and cluster-flip decisions, and the exact
// conversions between FP64 times and integer fixed point.
//
// GB300 runs FP64 at a small fraction of its FP32/INT32 rate, so the hot path never does FP64
// arithmetic: imaginary times are FP64 values (as in the reference, time_t = double,
// loop_config.h:48) on an exact 2^-52 grid, compared as unsigned 64-bit bit patterns (non-negative
// IEEE doubles order like their bits), generated by integer accumulation and integrated in
// 2^-40 fixed point.  Every float formula below uses only correctly rounded IEEE operations
// written as explicit __f*_rn / fmaf calls, so a host implementation of the same formulas
// returns the same bits.
#pragma once
#include <cstdint>

namespace lg {

// Stream tags (third Philox counter word).
enum : uint32_t {
  TAG_PROPOSAL = 1, TAG_OFFDIAG = 2, TAG_FLIP = 3, TAG_SPIN = 4, TAG_EXCHANGE = 5, TAG_PERM = 6,
  TAG_TAIL = 7, TAG_SSE = 8
};

// Philox4x32-10 (Salmon et al., SC'11): 10 rounds of two 32x32->64 multiplies with the paper's
// constants, key bumped by the Weyl increments between rounds.
struct rnd4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ rnd4 philox(uint64_t seed, uint32_t c0, uint32_t c1,
                                                uint32_t c2, uint32_t c3) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return {c0, c1, c2, c3};
}

// (2x+1) * 2^-24 with x = the top 23 bits of w: an exact float in (0,1).
__device__ __forceinline__ float uniform_open(uint32_t w) {
  return __fmul_rn(__uint2float_rn(((w >> 9) << 1) | 1u), 5.9604644775390625e-8f);
}

// ln(u), u in (0,1]: m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1), atanh series through z^4,
// ln u = e*ln2_hi + (e*ln2_lo + ln m).
__device__ __forceinline__ float log_open(float u) {
  uint32_t b = __float_as_uint(u);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  uint32_t mb = (b & 0x7FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) { mb -= 0x00800000u; e += 1; }
  float m = __uint_as_float(mb);
  float f = __fsub_rn(m, 1.0f);
  float s = __fdiv_rn(f, __fadd_rn(2.0f, f));
  float z = __fmul_rn(s, s);
  float R = fmaf(z, 0.22222222f, 0.28571429f);
  R = fmaf(z, R, 0.4f);
  R = fmaf(z, R, 0.66666669f);
  R = __fmul_rn(z, R);
  float lnm = fmaf(s, R, __fadd_rn(s, s));
  float ef = (float)e;
  float t = fmaf(ef, 1.42860677e-06f, lnm);
  return fmaf(ef, 0.693145752f, t);
}

// The uniform of an exponential gap, -ln U of which is the gap in mean gaps.  U = (2x+1) 2^-24
// from the top 23 bits x of w; in the lowest bin (x = 0: U < 2^-23, probability 2^-23) U is
// refined by the top 23 bits t of a second word, U = (2t+1) 2^-47 (exact: a power-of-two scale).
// The largest gap is so -ln 2^-47 = 32.6 mean gaps, and a draw reaches the end of the table with
// probability 2^-47 (7e-15).  `tail` is read only in the lowest bin.
__device__ __forceinline__ float gap_uniform(uint32_t w, uint32_t tail) {
  return (w >> 9) ? uniform_open(w) : __fmul_rn(uniform_open(tail), 1.1920928955078125e-7f);
}

// The refining word of proposal k of a bond (needed in the lowest bin only, once per 2^23
// draws), kept out of line so that the common path carries no second Philox.
__device__ __noinline__ uint32_t gap_tail_word(uint64_t seed, uint32_t sweep, uint32_t bond,
                                               uint32_t k) {
  return philox(seed, sweep, bond, TAG_TAIL, k).x;
}

// exp(x), |x| <= 80 (clamped): x = k ln2 + r, degree-7 Taylor polynomial, times 2^k.
__device__ __forceinline__ float exp_clamped(float x) {
  x = fminf(fmaxf(x, -80.0f), 80.0f);
  float kf = rintf(__fmul_rn(x, 1.44269502f));
  float r = fmaf(-kf, 0.693145752f, x);
  r = fmaf(-kf, 1.42860677e-06f, r);
  float p = fmaf(r, 1.98412698e-04f, 1.38888889e-03f);
  p = fmaf(r, p, 8.33333377e-03f);
  p = fmaf(r, p, 4.16666679e-02f);
  p = fmaf(r, p, 0.166666672f);
  p = fmaf(r, p, 0.5f);
  p = fmaf(r, p, 1.0f);
  p = fmaf(r, p, 1.0f);
  int k = (int)kf;
  return __fmul_rn(p, __uint_as_float((uint32_t)(k + 127) << 23));
}

constexpr uint64_t FIX52_ONE = 1ull << 52;
constexpr uint64_t TIME_INF = ~0ull;  // sorts after every time bit pattern in [0,1)

// Gap g (float, 0 <= g < 1) on the 2^-52 grid: floor(g * 2^52) with the bits below g's float
// resolution taken from `dither`, which spreads the gap uniformly over its float ulp (times stay
// continuous at 2^-52 and two gaps coincide only with probability ~2^-52).  FIX52_ONE if g >= 1.
__device__ __forceinline__ uint64_t gap_fix52(float g, uint64_t dither) {
  uint32_t b = __float_as_uint(g);
  uint32_t ex = (b >> 23) & 0xFFu;
  if (ex == 0) return 0;
  int e = (int)ex - 127;
  if (e >= 0) return FIX52_ONE;
  uint64_t m = (uint64_t)((b & 0x7FFFFFu) | 0x800000u);
  int sh = e + 29;
  if (sh < 0) return m >> (-sh);
  return (m << sh) | (dither & ((1ull << sh) - 1));
}

// Bit pattern of the FP64 value k * 2^-52 (exact for k < 2^52).
__device__ __forceinline__ uint64_t fix52_bits(uint64_t k) {
  if (k == 0) return 0;
  int p = 63 - __clzll((long long)k);
  uint64_t mant = (k << (52 - p)) & ((1ull << 52) - 1);
  return ((uint64_t)(p - 52 + 1023) << 52) | mant;
}

// floor(t * 2^40) from the bit pattern of an FP64 time t in [0,1).
__device__ __forceinline__ int64_t bits_fix40(uint64_t b) {
  if (b == 0) return 0;
  int e = (int)((b >> 52) & 0x7FF) - 1023;
  uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
  int sh = 12 - e;
  return sh >= 64 ? 0 : (int64_t)(m >> sh);
}

}  // namespace lg
