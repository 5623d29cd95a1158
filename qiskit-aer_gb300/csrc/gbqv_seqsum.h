// gbqv_seqsum.h — the reference's sequential double sums
//     s_t = fl(s_{t-1} + x_t),   x_t >= 0
// (the block sums and the block walk of QubitVector::sample_measure,
// src/simulators/statevector/qubitvector.hpp:2184-2220) evaluated many terms
// at a time, bit for bit.  __host__ __device__ so the host test suite checks
// them against plain sequential sums.
//
// While the running sum s lies in one binade [2^e, 2^(e+1)), every double
// there is a multiple of its unit in the last place g = 2^(e-52), so
//     fl(s + x) = s + g * round(x / g),
// and the rounding of x / g to an integer depends on x alone, except when
// x / g ends in exactly one half (a tie: round-half-to-even then depends on
// s).  A run of terms therefore advances s by g times the integer sum M of
// its rounded terms, exactly, provided that
//   (1) no term reaches 2^(e+1), and
//   (2) s + g*M < 2^(e+1).
// (2) covers every intermediate sum as well: the grid values rise with t,
// and each exact s_{t-1} + x_t lies below the next grid value plus g/2,
// hence below 2^(e+1).  A run that fails a condition, or that starts from
// s = 0, a subnormal, negative or non-finite s, is added one term at a time.
//
// Ties.  Write S for s / g (the significand as an integer), D_k for the sum
// of the first k terms' units with every tie rounded down, and C_k for the
// number of ties rounded up among them: S_k = S_0 + D_k + C_k.  A tie at k
// rounds up iff S_0 + D_k + C_(k-1) is odd and leaves S_k even, so
// C_k = S_0 + D_k (mod 2).  Hence a tie after an earlier tie k' rounds up
// iff D_k - D_k' is odd, whatever S_0, and only the first tie of a run
// depends on S_0: it rounds up iff S_0 + D_k is odd.  Ties thus cost no
// sequential pass: parities of prefix sums decide them all.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#endif

namespace gbqv {
namespace seq {

constexpr uint64_t kFrac = (1ULL << 52) - 1;

__host__ __device__ __forceinline__ int bexp(uint64_t b) { return (int)((b >> 52) & 0x7ff); }

// s (as bits) admits grid steps: positive, normal, finite
__host__ __device__ __forceinline__ bool grid_ok(uint64_t sb) {
  const int e = bexp(sb);
  return !(sb >> 63) && e >= 1 && e <= 2046;
}

// round(x / g) for g the unit in the last place of the binade with biased
// exponent e, a tie rounded down and flagged in `tie`; `bad` is set for
// x >= 2^(e+1) (non-finite x included) and for a negative x (-0 adds
// nothing and is fine).
__host__ __device__ __forceinline__ uint64_t grid_units(uint64_t xb, int e, bool &bad, bool &tie) {
  if (xb >> 63) {
    bad |= (xb << 1) != 0;
    return 0;
  }
  const int ex = bexp(xb);
  if (ex > e) {
    bad = true;
    return 0;
  }
  // x = mant * 2^(max(ex, 1) - 1075), g = 2^(e - 1075): x / g = mant / 2^d
  const uint64_t mant = (xb & kFrac) | (ex ? (1ULL << 52) : 0);
  const int d = e - (ex ? ex : 1);
  if (d == 0) return mant;
  if (d > 53) return 0;  // x / g < 1/2, never exactly one half
  const uint64_t half = 1ULL << (d - 1);
  const uint64_t rem = mant & ((half << 1) - 1);
  tie = rem == half;
  return (mant >> d) + (rem > half ? 1 : 0);
}

// The same on the two 32-bit words of x (hi, lo), for kernels where 64-bit
// shifts by a variable amount are costly; bit for bit grid_units.
__host__ __device__ __forceinline__ uint32_t fsr32(uint32_t lo, uint32_t hi, int s) {  // (hi:lo) >> s, s in [1, 31]
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, (unsigned)s);
#else
  return (lo >> s) | (hi << (32 - s));
#endif
}

__host__ __device__ __forceinline__ uint64_t grid_units32(uint32_t hi, uint32_t lo, int e, bool &bad, bool &tie) {
  if (hi >> 31) {
    bad |= ((hi << 1) | lo) != 0;
    return 0;
  }
  const int ex = (int)(hi >> 20);
  if (ex > e) {
    bad = true;
    return 0;
  }
  const uint32_t mh = (hi & 0xfffffu) | (ex ? 0x100000u : 0u);
  const int d = e - (ex ? ex : 1);
  if (d > 53) return 0;
  if (d == 0) return ((uint64_t)mh << 32) | lo;
  // y = mant + 2^(d-1); m = y >> d rounds half up; a tie leaves the low d
  // bits of y zero and is taken back down
  uint32_t yl, yh;
  if (d <= 32) {
    yl = lo + (1u << (d - 1));
    yh = mh + (yl < lo ? 1u : 0u);
  } else {
    yl = lo;
    yh = mh + (1u << (d - 33));
  }
  uint64_t m;
  if (d < 32) {
    tie = (yl << (32 - d)) == 0;
    m = ((uint64_t)(yh >> d) << 32) | fsr32(yl, yh, d);
  } else {
    tie = yl == 0 && (d == 32 || (yh << (64 - d)) == 0);
    m = yh >> (d - 32);
  }
  return m - (tie ? 1 : 0);
}

// The short forms for the common case, a normal positive x at 1..53
// binades below e: at 1..21 (units up to 2^52) one 64-bit add of the half
// unit on the two words and a funnel shift; at 22..53 (units below 2^32) the
// top 32 bits of the significand plus a zero test of the 21 below.  Every
// other x takes grid_units32.  Bit for bit grid_units.
__host__ __device__ __forceinline__ uint64_t grid_units_fast(uint32_t hi, uint32_t lo, int e, bool &bad,
                                                             bool &tie) {
  const int ex = (int)(hi >> 20);  // the sign bit sends negative x to the general form
  const int d = e - ex;
  if (ex >= 1 && (unsigned)(d - 1) < 53u) {
    const uint32_t mh = (hi & 0xfffffu) | 0x100000u;
    if (d <= 21) {
      const uint32_t yl = lo + (1u << (d - 1)), yh = mh + (yl < lo ? 1u : 0u);
      tie = (yl << (32 - d)) == 0;
      return ((((uint64_t)(yh >> d)) << 32) | fsr32(yl, yh, d)) - (tie ? 1 : 0);
    }
    const uint32_t z = fsr32(lo, mh, 21);  // significand >> 21
    const uint32_t h = z >> (d - 22);      // h & 1: the half bit
    tie = (h & 1u) && (z & ((1u << (d - 22)) - 1u)) == 0 && (lo & 0x1fffffu) == 0;
    return (h >> 1) + ((h & 1u) && !tie ? 1u : 0u);
  }
  return grid_units32(hi, lo, e, bad, tie);
}

// fl(a + b) for doubles a, b >= 0 given as bits, rounded to nearest even, in
// integer arithmetic (an add on the FP64 pipe, moved to the integer pipe):
// significands aligned with 10 guard bits and a sticky bit, added,
// renormalised and rounded.  False where the hardware add is wanted: a
// subnormal b other than zero, an infinite, NaN or negative operand.
__host__ __device__ __forceinline__ bool add_nonneg(uint64_t a, uint64_t b, uint64_t &r) {
  if (a < b) {  // a >= b: bit order is value order for non-negative doubles
    const uint64_t t = a;
    a = b;
    b = t;
  }
  const int ea = (int)(a >> 52), eb = (int)(b >> 52);
  if (ea >= 2047) return false;  // a infinite, NaN or negative (b > a as bits then)
  if (b == 0) {
    r = a;
    return true;
  }
  if (eb == 0) return false;
  const int d = ea - eb;
  if (d > 60) {  // b below 2^-8 units of a: rounds to a
    r = a;
    return true;
  }
  const uint64_t ma = ((a & kFrac) | (1ULL << 52)) << 10;  // leading bit 62
  const uint64_t mb0 = ((b & kFrac) | (1ULL << 52)) << 10;
  const uint64_t mb = d ? mb0 >> d : mb0;
  bool sticky = d ? (mb0 << (64 - d)) != 0 : false;
  uint64_t sum = ma + mb;
  int e = ea;
  if (sum >> 63) {
    sticky |= (sum & 1) != 0;
    sum >>= 1;
    ++e;
  }
  uint64_t m = sum >> 10;  // 53 bits
  const uint32_t g = (uint32_t)(sum & 0x3ff);
  if (g > 0x200 || (g == 0x200 && (sticky || (m & 1)))) ++m;
  if (m >> 53) {
    m >>= 1;
    ++e;
  }
  r = e >= 2047 ? 0x7ffULL << 52 : ((uint64_t)e << 52) | (m & kFrac);
  return true;
}

// Tie bookkeeping of a step from bit masks, terms in groups of 32 (term
// 32 u + l is bit l of group u): tm[u] marks the ties, om[u] the odd units
// (ties rounded down).  Returns the number of ties after the first that
// round up (each one whose rounded-down prefix parity differs from that of
// the tie before it), has_tie, and fp = the prefix parity at the first tie.
// Prefix parities by a prefix xor of om; the parity of the tie before each
// position by a doubling fill (log2 32 steps) that copies each tie's parity
// forward over the positions without a tie.
__host__ __device__ __forceinline__ uint32_t prefix_xor32(uint32_t x) {
  x ^= x << 1;
  x ^= x << 2;
  x ^= x << 4;
  x ^= x << 8;
  x ^= x << 16;
  return x;
}
__host__ __device__ __forceinline__ uint32_t popc32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__popc(x);
#else
  return (uint32_t)__builtin_popcount(x);
#endif
}
template <int G>
__host__ __device__ __forceinline__ uint32_t tie_rounds(const uint32_t (&tm)[G], const uint32_t (&om)[G], bool &has_tie,
                                                        bool &fp) {
  uint32_t extra = 0, odd_before = 0, prev_par = 0;
  bool have_prev = false;
  has_tie = false;
  fp = false;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int u = 0; u < G; ++u) {
    const uint32_t T = tm[u];
    const uint32_t Px = prefix_xor32(om[u]) ^ (odd_before ? 0xffffffffu : 0u);  // parity at each position
    if (T) {
      uint32_t val = Px & T, hv = T;  // the last tie's parity at or below each position
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
      for (int sh = 1; sh < 32; sh <<= 1) {
        val |= (val << sh) & ~hv;
        hv |= hv << sh;
      }
      const uint32_t carry = have_prev ? 0xffffffffu : 0u;
      const uint32_t hv_prev = (hv << 1) | carry;  // a tie strictly before the position
      const uint32_t f_prev = (val << 1) | (~(hv << 1) & (prev_par ? carry : 0u));
      extra += popc32(T & hv_prev & (Px ^ f_prev));
#ifdef __CUDA_ARCH__
      const int low = __ffs(T) - 1, high = 31 - __clz(T);
#else
      const int low = __builtin_ctz(T), high = 31 - __builtin_clz(T);
#endif
      if (!has_tie) {
        fp = (Px >> low) & 1;
        has_tie = true;
      }
      prev_par = (Px >> high) & 1;
      have_prev = true;
    }
    odd_before ^= popc32(om[u]) & 1;
  }
  return extra;
}

// s += g * M when the result stays below 2^(e+1); false (s unchanged) if not
__host__ __device__ __forceinline__ bool grid_add(uint64_t &sb, uint64_t M) {
  const uint64_t f = (sb & kFrac) + M;
  if (f > kFrac) return false;
  sb = (sb & ~kFrac) | f;
  return true;
}

}  // namespace seq
}  // namespace gbqv
