// gbqv_ozaki.h — exact digit-slice arithmetic for complex128 gates on tensor
// cores (the "Ozaki" error-free splitting, Ozaki et al., Numer. Algorithms
// 59 (2012)), written as __host__ __device__ helpers so the host test suite
// can check them bit for bit.
//
// A real value x of a column (the 2^(k+1) real parts of one gate group) is
// written against the column's exponent E (max over the column of the
// exponent of 2^e > |x|):
//     x ~= sum_{s=0..5} d_s * 2^(40 - 8 s) * 2^(E - 1071)
// with balanced digits d_0 in [0, 256], d_1..5 in [-128, 127] (times the
// sign of x): its significand aligned to the column maximum, rounded to 48
// bits (truncated to 48 bits in the tcgen05 kernels' state split).
// Matrix rows get the same treatment with their own row exponent R.  Every
// product of two digits is <= 2^16, a dot product over K reals is
// <= K * 2^16 (level 0) or <= K * 2^15 (levels >= 1, one digit is
// balanced), and level l = s + t sums min(l, 5) + 1 such products: for
// K <= 64 (gates of up to 5 qubits) every level sum stays below 2^24, so
// FP32 accumulation on a tensor core is exact.  Levels
// 0..5 are recombined exactly in int64:
//     v = sum_l T_l * 2^(8 (5 - l))   (|v| < 2^63)
// and y = v * 2^(R + E - 2102), rounded once to double.  The dropped levels
// (l >= 6) and the 5 truncated significand bits bound the error by about
// 2^-44 of (row max * column max): ~6e-14 relative to the group's largest
// amplitude, far inside the 1e-12 parity tolerance.
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
namespace oz {

constexpr int kSlices = 6;
constexpr int kLevels = 6;

__host__ __device__ __forceinline__ uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  __builtin_memcpy(&b, &x, 8);
  return b;
#endif
}

__host__ __device__ __forceinline__ double bitsd(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
#endif
}

__host__ __device__ __forceinline__ int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

// Exponent key of |x|: the e with 2^(e-1) <= |x| < 2^e for normal x, as a
// biased value (biased exponent field + 1); 0 for zero / subnormal.
__host__ __device__ __forceinline__ int exp_key(double x) {
  const int ex = (int)((dbits(x) >> 52) & 0x7ff);
  return ex == 0 ? 0 : ex + 1;
}

// Balanced digits of x against the column key E (E >= exp_key(x)): writes
// d[0] in [0, 256] and d[1..5] in [-128, 127] (then all times the sign of x).
__host__ __device__ __forceinline__ void split6(double x, int E, int32_t *d) {
  const uint64_t b = dbits(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  uint64_t m = ex ? ((b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) : 0;  // subnormals flush to 0
  // x = m * 2^(ex - 1075); align to the column top 2^(E - 1023): shift by (E - 1) - ex
  const int sh = (E - 1) - ex;
  m = (sh >= 53 || m == 0) ? 0 : (m >> sh);
  const uint64_t a = (m + 16) >> 5;  // the top 48 of the 53 aligned bits, rounded (<= 2^48)
  // balanced base-256 digits: adding 128 at digits 1..5 lets one 64-bit add
  // carry for all of them; digit s is then the byte minus 128
  const uint64_t bsum = a + 0x8080808080ULL;
  int32_t dd[6];
  dd[0] = (int32_t)(bsum >> 40);  // <= 256
#pragma unroll
  for (int s = 1; s < 6; ++s) dd[s] = (int32_t)((bsum >> (40 - 8 * s)) & 255u) - 128;
  const int32_t sg = (b >> 63) ? -1 : 1;
#pragma unroll
  for (int s = 0; s < 6; ++s) d[s] = sg * dd[s];
}

// Round a signed int64 times 2^scale to the nearest double (ties to even).
__host__ __device__ __forceinline__ double i64_to_double(int64_t v, int scale) {
  if (v == 0) return 0.0;
  const uint64_t neg = v < 0 ? 1 : 0;
  uint64_t u = neg ? (uint64_t)(-v) : (uint64_t)v;
  const int lz = clz64(u);
  const int top = 63 - lz;  // index of the leading bit
  uint64_t mant;
  int e = top;              // value = 1.mant * 2^(top + scale)
  if (top > 52) {
    const int drop = top - 52;
    mant = u >> drop;
    const uint64_t rem = u & ((1ULL << drop) - 1), half = 1ULL << (drop - 1);
    if (rem > half || (rem == half && (mant & 1))) {
      ++mant;
      if (mant == (1ULL << 53)) {
        mant >>= 1;
        ++e;
      }
    }
  } else {
    mant = u << (52 - top);
  }
  const int biased = e + scale + 1023;
  if (biased <= 0) return 0.0;  // below the normal range: |y| < 2^-1022, flush
  return bitsd((neg << 63) | ((uint64_t)biased << 52) | (mant & 0xFFFFFFFFFFFFFULL));
}

// Scale exponent of the recombined v for a row key R and column key E:
// x = a48 * 2^(E - 1 - 1023 - 47) per input, matrix likewise; the product of
// the two level-0 weights 2^40 * 2^40 is folded into v's 2^(8*(5-l)) shifts.
__host__ __device__ __forceinline__ int out_scale(int R, int E) {
  // input unit: 2^(E - 1 - 1023 - 47) per unit of a48; a48 = sum d_s 2^(40-8s)
  // => per digit unit at level s: 2^(40-8s) * 2^(E - 1071)
  // product of row digit t and column digit s: 2^(80 - 8l) * 2^(R - 1071 + E - 1071)
  // v = sum_l T_l 2^(8(5-l)) = sum_l T_l 2^(40 - 8l)  => y = v * 2^(40) * 2^(R + E - 2142)
  return R + E - 2142 + 40;
}


// ---- signed digits (tcgen05 kernel) ----
// Same value x ~= a * 2^(E - 1071) with a the aligned significand rounded to
// 48 bits (ties away from zero), but signed: returns bsum = a + 0x8080808080
// so that digit 0 = bsum >> 40 (arithmetic, in [-256, 256]) and digit s =
// byte (5 - s) of bsum minus 128 (in [-128, 127]) for s = 1..5, i.e.
//     a = sum_s d_s * 2^(40 - 8 s).
// Rounding and the sign come from one identity: with t the significand
// shifted right by one bit more than needed and S the sign mask (0 or -1),
// (t ^ S) + 1 is t + 1 for S = 0 and -t for S = -1, and halving
// 2 * 0x8080808080 + that gives C + round(t / 2) or C - round(t / 2).
__host__ __device__ __forceinline__ int64_t split_bsum(double x, int E) {
  const uint64_t b = dbits(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  int sh = E + 3 - ex;
  sh = sh > 63 ? 63 : sh;
  sh = ex == 0 ? 63 : sh;  // zero and subnormals give digit 0
  const uint64_t m = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const uint64_t t = m >> sh;
  const uint64_t sgn = (uint64_t)((int64_t)b >> 63);
  return (int64_t)((t ^ sgn) + (1ULL + 2ULL * 0x8080808080ULL)) >> 1;
}

__host__ __device__ __forceinline__ void bsum_digits(int64_t bs, int32_t *d) {
  d[0] = (int32_t)(bs >> 40);
#pragma unroll
  for (int s = 1; s < 6; ++s) d[s] = (int32_t)((bs >> (40 - 8 * s)) & 255) - 128;
}

// ---- the tcgen05 kernel's arithmetic (host + device, bit-identical) ----
// PTX shifts clamp the shift amount to the register width; the host
// versions do the same so both sides agree for every input.
__host__ __device__ __forceinline__ uint64_t shr64(uint64_t x, uint32_t s) {
#ifdef __CUDA_ARCH__
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
#else
  return s >= 64 ? 0 : x >> s;
#endif
}
__host__ __device__ __forceinline__ uint64_t shl64(uint64_t x, uint32_t s) {
#ifdef __CUDA_ARCH__
  uint64_t r;
  asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
#else
  return s >= 64 ? 0 : x << s;
#endif
}

// Digit word of |x| against the column key E (E4 = E + 4), given x's biased
// exponent field ex: the aligned significand truncated to 48 bits (a <
// 2^48, x ~= sign * a * 2^(E - 1071); truncation toward zero is symmetric
// in the sign, so the state's phases carry no bias, and exact values stay
// exact) plus 0x8080808080 + 0x6600 * 2^40, so that bytes 0..3 and 4 are
// digits 5..2 and 1 plus 128 and bits 40..55 are the fp16 bits of 1536 +
// d_0 (d_0 in [0, 256]); the digits of x are these times the sign of x
// (balanced digits negate digit by digit).  One 64-bit add of a constant
// makes the balanced digits.  Zeros (ex = 0) give digit 0 whenever E >= 49;
// groups whose largest entry is below 2^-974 are the only ones where a zero
// turns into a value of order 2^-1022.
constexpr uint64_t kSplitK = 0x8080808080ULL + (0x6600ULL << 40);

__host__ __device__ __forceinline__ uint64_t split_word_abs(double x, uint32_t ex, uint32_t E4) {
  const uint64_t m = (dbits(x) & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  return shr64(m, E4 - ex) + kSplitK;
}

// The same word with two 32-bit funnel shifts, for the common case of a
// non-zero x whose shift E4 - ex is at most 31 (x within 2^-26 of its
// group's largest entry): xhi, xlo are the two words of x's bits.  Bit for
// bit equal to split_word_abs there (checked on the host for every shift).
__host__ __device__ __forceinline__ uint32_t funnel_r(uint32_t lo, uint32_t hi, uint32_t s) {  // s in [0, 31]
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, s);
#else
  return s == 0 ? lo : (lo >> s) | (hi << (32 - s));
#endif
}

__host__ __device__ __forceinline__ uint64_t split_word_abs_near(uint32_t xhi, uint32_t xlo, uint32_t s) {
  const uint32_t mh = (xhi & 0xFFFFFu) | 0x100000u;
  const uint64_t t = ((uint64_t)(mh >> s) << 32) | funnel_r(xlo, mh, s);
  return t + kSplitK;
}

// Signed digits of x from its word (host side of the kernel's fp16 planes).
__host__ __device__ __forceinline__ void word_digits(uint64_t w, bool negative, int32_t *d) {
  d[0] = (int32_t)((w >> 40) & 0xFFFF) - 0x6600;
#pragma unroll
  for (int s = 1; s < 6; ++s) d[s] = (int32_t)((w >> (40 - 8 * s)) & 255) - 128;
  if (negative)
#pragma unroll
    for (int s = 0; s < 6; ++s) d[s] = -d[s];
}

// Six exact level sums to the output double, v * 2^(ebase - 1085) with
// v = sum_l T_l 2^(40 - 8 l), from the fp32 words u_l = bits(1.5 * 2^23 +
// T_l) = 0x4B400000 + T_l (exact for |T_l| <= 2^22: the sum stays in [2^23,
// 2^24], spacing 1).  The words pair up without wrapping (257 * 0x4B400000
// mod 2^32 +- 2^30 stays inside [0, 2^32)), so one 64-bit constant removes
// all biases.  |v| is taken in ones' complement (|v| - 1 for v < 0) and its
// 53 leading bits are kept (truncation); both errors are below 2^-52 of the
// result or 2^-55 of row max x column max.  Zero and results below 2^-1022
// give 0.  When the high word of |v| is non-zero (every output above 2^-23
// of row max x column max) and ebase >= 32, the normalisation is two 32-bit
// funnel shifts and no range check is needed; the other path gives the same
// bits.
__host__ __device__ __forceinline__ uint32_t funnel_l(uint32_t lo, uint32_t hi, uint32_t s) {  // s in [0, 31]
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, s);
#else
  return s == 0 ? hi : (hi << s) | (lo >> (32 - s));
#endif
}

// The two steps separately (the tcgen05 epilogue checks the fast path's
// condition for a whole chunk of outputs at once): words -> the ones'
// complement magnitude (ah, al) of v and its sign mask sg, then the double.
// v itself (two's complement, as its two words)
__host__ __device__ __forceinline__ void words_to_v(uint32_t u0, uint32_t u1, uint32_t u2, uint32_t u3, uint32_t u4,
                                                    uint32_t u5, uint32_t &vh, uint32_t &vl) {
  constexpr uint32_t kPair = 257u * 0x4B400000u;
  constexpr uint64_t kBias = (uint64_t)kPair * 0x100010001ULL;  // kPair * (2^32 + 2^16 + 1) mod 2^64
  const uint32_t p01 = u0 * 256u + u1, p23 = u2 * 256u + u3, p45 = u4 * 256u + u5;
  // v = p01 2^32 + p23 2^16 + p45 - kBias: the register pair (p01, p45) plus one wide multiply-add
  const uint64_t v = ((((uint64_t)p01 << 32) | p45) + (uint64_t)p23 * 0x10000u) - kBias;
  vh = (uint32_t)(v >> 32);
  vl = (uint32_t)v;
}

__host__ __device__ __forceinline__ void words_to_mag(uint32_t u0, uint32_t u1, uint32_t u2, uint32_t u3, uint32_t u4,
                                                      uint32_t u5, uint32_t &ah, uint32_t &al, uint32_t &sg) {
  uint32_t vh, vl;
  words_to_v(u0, u1, u2, u3, u4, u5, vh, vl);
  sg = (uint32_t)((int32_t)vh >> 31);
  ah = vh ^ sg;
  al = vl ^ sg;
}

// The double v * 2^(ebase - 1085) through the int64 -> double conversion
// (rounded to nearest) and an add to its exponent field, escale = (ebase -
// 1085) * 2^20: for |v| >= 2^32 (the high word of v neither 0 nor -1) and
// ebase >= 32, where the scaled exponent stays in the normal range.  The
// conversion runs on the FP64 pipe, the integer path (mag_to_double_fast)
// on the integer pipe; the two agree to the last bit but one (rounding vs
// truncation).
__host__ __device__ __forceinline__ double v_to_double_cvt(uint32_t vh, uint32_t vl, int escale) {
  const int64_t v = (int64_t)(((uint64_t)vh << 32) | vl);
#ifdef __CUDA_ARCH__
  const double d = __ll2double_rn((long long)v);
  return __hiloint2double(__double2hiint(d) + escale, __double2loint(d));
#else
  const uint64_t b = dbits((double)v);
  return bitsd(b + ((uint64_t)(uint32_t)escale << 32));
#endif
}

// The double from (ah, al, sg) when ah != 0 and ebase >= 32: normalisation
// by two 32-bit funnel shifts, no range check.
__host__ __device__ __forceinline__ double mag_to_double_fast(uint32_t ah, uint32_t al, uint32_t sg, int ebase) {
  const uint32_t lz = (uint32_t)clz64((uint64_t)ah << 32);
  const uint32_t nh = funnel_l(al, ah, lz), nl = al << lz;
  const uint32_t mhi = nh >> 11, mlo = (nh << 21) | (nl >> 11);
  const uint32_t e1 = (uint32_t)(ebase - (int)lz);
  return bitsd(((uint64_t)(mhi + (e1 << 20) + (sg << 31)) << 32) | mlo);
}

// Any (ah, al, sg): the fast form when it applies, else the general 64-bit
// normalisation (zero and results below 2^-1022 give 0).
__host__ __device__ __forceinline__ double mag_to_double(uint32_t ah, uint32_t al, uint32_t sg, int ebase) {
  if (ah != 0 && ebase >= 32) return mag_to_double_fast(ah, al, sg, ebase);
  const uint64_t a = ((uint64_t)ah << 32) | al;
  const int lz = clz64(a);
  const uint64_t n = shl64(a, (uint32_t)lz);
  const int e1 = ebase - lz;
  const uint64_t bits = (n >> 11) + ((uint64_t)(((uint32_t)e1 << 20) | (sg & 0x80000000u)) << 32);
  return (a == 0 || e1 < 0) ? 0.0 : bitsd(bits);
}

__host__ __device__ __forceinline__ double words_to_double(uint32_t u0, uint32_t u1, uint32_t u2, uint32_t u3,
                                                           uint32_t u4, uint32_t u5, int ebase) {
  uint32_t ah, al, sg;
  words_to_mag(u0, u1, u2, u3, u4, u5, ah, al, sg);
  return mag_to_double(ah, al, sg, ebase);
}

// The same from fp32 level sums (the magic add done here).
__host__ __device__ __forceinline__ double levels_to_double(float t0, float t1, float t2, float t3, float t4,
                                                            float t5, int ebase) {
  auto u = [](float t) -> uint32_t {
    const float f = t + 12582912.0f;
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t r;
    __builtin_memcpy(&r, &f, 4);
    return r;
#endif
  };
  return words_to_double(u(t0), u(t1), u(t2), u(t3), u(t4), u(t5), ebase);
}

}  // namespace oz
}  // namespace gbqv
