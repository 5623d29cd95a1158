// Host check of the digit-slice scheme in qiskit-aer_gb300/csrc/gbqv_ozaki.h:
// the tensor-core level sums are emulated with exact integer dot products
// (what FP32 accumulation yields for these bounded integers) and the result
// is compared against a __float128 matrix-vector product.  Prints the worst
// error relative to (row max * column max) and the worst absolute error.
// Mode "signed" (third argument) checks the tcgen05 kernel's arithmetic: the
// state's digits from split_word_abs (truncated, one unit added to the
// imaginary parts as in the kernel's fast path, sign applied per digit),
// the matrix's from split_bsum, level sums held as fp32 (|T| <= 2^22) and
// turned into the double by levels_to_double.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "gbqv_ozaki.h"

using namespace gbqv::oz;

// Mode "near": split_word_abs_near against split_word_abs, bit for bit, for
// every shift 5..31 and random magnitudes and signs.
static int check_near(int trials) {
  std::mt19937_64 rng(777);
  std::uniform_int_distribution<int> sd(5, 31);
  std::uniform_int_distribution<uint64_t> bits;
  long bad = 0;
  for (int t = 0; t < trials; ++t) {
    uint64_t b = bits(rng);
    uint32_t ex = (uint32_t)((b >> 52) & 0x7ff);
    if (ex == 0 || ex == 0x7ff) continue;  // zeros and non-finite values take the generic path
    const uint32_t s = (uint32_t)sd(rng), E4 = ex + s;
    const double x = bitsd(b);
    if (split_word_abs_near((uint32_t)(b >> 32), (uint32_t)b, s) != split_word_abs(x, ex, E4)) ++bad;
  }
  printf("%ld 0\n", bad);
  return 0;
}

// Mode "cvt": the converting output path (int64 -> double, round to
// nearest, exponent-field add) against the integer normalisation
// (truncating) for random level words whose v has |v| >= 2^32 and scales
// ebase in [32, 1100]: at most one unit in the last place plus one unit of v
// apart.  Prints the
// count of larger differences and the count of cases checked.
static int check_cvt(int trials) {
  std::mt19937_64 rng(4242);
  std::uniform_int_distribution<int32_t> td(-(1 << 22), 1 << 22);
  std::uniform_int_distribution<int> ed(32, 1100);
  long bad = 0, seen = 0;
  for (int t = 0; t < trials; ++t) {
    uint32_t u[6];
    for (auto &x : u) x = 0x4B400000u + (uint32_t)td(rng);
    uint32_t vh, vl, ah, al, sg;
    words_to_v(u[0], u[1], u[2], u[3], u[4], u[5], vh, vl);
    if (vh + 1u <= 1u) continue;
    words_to_mag(u[0], u[1], u[2], u[3], u[4], u[5], ah, al, sg);
    const int eb = ed(rng);
    const double a = v_to_double_cvt(vh, vl, (int)((uint32_t)(eb - 1085) << 20));
    const double b = mag_to_double_fast(ah, al, sg, eb);
    ++seen;
    // the integer path takes |v| - 1 for negative v (ones' complement): one
    // unit of v, 2^(ebase - 1085), besides its truncation
    const double unit = std::ldexp(1.0, eb - 1085);
    if (std::signbit(a) != std::signbit(b) || std::fabs(a - b) > std::ldexp(std::fabs(b), -51) + unit) ++bad;
  }
  printf("%ld %ld\n", bad, seen);
  return 0;
}

int main(int argc, char **argv) {
  if (argc > 3 && std::string(argv[3]) == "near") return check_near(argc > 2 ? atoi(argv[2]) : 100000);
  if (argc > 3 && std::string(argv[3]) == "cvt") return check_cvt(argc > 2 ? atoi(argv[2]) : 100000);
  const int K = argc > 1 ? atoi(argv[1]) : 32;   // reals per column
  const int trials = argc > 2 ? atoi(argv[2]) : 2000;
  const bool sgn = argc > 3 && std::string(argv[3]) == "signed";
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_int_distribution<int> ed(-60, 2);
  double worst_rel = 0, worst_abs = 0;
  for (int t = 0; t < trials; ++t) {
    std::vector<double> A(K * K), x(K);
    for (auto &a : A) a = nd(rng) / std::sqrt((double)K);
    const int mode = t % 4;
    for (int j = 0; j < K; ++j) {
      double v = nd(rng) * 1e-4;
      if (mode == 1) v = std::ldexp(nd(rng), ed(rng));          // wide dynamic range
      if (mode == 2 && j % 3 == 0) v = 0.0;                       // zeros
      if (mode == 3) v = (j == 0 ? 1.0 : nd(rng) * 1e-9);         // one dominant entry
      x[j] = v;
    }
    int E = 0;
    for (double v : x) E = E > exp_key(v) ? E : exp_key(v);
    std::vector<int64_t> dx(K * kSlices);
    for (int j = 0; j < K; ++j) {
      int32_t d[6];
      if (sgn) {
        const uint32_t ex = (uint32_t)((dbits(x[j]) >> 52) & 0x7ff);
        // the kernel's fast path adds one unit to the imaginary parts
        // (odd j) of non-zero reals
        const uint64_t w = split_word_abs(x[j], ex, (uint32_t)E + 4) + ((j & 1) && x[j] != 0.0 ? 1 : 0);
        word_digits(w, std::signbit(x[j]), d);
      } else
        split6(x[j], E, d);
      for (int s = 0; s < 6; ++s) dx[j * 6 + s] = d[s];
    }
    for (int r = 0; r < K; ++r) {
      int R = 0;
      for (int j = 0; j < K; ++j) R = R > exp_key(A[r * K + j]) ? R : exp_key(A[r * K + j]);
      std::vector<int64_t> da(K * 6);
      for (int j = 0; j < K; ++j) {
        int32_t d[6];
        if (sgn)
          bsum_digits(split_bsum(A[r * K + j], R), d);
        else
          split6(A[r * K + j], R, d);
        for (int s = 0; s < 6; ++s) da[j * 6 + s] = d[s];
      }
      int64_t v = 0;
      float Tf[kLevels];
      for (int l = 0; l < kLevels; ++l) {
        int64_t T = 0;
        for (int tt = 0; tt <= l; ++tt) {
          const int s = l - tt;
          for (int j = 0; j < K; ++j) T += da[j * 6 + tt] * dx[j * 6 + s];
        }
        if (T >= (1 << 24) || T <= -(1 << 24)) {  // FP32 accumulation would round here
          printf("level sum out of the exact range\n");
          return 1;
        }
        if (sgn && (T > (1 << 22) || T < -(1 << 22))) {  // outside the magic-add range
          printf("level sum above 2^22\n");
          return 1;
        }
        Tf[l] = (float)T;
        v += T * (int64_t(1) << (8 * (5 - l)));
      }
      double y;
      if (sgn) {
        y = (R == 0 || E == 0) ? 0.0 : levels_to_double(Tf[0], Tf[1], Tf[2], Tf[3], Tf[4], Tf[5], R + E - 1017);
      } else {
        y = (R == 0 || E == 0) ? 0.0 : i64_to_double(v, out_scale(R, E));
      }
      __float128 ref = 0;
      double amax = 0, xmax = 0;
      for (int j = 0; j < K; ++j) {
        ref += (__float128)A[r * K + j] * (__float128)x[j];
        amax = std::fmax(amax, std::fabs(A[r * K + j]));
        xmax = std::fmax(xmax, std::fabs(x[j]));
      }
      const double err = std::fabs((double)((__float128)y - ref));
      const double scale = amax * xmax;
      if (scale > 0) worst_rel = std::fmax(worst_rel, err / scale);
      worst_abs = std::fmax(worst_abs, err);
    }
  }
  printf("%.3e %.3e\n", worst_rel, worst_abs);
  return 0;
}
