// Host check of the grid-step evaluation of sequential double sums
// (qiskit-aer_gb300/csrc/gbqv_seqsum.h): the sampler's steps of 256 terms
// (integer sums on the running sum's ulp grid, one term at a time where a
// step fails a condition) against plain in-order double additions, compared
// bit for bit after every step.  Term distributions: probabilities of random
// states, a uniform superposition, powers of two and few-bit dyadics (ties on
// most grids), complex64 probabilities (24-bit terms: ties on most steps of
// the block walk), a 2^-60..1 dynamic range, sparse terms among zeros,
// subnormals, steps that cross several binades, and negative or non-finite
// terms (density-matrix diagonals with rounding noise).
//
// Usage: seqsum_check <terms per case> <cases>; prints
// "<mismatches> <steps> <steps added one term at a time> <add_lanes
// mismatches> <32-step batch mismatches>".
// seqsum_check words <trials>: the 32-bit-word forms of the grid units
// against the 64-bit one; prints the number of differences.
// seqsum_check add <trials>: the integer add of non-negative doubles against
// the host's; prints the number of differences.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "gbqv_seqsum.h"

using namespace gbqv;

static uint64_t bits(double x) {
  uint64_t b;
  __builtin_memcpy(&b, &x, 8);
  return b;
}
static double dbl(uint64_t b) {
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
}

constexpr int kStep = 256;
static constexpr uint64_t kFracMask() { return (1ULL << 52) - 1; }

// A step's record as the grid-units kernel builds it for binade e (terms in
// order, ties rounded down): M = units + the ties after the first decided by
// prefix parities; has_tie / fp = whether there is a tie and the parity of
// the rounded-down prefix up to and including the first one.
struct Record {
  uint64_t M = 0;
  bool bad = false, nz = false, has_tie = false, fp = false;
};

static Record record_of(const double *x, int e) {
  Record r;
  bool prev_par = false, par = false;
  for (int p = 0; p < kStep; ++p) {
    const uint64_t xb = bits(x[p]);
    bool tie = false;
    const uint64_t m = seq::grid_units_fast((uint32_t)(xb >> 32), (uint32_t)xb, e, r.bad, tie);
    r.nz |= (xb << 1) != 0;
    r.M += m;
    par ^= (m & 1) != 0;
    if (tie) {
      if (r.has_tie) r.M += par != prev_par;
      else r.fp = par;
      r.has_tie = true;
      prev_par = par;
    }
  }
  return r;
}

// the same record from the kernel's masks (terms 32 u + l, seq::tie_rounds)
static Record record_bits(const double *x, int e) {
  Record r;
  uint32_t tm[kStep / 32] = {0}, om[kStep / 32] = {0};
  for (int p = 0; p < kStep; ++p) {
    const uint64_t xb = bits(x[p]);
    bool tie = false;
    const uint64_t m = seq::grid_units_fast((uint32_t)(xb >> 32), (uint32_t)xb, e, r.bad, tie);
    r.nz |= (xb << 1) != 0;
    r.M += m;
    tm[p / 32] |= (tie ? 1u : 0u) << (p % 32);
    om[p / 32] |= (uint32_t)(m & 1) << (p % 32);
  }
  r.M += seq::tie_rounds(tm, om, r.has_tie, r.fp);
  return r;
}

// the step's units for a running sum whose significand has parity `odd`
static uint64_t step_units(const Record &r, bool odd) { return r.M + (r.has_tie && (odd != r.fp) ? 1 : 0); }

// one step as the chain kernel takes it with a record of the right binade:
// returns true when it was added one term at a time
static bool grid_step(uint64_t &sb, const double *x) {
  bool one_by_one;
  if (seq::grid_ok(sb)) {
    const Record r = record_of(x, seq::bexp(sb));
    one_by_one = r.bad || !seq::grid_add(sb, step_units(r, sb & 1));
  } else if (sb == 0) {
    bool nz = false;
    for (int i = 0; i < kStep; ++i) nz |= (bits(x[i]) << 1) != 0;
    one_by_one = nz;
  } else {
    one_by_one = true;
  }
  if (one_by_one) {
    double s = dbl(sb);
    for (int i = 0; i < kStep; ++i) s = s + x[i];
    sb = bits(s);
  }
  return one_by_one;
}

// The chain kernel's 32-step batch, lane by lane: the parity of the sum at
// each step's start from the masks of tie steps, odd units and first-tie
// parities; clean steps advance by the prefix sum of their units up to the
// first violation, which is added term by term.  vals[i] = the sum after
// step i.  Records are built for the binade of the reference's own sums.
static uint64_t add_lanes_host(uint64_t sb, const uint64_t *xb, uint64_t *mine);

static uint64_t batch_host(uint64_t sb, const double *x, const Record *rec, const int *e_rec, int cnt,
                           uint64_t *vals) {
  int from = 0;
  while (from < cnt) {
    int f;
    if (sb == 0) {
      f = cnt;
      for (int l = from; l < cnt; ++l)
        if (rec[l].nz) {
          f = l;
          break;
        }
      for (int l = from; l < f; ++l) vals[l] = 0;
    } else if (seq::grid_ok(sb)) {
      uint32_t T = 0, A = 0, F = 0;
      for (int l = from; l < cnt; ++l) {
        T |= (uint32_t)rec[l].has_tie << l;
        A |= (uint32_t)(rec[l].M & 1) << l;
        F |= (uint32_t)rec[l].fp << l;
      }
      const uint64_t frac = sb & seq::kFrac;
      uint64_t acc = 0;
      f = cnt;
      for (int l = from; l < cnt; ++l) {
        const uint32_t below = (l == 0 ? 0u : (0xffffffffu >> (32 - l))) & ~((1u << from) - 1);
        const uint32_t tb = T & below;
        bool pin;
        if (tb) {
          const int k = 31 - __builtin_clz(tb);
          pin = (((A >> k) ^ (F >> k)) & 1) ^ (__builtin_popcount(A & below & ~((2u << k) - 1)) & 1);
        } else {
          pin = (frac & 1) ^ (__builtin_popcount(A & below) & 1);
        }
        const bool clean = !rec[l].bad && e_rec[l] == seq::bexp(sb);
        acc += rec[l].M + (rec[l].has_tie && (pin != rec[l].fp) ? 1 : 0);
        if (!clean || frac + acc > seq::kFrac) {
          f = l;
          break;
        }
        vals[l] = (sb & ~seq::kFrac) | (frac + acc);
      }
      if (f > from) sb = vals[f - 1];
    } else {
      f = from;
    }
    if (f >= cnt) break;
    uint64_t xs[32], mine[32];
    for (int k = 0; k < kStep / 32; ++k) {
      for (int l = 0; l < 32; ++l) xs[l] = bits(x[f * kStep + 32 * k + l]);
      sb = add_lanes_host(sb, xs, mine);
    }
    vals[f] = sb;
    from = f + 1;
  }
  return sb;
}

// The sampler's warp routine add_lanes (gbqv_sample.cu), lane by lane: 32
// terms, runs on one grid advanced by prefix sums of grid units, the first
// term that ties or leaves the binade added on its own; `mine` = the sum
// after each lane's term.
static uint64_t add_lanes_host(uint64_t sb, const uint64_t *xb, uint64_t *mine) {
  int from = 0;
  while (from < 32) {
    int f;
    if (sb == 0) {
      f = 32;
      for (int l = from; l < 32; ++l)
        if ((xb[l] << 1) != 0) {
          f = l;
          break;
        }
      for (int l = from; l < f; ++l) mine[l] = 0;
      if (f == 32) return 0;
      sb = xb[f];
      mine[f] = sb;
      from = f + 1;
      continue;
    }
    if (seq::grid_ok(sb)) {
      const uint64_t frac = sb & seq::kFrac;
      uint64_t incl[32], acc = 0;
      f = 32;
      for (int l = 0; l < 32; ++l) {
        bool bad = false, tie = false;
        acc += l >= from ? seq::grid_units_fast((uint32_t)(xb[l] >> 32), (uint32_t)xb[l], seq::bexp(sb), bad, tie) : 0;
        incl[l] = acc;
        if (l >= from && f == 32 && (bad || tie || frac + acc > seq::kFrac)) f = l;
      }
      for (int l = from; l < f; ++l) mine[l] = (sb & ~seq::kFrac) | (frac + incl[l]);
      sb = (sb & ~seq::kFrac) | (frac + (f ? incl[f - 1] : 0));
      if (f == 32) return sb;
    } else {
      f = from;
    }
    sb = bits(dbl(sb) + dbl(xb[f]));
    mine[f] = sb;
    from = f + 1;
  }
  return sb;
}

// grid_units32 and grid_units_fast against grid_units on random and
// edge-case terms and binades (the flags always, the value where `bad` is
// clear)
static long check_words(long trials, std::mt19937_64 &rng) {
  long bad_count = 0;
  for (long i = 0; i < trials; ++i) {
    uint64_t xb = rng();
    switch (i % 6) {
      case 0: xb &= ~(1ULL << 63); break;                                  // any positive
      case 1: xb = (xb & ~(0xfffULL << 52)) | ((uint64_t)(1023 - 30 + (int)(rng() % 8)) << 52); break;
      case 2: xb &= (rng() % 2) ? ~((1ULL << (rng() % 53)) - 1) : ~0ULL; xb &= ~(1ULL << 63); break;  // low zeros
      case 3: xb = (xb & (0x7ffULL << 52)) | (1ULL << (rng() % 52)); break;  // one fraction bit: ties
      case 4: xb &= (1ULL << 52) - 1; break;                                // subnormal
      default: break;                                                      // negative too
    }
    const int ex = seq::bexp(xb);
    const int e = (ex + (int)(rng() % 70) - 3 + 2048) % 2047;
    for (int de : {0, 1, 20, 21, 22, 23, 30, 31, 32, 33, 40, 52, 53, 54, 60}) {
      const int ee = (i & 1) ? e : ex + de;
      if (ee < 1 || ee > 2046) continue;
      bool b1 = false, b2 = false, t1 = false, t2 = false;
      const uint64_t m1 = seq::grid_units(xb, ee, b1, t1);
      const uint64_t m2 = seq::grid_units32((uint32_t)(xb >> 32), (uint32_t)xb, ee, b2, t2);
      bool b3 = false, t3 = false;
      const uint64_t m3 = seq::grid_units_fast((uint32_t)(xb >> 32), (uint32_t)xb, ee, b3, t3);
      if (b1 != b2 || t1 != t2 || (!b1 && m1 != m2)) ++bad_count;
      if (b1 != b3 || t1 != t3 || (!b1 && m1 != m3)) ++bad_count;
    }
  }
  return bad_count;
}

// add_nonneg against the host's double addition (round to nearest even) on
// squares of random doubles, near-ties, wide exponent gaps, zeros, values at
// the top of the range and operands it hands back to the hardware
static long check_add(long trials, std::mt19937_64 &rng) {
  long bad_count = 0;
  std::normal_distribution<double> g(0.0, 1.0);
  for (long i = 0; i < trials; ++i) {
    double x, y;
    switch (i % 8) {
      case 0: { const double a = g(rng), b = g(rng); x = a * a; y = b * b; break; }  // probabilities
      case 1: { const double a = g(rng); x = a * a; y = std::ldexp(a * a, -(int)(rng() % 64)); break; }
      case 2: x = std::ldexp(1.0, (int)(rng() % 40) - 20); y = std::ldexp(1.0 + (double)(rng() % 8), (int)(rng() % 120) - 110); break;  // near ties
      case 3: x = dbl(rng() >> 1); y = dbl(rng() >> 1); break;  // any bits, non-negative (incl. nan, inf, subnormal)
      case 4: x = std::ldexp(g(rng) * g(rng) + 1.0, 1020); y = std::ldexp(std::abs(g(rng)) + 1.0, 1020 - (int)(rng() % 3)); break;  // overflow
      case 5: x = std::abs(g(rng)); y = (rng() % 2) ? 0.0 : std::ldexp(1.0, -1074 + (int)(rng() % 60)); break;  // zero, subnormal
      case 6: { const uint64_t m = (rng() & kFracMask()) | 1; x = dbl((1023ULL << 52) | m); y = dbl(((1023ULL - 53 - (rng() % 3)) << 52) | (rng() & 7)); break; }  // ties at the unit
      default: { const float a = (float)g(rng), b = (float)g(rng); x = (double)(a * a); y = (double)(b * b); break; }
    }
    uint64_t r;
    if (seq::add_nonneg(bits(x), bits(y), r)) {
      const double want = x + y;
      if (r != bits(want) && !(std::isnan(want) && std::isnan(dbl(r)))) ++bad_count;
    }
  }
  return bad_count;
}

int main(int argc, char **argv) {
  if (argc > 1 && std::string(argv[1]) == "add") {
    std::mt19937_64 rng(7);
    printf("%ld\n", check_add(argc > 2 ? atol(argv[2]) : 1000000, rng));
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "words") {
    std::mt19937_64 rng(99);
    printf("%ld\n", check_words(argc > 2 ? atol(argv[2]) : 200000, rng));
    return 0;
  }
  const int n = argc > 1 ? atoi(argv[1]) : 65536;
  const int cases = argc > 2 ? atoi(argv[2]) : 40;
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> gauss(0.0, 1.0);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  long mismatches = 0, steps = 0, slow = 0, lane_mismatches = 0, batch_mismatches = 0;
  const int L = (n / kStep) * kStep;
  std::vector<double> x(L);
  for (int c = 0; c < cases; ++c) {
    const int kind = c % 11;
    double norm = 0;
    for (int i = 0; i < L; ++i) {
      double v = 0;
      switch (kind) {
        case 0: {  // |amplitude|^2 of a Gaussian state (normalised below)
          const double a = gauss(rng), b = gauss(rng);
          v = a * a + b * b;
          break;
        }
        case 1:  // uniform superposition
          v = 1.0 / L;
          break;
        case 2:  // powers of two
          v = std::ldexp(1.0, -(int)(rng() % 40) - 10);
          break;
        case 3:  // few-bit dyadics: ties on most grids
          v = std::ldexp((double)(1 + rng() % 7), -(int)(rng() % 30) - 14);
          break;
        case 4:  // 2^-60..1
          v = std::ldexp(uni(rng), -(int)(rng() % 60));
          break;
        case 5:  // sparse among zeros
          v = (rng() % 97 == 0) ? uni(rng) : 0.0;
          break;
        case 6:  // subnormals and tiny values
          v = (rng() % 2) ? std::ldexp(uni(rng), -1060) : std::ldexp(uni(rng), -1000);
          break;
        case 7:  // growing terms: steps that cross several binades
          v = std::ldexp(1.0 + uni(rng), i / 64 - 60);
          break;
        case 8: {  // rounding noise: a few negative and -0 terms
          const double a = gauss(rng);
          v = a * a;
          const uint64_t r = rng() % 1000;
          if (r == 0) v = -1e-20 * uni(rng);
          if (r == 1) v = -0.0;
          break;
        }
        case 10: {  // complex64 probabilities (float products, widened): ties on most steps
          const float a = (float)(gauss(rng) * 3e-5), b = (float)(gauss(rng) * 3e-5);
          v = (double)(a * a + b * b);
          break;
        }
        default: {  // probabilities of a state with one dominant block
          const double a = gauss(rng), b = gauss(rng);
          v = (a * a + b * b) * ((i / 4096) % 7 == 3 ? 1e6 : 1.0);
          break;
        }
      }
      x[i] = v;
      norm += v > 0 ? v : 0;
    }
    if (kind == 0 || kind == 9)
      for (auto &v : x) v /= norm;
    if (c % 20 == 19) x[L / 2] = INFINITY;
    // start from 0 (the block sums) and from a prefix value (the block walk)
    const double starts[3] = {0.0, uni(rng), std::ldexp(uni(rng), -(int)(rng() % 20))};
    for (double s0 : starts) {
      // the warp routine: the sum after every term
      {
        double ref = s0;
        uint64_t sb = bits(s0), xb[32], mine[32];
        for (int g = 0; g < L / 32; ++g) {
          for (int l = 0; l < 32; ++l) xb[l] = bits(x[32 * g + l]);
          sb = add_lanes_host(sb, xb, mine);
          for (int l = 0; l < 32; ++l) {
            ref = ref + x[32 * g + l];
            if (mine[l] != bits(ref) && !(std::isnan(ref) && std::isnan(dbl(mine[l])))) ++lane_mismatches;
          }
          sb = bits(ref);
        }
      }
      // the chain kernel's batches of 32 steps
      {
        const int NS = L / kStep;
        std::vector<uint64_t> want(NS);
        std::vector<int> e_rec(NS);
        double ref = s0;
        for (int st = 0; st < NS; ++st) {
          e_rec[st] = seq::bexp(bits(ref));
          for (int i = 0; i < kStep; ++i) ref = ref + x[st * kStep + i];
          want[st] = bits(ref);
        }
        std::vector<Record> rec(NS);
        for (int st = 0; st < NS; ++st) {
          rec[st] = record_of(&x[st * kStep], e_rec[st]);
          const Record rb = record_bits(&x[st * kStep], e_rec[st]);
          if (rb.M != rec[st].M || rb.has_tie != rec[st].has_tie || (rb.has_tie && rb.fp != rec[st].fp) ||
              rb.bad != rec[st].bad)
            ++batch_mismatches;
        }
        uint64_t sb = bits(s0), vals[32];
        for (int t0 = 0; t0 < NS; t0 += 32) {
          const int cnt = NS - t0 < 32 ? NS - t0 : 32;
          sb = batch_host(sb, &x[t0 * kStep], &rec[t0], &e_rec[t0], cnt, vals);
          for (int l = 0; l < cnt; ++l)
            if (vals[l] != want[t0 + l] && !(std::isnan(dbl(want[t0 + l])) && std::isnan(dbl(vals[l]))))
              ++batch_mismatches;
          sb = want[t0 + cnt - 1];
        }
      }
      double ref = s0;
      uint64_t sb = bits(s0);
      for (int st = 0; st < L / kStep; ++st) {
        for (int i = 0; i < kStep; ++i) ref = ref + x[st * kStep + i];
        slow += grid_step(sb, &x[st * kStep]);
        ++steps;
        if (sb != bits(ref) && !(std::isnan(ref) && std::isnan(dbl(sb)))) ++mismatches;
        sb = bits(ref);  // compare each step from the reference's own value
      }
    }
  }
  printf("%ld %ld %ld %ld %ld\n", mismatches, steps, slow, lane_mismatches, batch_mismatches);
  return 0;
}
