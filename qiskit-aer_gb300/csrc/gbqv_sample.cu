// gbqv_sample.cu — sample_measure (QubitVector::sample_measure,
// src/simulators/statevector/qubitvector.hpp:2148-2228) in the reference's
// own order of floating-point operations, so that every shot is the
// reference's for the same uniform, boundaries included:
//   prob(k)  = fl(fl(re*re) + fl(im*im)) (std::real(z * conj(z)) without
//              contraction; complex64 in float, then widened), or Re rho_kk
//              for a density matrix (densitymatrix.hpp:530-534);
//   idxs[j]  = sequential sum of prob over block j (2^isz blocks of L);
//   P[j+1]   = fl(P[j] + idxs[j]), the values the block walk compares with;
//   shot r   : block j = first j with r < P[j+1] (none: the walk ends at
//              2^n, as the reference's does); then p = P[j] plus prob(k), one
//              index at a time, until r < p, stopping at 2^n - 1.
// The in-block walk is the same sequence for every shot of a block, so for
// blocks of 1024 amplitudes and more one chain per block runs it once and
// keeps every 1024th partial sum; a shot then restarts from the checkpoint
// before its hit and walks at most 1024 indices (plus the rare continuation
// past a block end that the reference's walk also makes).
//
// The sequential sums are 2^isz chains (1024 by default) of L terms each.
// For blocks longer than 1024 terms:
//   1. the probabilities are written out (8 bytes per outcome) with an
//      approximate sum per step of 256 outcomes;
//   2. prefix sums of those predict every chain's running sum at each step;
//   3. one parallel pass computes, per step and for both chains, the integer
//      sum of the step's terms on the ulp grid of the predicted running sum
//      (gbqv_seqsum.h: exact while the sum keeps its binade; a term that
//      rounds on a tie is decided by prefix parities, the first one of a
//      step by the running sum's parity when the chain reaches it);
//   4. each chain (one warp) then advances 32 steps per warp scan, adding
//      the steps' grid units where their binade was predicted right and the
//      sum stays in it, and adding term by term otherwise.
// When the probability buffer cannot be allocated, or the blocks are short,
// one thread per chain adds term by term from the state itself.
#include <algorithm>
#include <cstdint>

#include "gbqv_internal.h"
#include "gbqv_seqsum.h"

namespace gbqv {
namespace {

template <typename T>
__device__ __forceinline__ double prob_exact(const T *psi, uint64_t i, uint64_t diag_stride);

template <>
__device__ __forceinline__ double prob_exact<double2>(const double2 *psi, uint64_t i, uint64_t diag_stride) {
  if (diag_stride) return psi[i * diag_stride].x;
  const double2 a = psi[i];
  return __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y));
}

template <>
__device__ __forceinline__ double prob_exact<float2>(const float2 *psi, uint64_t i, uint64_t diag_stride) {
  if (diag_stride) return (double)psi[i * diag_stride].x;
  const float2 a = psi[i];
  return (double)__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y));
}

constexpr int kStep = 256;  // terms per grid step (one warp, 8 per lane)

__device__ __forceinline__ uint64_t umin(uint64_t a, uint64_t b) { return a < b ? a : b; }

// A float no larger than the double x (truncated significand; 0 below the
// float range): the step sums only predict the running sums' binades.
__device__ __forceinline__ float approx_float(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.0f;
  const uint32_t f = e >= 255 ? 0x7f7fffffu : ((uint32_t)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float(f | (hi & 0x80000000u));
}

// prob_exact with the final add on the integer pipe (seq::add_nonneg, the
// hardware add where it declines): the pass that writes every probability
// is otherwise bound by the FP64 pipe.
template <typename T>
__device__ __forceinline__ double prob_split(const T *psi, uint64_t i, uint64_t diag_stride) {
  return prob_exact<T>(psi, i, diag_stride);
}
template <>
__device__ __forceinline__ double prob_split<double2>(const double2 *psi, uint64_t i, uint64_t diag_stride) {
  if (diag_stride) return psi[i * diag_stride].x;
  const double2 a = psi[i];
  const double x = __dmul_rn(a.x, a.x), y = __dmul_rn(a.y, a.y);
  uint64_t r;
  if (seq::add_nonneg((uint64_t)__double_as_longlong(x), (uint64_t)__double_as_longlong(y), r))
    return __longlong_as_double((long long)r);
  return __dadd_rn(x, y);
}

// Every outcome's probability in the reference's rounding, one warp per step
// of 256 outcomes, and each step's approximate sum.
template <typename T>
__global__ void __launch_bounds__(256) k_probs_steps(const T *__restrict__ psi, uint64_t nsteps, uint64_t diag_stride,
                                                     double *__restrict__ out, float *__restrict__ stepsum) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < nsteps; t += warps) {
    float acc = 0.0f;
#pragma unroll
    for (int u = 0; u < kStep / 32; ++u) {
      const uint64_t i = t * kStep + 32 * u + lane;
      const double p = prob_split<T>(psi, i, diag_stride);
      out[i] = p;
      acc += approx_float(p);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) stepsum[t] = acc;
  }
}

// Per chain (one CTA of 256 threads): the exclusive prefix of its step sums
// (the predicted running sum at each step's start) and the chain's total.
__global__ void __launch_bounds__(256) k_step_prefix(const float *__restrict__ stepsum, uint64_t steps_per_chain,
                                                     double *__restrict__ pred, double *__restrict__ total) {
  __shared__ double wsum[8];
  const uint64_t base = (uint64_t)blockIdx.x * steps_per_chain;
  const uint64_t per = (steps_per_chain + 255) / 256;
  const uint64_t t0 = umin(threadIdx.x * per, steps_per_chain), t1 = umin(t0 + per, steps_per_chain);
  double own = 0.0;
  for (uint64_t t = t0; t < t1; ++t) own += stepsum[base + t];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  double before = incl - own;
  for (int k = 0; k < w; ++k) before += wsum[k];
  for (uint64_t t = t0; t < t1; ++t) {
    pred[base + t] = before;
    before += stepsum[base + t];
  }
  if (threadIdx.x == 255) {
    double all = 0.0;
    for (int k = 0; k < 8; ++k) all += wsum[k];
    total[blockIdx.x] = all;
  }
}

// Exclusive prefix of the chain totals (one CTA, chains <= 2^24): the
// predicted start of each block's walk.
__global__ void __launch_bounds__(1024) k_chain_prefix(const double *__restrict__ total, uint64_t nchains,
                                                       double *__restrict__ start) {
  __shared__ double wsum[32];
  const uint64_t per = (nchains + 1023) / 1024;
  const uint64_t c0 = umin(threadIdx.x * per, nchains), c1 = umin(c0 + per, nchains);
  double own = 0.0;
  for (uint64_t c = c0; c < c1; ++c) own += total[c];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  double before = incl - own;
  for (int k = 0; k < w; ++k) before += wsum[k];
  for (uint64_t c = c0; c < c1; ++c) {
    start[c] = before;
    before += total[c];
  }
}

// One thread per block reading the state itself: the block's sequential sum
// (start = 0), or the walk from P[j] with every `ck`-th partial sum stored.
template <typename T, bool CHECKPOINTS>
__global__ void __launch_bounds__(32) k_seq_blocks(const T *__restrict__ psi, uint64_t nblocks, uint64_t L,
                                                   uint64_t diag_stride, const double *__restrict__ P,
                                                   double *__restrict__ out, uint64_t ck) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nblocks) return;
  const uint64_t base = j * L;
  double s = CHECKPOINTS ? P[j] : 0.0;
  uint64_t t = 0;
  // eight loads ahead of the dependent adds
  for (; t + 8 <= L; t += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = prob_exact<T>(psi, base + t + u, diag_stride);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      s = __dadd_rn(s, v[u]);
      if (CHECKPOINTS && ((t + u + 1) & (ck - 1)) == 0) out[(base + t + u) / ck] = s;
    }
  }
  for (; t < L; ++t) {
    s = __dadd_rn(s, prob_exact<T>(psi, base + t, diag_stride));
    if (CHECKPOINTS && ((t + 1) & (ck - 1)) == 0) out[(base + t) / ck] = s;
  }
  if (!CHECKPOINTS) out[j] = s;
}

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ bool parity(uint32_t m) { return __popc(m) & 1; }

// One step's record for binade e (warp-wide; this lane holds terms 32u + lane
// as words hi[u], lo[u]): M = the grid units with ties rounded down plus the
// ties after the first that round up, decided by prefix parities from the
// warp's tie and odd-unit masks (seq::tie_rounds); has_tie and fp = whether
// the step has a tie and the parity of the rounded-down prefix up to and
// including the first one, which decides it against the running sum's
// parity.
struct StepRecord {
  uint64_t M;
  bool bad, has_tie, fp;
};

__device__ __forceinline__ StepRecord step_record(const uint32_t (&hi)[kStep / 32], const uint32_t (&lo)[kStep / 32],
                                                  int e, bool bad) {
  uint64_t m[kStep / 32], sum = 0;
  uint32_t ties = 0;
#pragma unroll
  for (int u = 0; u < kStep / 32; ++u) {
    bool tie = false;
    m[u] = seq::grid_units_fast(hi[u], lo[u], e, bad, tie);
    ties |= (tie ? 1u : 0u) << u;
    sum += m[u];
  }
  StepRecord r{0, __any_sync(kFull, bad) != 0, false, false};
  uint32_t extra = 0;
  if (__any_sync(kFull, ties != 0)) {  // warp-uniform: the ties from the masks (seq::tie_rounds)
    uint32_t tm[kStep / 32], om[kStep / 32];
#pragma unroll
    for (int u = 0; u < kStep / 32; ++u) {
      tm[u] = __ballot_sync(kFull, (ties >> u) & 1);
      om[u] = __ballot_sync(kFull, m[u] & 1);
    }
    extra = seq::tie_rounds(tm, om, r.has_tie, r.fp);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
  r.M = sum + extra;
  return r;
}

// The records of every step, for both chains of its block: the block sum
// (running sum predicted by pred[t]) and the walk (start[j] + pred[t]).  One
// record per step and chain: {M (2 words), e | bad << 16 | nonzero << 17 |
// has_tie << 18 | fp << 19}.
__global__ void __launch_bounds__(256) k_grid_units(const double *__restrict__ probs, uint64_t nsteps,
                                                    int chain_shift, const double *__restrict__ pred,
                                                    const double *__restrict__ start, uint4 *__restrict__ rec_sum,
                                                    uint4 *__restrict__ rec_walk) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < nsteps; t += warps) {
    const double pr = pred[t];
    const uint64_t b1 = (uint64_t)__double_as_longlong(pr),
                   b2 = (uint64_t)__double_as_longlong(__dadd_rn(start[t >> chain_shift], pr));
    uint32_t hi[kStep / 32], lo[kStep / 32];
    bool nz = false;
#pragma unroll
    for (int u = 0; u < kStep / 32; ++u) {
      const double x = probs[t * kStep + 32 * u + lane];
      hi[u] = (uint32_t)__double2hiint(x);
      lo[u] = (uint32_t)__double2loint(x);
      nz |= ((hi[u] << 1) | lo[u]) != 0;
    }
    nz = __any_sync(kFull, nz);
    const StepRecord r1 = step_record(hi, lo, seq::bexp(b1), !seq::grid_ok(b1));
    const StepRecord r2 = step_record(hi, lo, seq::bexp(b2), !seq::grid_ok(b2));
    if (lane == 0) {
      auto meta = [&](const StepRecord &r, uint64_t b) {
        return (uint32_t)seq::bexp(b) | (r.bad ? 1u << 16 : 0u) | (nz ? 1u << 17 : 0u) | (r.has_tie ? 1u << 18 : 0u) |
               (r.fp ? 1u << 19 : 0u);
      };
      rec_sum[t] = make_uint4((uint32_t)r1.M, (uint32_t)(r1.M >> 32), meta(r1, b1), 0u);
      rec_walk[t] = make_uint4((uint32_t)r2.M, (uint32_t)(r2.M >> 32), meta(r2, b2), 0u);
    }
  }
}


__device__ __forceinline__ uint64_t warp_incl_u64(uint64_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t u = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// The running sum s (bits, warp-uniform) after the terms held one per lane
// (x bits, in lane order), equal to sequential double additions: runs of
// terms on one grid advance by a prefix sum of their grid units; a term that
// ties, reaches the next binade or crosses it is added on its own.  `mine`
// receives the sum after this lane's term.
__device__ uint64_t add_lanes(uint64_t sb, uint64_t xb, int lane, uint64_t &mine) {
  int from = 0;
  while (from < 32) {
    int f;
    if (sb == 0) {  // 0 + x = x for the first term that is not a zero
      const unsigned nz = __ballot_sync(kFull, lane >= from && (xb << 1) != 0);
      f = nz ? __ffs(nz) - 1 : 32;
      if (lane >= from && lane < f) mine = 0;
      if (f == 32) return 0;
      sb = __shfl_sync(kFull, xb, f);
      if (lane == f) mine = sb;
      from = f + 1;
      continue;
    }
    if (seq::grid_ok(sb)) {
      bool bad = false, tie = false;
      const uint64_t m =
          lane >= from ? seq::grid_units_fast((uint32_t)(xb >> 32), (uint32_t)xb, seq::bexp(sb), bad, tie) : 0;
      const uint64_t incl = warp_incl_u64(m, lane), frac = sb & seq::kFrac;
      const unsigned viol = __ballot_sync(kFull, lane >= from && (bad || tie || frac + incl > seq::kFrac));
      f = viol ? __ffs(viol) - 1 : 32;
      if (lane >= from && lane < f) mine = (sb & ~seq::kFrac) | (frac + incl);
      sb = (sb & ~seq::kFrac) | (frac + (f ? __shfl_sync(kFull, incl, f - 1) : 0));
      if (f == 32) return sb;
    } else {
      f = from;
    }
    sb = (uint64_t)__double_as_longlong(
        __dadd_rn(__longlong_as_double((long long)sb), __longlong_as_double(__shfl_sync(kFull, (long long)xb, f))));
    if (lane == f) mine = sb;
    from = f + 1;
  }
  return sb;
}

// The chains over the probability buffer, one warp per chain (block j of
// nsteps steps of 256 terms).  32 steps at a time, one per lane: the steps
// whose record holds the running sum's binade and no tie advance together by
// a prefix sum of their grid units, up to the first step that does not
// (mispredicted binade, a tie, a term that reaches the next binade, a sum
// that crosses it), which is added term by term (add_lanes over its 256
// terms).  A zero sum stays zero over steps of zeros.  WALK starts from P[j]
// and stores the sum after every 4th step (1024 terms); otherwise the chain
// starts from 0 and stores its total.
template <bool WALK>
__global__ void __launch_bounds__(32) k_grid_chain(const double *__restrict__ probs, uint64_t nsteps,
                                                   const uint4 *__restrict__ rec, const double *__restrict__ P,
                                                   double *__restrict__ out) {
  const uint64_t j = blockIdx.x;
  const int lane = threadIdx.x;
  const uint64_t step0 = j * nsteps, ncp = nsteps / 4;
  uint64_t sb = (uint64_t)__double_as_longlong(WALK ? P[j] : 0.0);
  uint4 next = lane < nsteps ? rec[step0 + lane] : make_uint4(0, 0, 0, 0);
  for (uint64_t t0 = 0; t0 < nsteps; t0 += 32) {
    const uint4 r = next;
    if (t0 + 32 + lane < nsteps) next = rec[step0 + t0 + 32 + lane];
    const int cnt = nsteps - t0 < 32 ? (int)(nsteps - t0) : 32;
    const uint64_t M = (uint64_t)r.x | ((uint64_t)r.y << 32);
    const int e_rec = (int)(r.z & 0x7ff);
    const bool bad_rec = (r.z >> 16) & 1, nz_rec = (r.z >> 17) & 1, tie_rec = (r.z >> 18) & 1,
               fp_rec = (r.z >> 19) & 1;
    const bool ck_lane = WALK && ((t0 + lane + 1) & 3) == 0;
    int from = 0;
    while (from < cnt) {
      int f;
      if (sb == 0) {
        const unsigned nz = __ballot_sync(kFull, lane >= from && lane < cnt && nz_rec);
        f = nz ? __ffs(nz) - 1 : cnt;
        if (ck_lane && lane >= from && lane < f) out[j * ncp + ((t0 + lane + 1) >> 2) - 1] = 0.0;
      } else if (seq::grid_ok(sb)) {
        // the parity of the sum at this step's start: after the last earlier
        // step with a tie (whose end parity is its units' parity xor fp),
        // else from the batch start, flipped by every odd M in between
        const uint64_t frac = sb & seq::kFrac;
        const uint32_t range = (cnt == 32 ? kFull : (1u << cnt) - 1) & ~((1u << from) - 1);
        const bool in = (range >> lane) & 1;
        const uint32_t T = __ballot_sync(kFull, in && tie_rec), A = __ballot_sync(kFull, in && (M & 1)),
                       F = __ballot_sync(kFull, in && fp_rec);
        const uint32_t below = range & ((1u << lane) - 1), tb = T & below;
        bool pin;
        if (tb) {
          const int k = 31 - __clz(tb);
          pin = (((A ^ F) >> k) & 1) ^ parity(A & below & ~((2u << k) - 1));
        } else {
          pin = (frac & 1) ^ parity(A & below);
        }
        const bool clean = !bad_rec && e_rec == seq::bexp(sb);
        const uint64_t units = M + (tie_rec && pin != fp_rec ? 1 : 0);
        const uint64_t incl = warp_incl_u64(in && clean ? units : 0, lane);
        const unsigned viol =
            __ballot_sync(kFull, lane >= from && lane < cnt && (!clean || frac + incl > seq::kFrac));
        f = viol ? __ffs(viol) - 1 : cnt;
        if (ck_lane && lane >= from && lane < f)
          out[j * ncp + ((t0 + lane + 1) >> 2) - 1] =
              __longlong_as_double((long long)((sb & ~seq::kFrac) | (frac + incl)));
        sb = (sb & ~seq::kFrac) | (frac + (f ? __shfl_sync(kFull, incl, f - 1) : 0));
      } else {
        f = from;
      }
      if (f >= cnt) break;
      // step f, term by term
      const double *x = probs + (step0 + t0 + f) * kStep;
      uint64_t xb[kStep / 32], mine;
#pragma unroll
      for (int k = 0; k < kStep / 32; ++k) xb[k] = (uint64_t)__double_as_longlong(x[32 * k + lane]);
#pragma unroll
      for (int k = 0; k < kStep / 32; ++k) sb = add_lanes(sb, xb[k], lane, mine);
      if (WALK && lane == 0 && ((t0 + f + 1) & 3) == 0)
        out[j * ncp + ((t0 + f + 1) >> 2) - 1] = __longlong_as_double((long long)sb);
      from = f + 1;
    }
  }
  if (!WALK && lane == 0) out[j] = __longlong_as_double((long long)sb);
}

// P[0] = 0, P[j + 1] = fl(P[j] + idxs[j]): the reference's running sum,
// 32 block totals at a time (add_lanes).
__global__ void __launch_bounds__(32) k_seq_prefix(const double *__restrict__ idxs, uint64_t nblocks,
                                                   double *__restrict__ P) {
  const int lane = threadIdx.x;
  uint64_t sb = 0, mine = 0;
  if (lane == 0) P[0] = 0.0;
  for (uint64_t j0 = 0; j0 < nblocks; j0 += 32) {
    const uint64_t xb = j0 + lane < nblocks ? (uint64_t)__double_as_longlong(idxs[j0 + lane]) : 0;
    sb = add_lanes(sb, xb, lane, mine);
    if (j0 + lane < nblocks) P[j0 + lane + 1] = __longlong_as_double((long long)mine);
  }
}

// One thread per shot.  n >= isz: the block from P, the checkpoint within
// the block, then the walk; n < isz: the walk from index 0.  Probabilities
// from the buffer when there is one, else from the state.
template <typename T>
__global__ void __launch_bounds__(256) k_sample_exact(const T *__restrict__ psi, const double *__restrict__ probs,
                                                      uint64_t END, uint64_t nblocks, uint64_t L, uint64_t diag_stride,
                                                      const double *__restrict__ P, const double *__restrict__ cps,
                                                      uint64_t ck, const double *__restrict__ rnds, uint64_t shots,
                                                      uint64_t *__restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < shots; s += stride) {
    const double r = rnds[s];
    double p = 0.0;
    uint64_t k = 0;
    if (nblocks) {
      // first block j with r < P[j + 1] (P is non-decreasing)
      uint64_t lo = 0, hi = nblocks;
      while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (r < P[mid + 1]) hi = mid; else lo = mid + 1;
      }
      if (lo == nblocks) {  // past the last block: the reference's walk ends at END
        out[s] = END;
        continue;
      }
      const uint64_t j = lo;
      p = P[j];
      k = j * L;
      if (cps) {
        const uint64_t ncp = L / ck;
        const double *c = cps + j * ncp;
        // first checkpoint of the block with r < c[m]
        uint64_t a = 0, b = ncp;
        while (a < b) {
          const uint64_t mid = (a + b) >> 1;
          if (r < c[mid]) b = mid; else a = mid + 1;
        }
        if (a == ncp) {  // r falls in the rounding gap after the block: walk on
          p = c[ncp - 1];
          k = (j + 1) * L;
        } else if (a) {
          p = c[a - 1];
          k = j * L + a * ck;
        }
      }
    }
    for (; k < END - 1; ++k) {
      p = __dadd_rn(p, probs ? probs[k] : prob_exact<T>(psi, k, diag_stride));
      if (r < p) break;
    }
    out[s] = k;
  }
}

uint64_t diag_stride_of(const Device &dev) { return dev.density ? (1ULL << dev.nq) + 1 : 0; }

template <typename T>
void sample_t(Device &dev, const double *d_rnds, uint64_t shots, uint64_t *d_out, uint64_t amp_offset, int n) {
  const T *psi = reinterpret_cast<const T *>(dev.state) + amp_offset;
  const int isz = dev.sample_index_size;
  const uint64_t END = 1ULL << n;
  const uint64_t ds = diag_stride_of(dev);
  const uint64_t nblocks = n >= isz ? 1ULL << isz : 0;
  const uint64_t L = nblocks ? END >> isz : 0;
  const uint64_t ck = 1024;  // checkpoint stride of the block walk
  // blocks of up to 1024 amplitudes are walked from P[j] by each shot;
  // longer blocks keep every 1024th partial sum of the walk
  const bool use_cps = L > ck;
  const uint64_t ncps = use_cps ? END / ck : 0;
  // idxs[nblocks], P[nblocks + 1], checkpoints[END / ck]
  grow(dev.aux, dev.aux_cap, sizeof(double) * (2 * nblocks + 1 + ncps + 1));
  double *idxs = reinterpret_cast<double *>(dev.aux);
  double *P = idxs + nblocks;
  double *cps = use_cps ? P + nblocks + 1 : nullptr;
  // the probability buffer (long blocks), followed by the grid steps' data:
  // step sums, predicted running sums, chain totals and starts, and one
  // record per step for each of the two chains
  const uint64_t NS = use_cps ? END / kStep : 0;
  const size_t step_bytes = NS * (sizeof(float) + sizeof(double) + 2 * sizeof(uint4)) + 2 * nblocks * sizeof(double);
  double *probs = nullptr;
  if (use_cps) {
    try {
      probs = static_cast<double *>(grow(dev.probs, dev.probs_cap, sizeof(double) * END + step_bytes));
    } catch (const Error &) {
      cudaGetLastError();  // no room for 8 bytes per outcome: the chains read the state
      probs = nullptr;
    }
  }
  if (probs) {
    float *stepsum = reinterpret_cast<float *>(probs + END);
    double *pred = reinterpret_cast<double *>(stepsum + NS);
    double *total = pred + NS, *start = total + nblocks;
    uint4 *rec_sum = reinterpret_cast<uint4 *>(start + nblocks), *rec_walk = rec_sum + NS;
    const unsigned gs = (unsigned)std::min<uint64_t>((NS + 7) / 8, (uint64_t)sm_count() * 8);
    k_probs_steps<T><<<gs, 256, 0, dev.stream>>>(psi, NS, ds, probs, stepsum);
    check_launch("sampling probabilities");
    k_step_prefix<<<(unsigned)nblocks, 256, 0, dev.stream>>>(stepsum, NS / nblocks, pred, total);
    check_launch("sampling step prefix");
    k_chain_prefix<<<1, 1024, 0, dev.stream>>>(total, nblocks, start);
    check_launch("sampling chain prefix");
    k_grid_units<<<gs, 256, 0, dev.stream>>>(probs, NS, n - isz - 8, pred, start, rec_sum, rec_walk);
    check_launch("sampling grid units");
    k_grid_chain<false><<<(unsigned)nblocks, 32, 0, dev.stream>>>(probs, L / kStep, rec_sum, nullptr, idxs);
    check_launch("sampling block sums");
    k_seq_prefix<<<1, 32, 0, dev.stream>>>(idxs, nblocks, P);
    check_launch("sampling block prefix");
    k_grid_chain<true><<<(unsigned)nblocks, 32, 0, dev.stream>>>(probs, L / kStep, rec_walk, P, cps);
    check_launch("sampling block walk");
  } else if (nblocks) {
    const unsigned g = (unsigned)((nblocks + 31) / 32);
    k_seq_blocks<T, false><<<g, 32, 0, dev.stream>>>(psi, nblocks, L, ds, nullptr, idxs, ck);
    check_launch("sampling block sums");
    k_seq_prefix<<<1, 32, 0, dev.stream>>>(idxs, nblocks, P);
    check_launch("sampling block prefix");
    if (use_cps) {
      k_seq_blocks<T, true><<<g, 32, 0, dev.stream>>>(psi, nblocks, L, ds, P, cps, ck);
      check_launch("sampling block walk");
    }
  }
  const unsigned g2 = (unsigned)std::min<uint64_t>((shots + 255) / 256, (uint64_t)sm_count() * 16);
  k_sample_exact<T><<<std::max(g2, 1u), 256, 0, dev.stream>>>(psi, probs, END, nblocks, L, ds, P, cps, ck, d_rnds,
                                                              shots, d_out);
  check_launch("sampling search");
  // the probability buffer is kept for the next call while at least a
  // quarter of the device's memory stays free, else released (cudaFree
  // waits for the kernels above)
  if (dev.probs && dev.probs_cap > (1ULL << 30)) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < total_b / 4) {
      cudaGetLastError();
      cuda_check(cudaFree(dev.probs), "sampling buffer release");
      dev.probs = nullptr;
      dev.probs_cap = 0;
    }
  }
}

}  // namespace

void sample_measure(Device &dev, const double *d_rnds, uint64_t shots, uint64_t *d_out, uint64_t amp_offset,
                    int nbits) {
  const int n = nbits >= 0 ? nbits : (dev.density ? dev.nq : dev.n);
  if (dev.dbl)
    sample_t<double2>(dev, d_rnds, shots, d_out, amp_offset, n);
  else
    sample_t<float2>(dev, d_rnds, shots, d_out, amp_offset, n);
}

}  // namespace gbqv
