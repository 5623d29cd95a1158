// gbqv_batch.cu — many independent circuit instances of uneven size in one
// persistent launch: forward pass, sampled shots, <H> and adjoint gradients
// per instance.  The reference's counterpart is the batched-shots /
// parameter-bind executor (src/simulators/batch_shots_executor.hpp:39-314,
// transpile/batch_converter.hpp), which launches one kernel per gate over a
// batch of equal-size states; here instances of different qubit counts share
// one launch.
//
// Design: a persistent kernel, one CTA per instance at a time, instances
// taken from a device work counter (largest first, so the long ones start
// early).  Each instance's gate list is cut on the host into runs whose
// qubits fit one shared-memory tile of m qubits (always including the 4 lowest
// qubits, so tiles are coalesced 16-amplitude segments); a run costs one read
// and one write of the instance's state.  The adjoint sweep walks the runs
// backwards with both psi and lambda tiles resident, reducing Im<lam|P|psi>
// for every rotation gate inside the tile before uncomputing it.  Per-instance
// start / end times come from %globaltimer for latency percentiles.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/gbqv.h"
#include "gbqv_gates.h"
#include "gbqv_internal.h"

namespace gbqv {
namespace {

#include "gbqv_fpair.cuh"

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxRunOps = 128;
constexpr int kSampleBits = 10;
constexpr int kTermCache = 128;  // Hamiltonian terms staged in shared memory per instance

enum BKind { B_RX = 0, B_RY = 1, B_RZ = 2, B_CX = 3, B_CZ = 4, B_H = 5 };

struct GateDev {
  int kind, q0, q1, param;  // param: -1 fixed, else the instance's parameter index
  double c, s;              // cos(theta/2), sin(theta/2) of rotation gates
};

struct RunDev {
  int first, count;  // gates [first, first + count) of the instance
  uint64_t tmask;    // tile qubits
};

struct TermDevB {
  uint64_t x_mask, z_mask;
  double re, im;  // coeff * (-i)^{num_y}
};

struct InstDev {
  int n, nops, nruns, nterms, nparams;
  int team;  // CTAs sharing the instance (1: one CTA); members split every run's tiles
  int op_off, run_off, term_off, grad_off;
  uint64_t psi_off, lam_off;  // element offsets in the arena
  uint64_t shots, rnd_off, smp_off;
};

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
  T r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// The register/data real of each instantiation: float (complex64), double
// (complex128 on the FP64 pipe) or a float pair (complex128 held as pairs of
// floats, ~48 bits, on the FP32 pipe: gbqv_fpair.cuh).  Conversions from
// double are explicit: a double would otherwise narrow to a float silently
// on its way to a pair.
template <typename R>
__device__ __forceinline__ R from_d(double d) {
  return (R)d;
}
template <>
__device__ __forceinline__ fpair from_d<fpair>(double d) {
  return fpair_from_double(d);
}
__device__ __forceinline__ double to_d(float v) { return (double)v; }
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(fpair v) { return fpair_to_double(v); }
__device__ __forceinline__ float shfl_xor_r(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_xor_r(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ fpair shfl_xor_r(fpair v, int o) {
  return fpair(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ fpair &operator+=(fpair &a, fpair b) {
  a = a + b;
  return a;
}

template <typename T>
__device__ __forceinline__ void cfma(T &acc, T a, T b) {
  acc.x = rfma(a.x, b.x, acc.x);
  acc.x = rfma(-a.y, b.y, acc.x);
  acc.y = rfma(a.x, b.y, acc.y);
  acc.y = rfma(a.y, b.x, acc.y);
}

template <typename T>
__device__ __forceinline__ T cplx(double re, double im) {
  T r;
  r.x = from_d<decltype(r.x)>(re);
  r.y = from_d<decltype(r.y)>(im);
  return r;
}

__device__ __forceinline__ double bsum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // thread 0
}

__device__ __forceinline__ uint32_t ins1(uint32_t i, int q) {
  const uint32_t m = (1u << q) - 1;
  return ((i & ~m) << 1) | (i & m);
}

// Apply gate g (or its inverse) to a tile; a, b are the local positions.
// MT > 0: the tile has MT qubits (compile-time trip counts, fully unrolled
// loops so that the shared-memory accesses of a thread overlap); MT = 0: m.
// gc, gs: cos(theta/2), sin(theta/2) of a rotation in the data precision
// (converted once per run: conversions and products in double would run on
// the narrow FP64 pipe for every tile).
template <typename T, int MT>
__device__ __forceinline__ void tile_gate(T *tile, int m, int kind, decltype(T::x) gc, decltype(T::x) gs, int a,
                                          int b, bool inverse) {
  using R = decltype(T::x);
  const uint32_t L = MT ? (1u << MT) : (1u << m);
  constexpr int kU = MT ? 16 : 1;
  if (kind == B_RZ) {
    // diag(e^{-i t/2}, e^{i t/2}); inverse conjugates
    const R s1 = inverse ? -gs : gs;
    T d0, d1;
    d0.x = gc;
    d0.y = -s1;
    d1.x = gc;
    d1.y = s1;
#pragma unroll kU
    for (uint32_t l = threadIdx.x; l < L; l += kBatchThreads) tile[l] = cmul(tile[l], (l >> a) & 1 ? d1 : d0);
    return;
  }
  if (kind == B_CX || kind == B_CZ) {
    const int lo = min(a, b), hi = max(a, b);
#pragma unroll kU
    for (uint32_t p = threadIdx.x; p < (L >> 2); p += kBatchThreads) {
      const uint32_t base = ins1(ins1(p, lo), hi) | (1u << a);  // control set
      const uint32_t i1 = base | (1u << b);
      if (kind == B_CX) {
        const T t0 = tile[base];
        tile[base] = tile[i1];
        tile[i1] = t0;
      } else {
        T v = tile[i1];
        v.x = -v.x;
        v.y = -v.y;
        tile[i1] = v;
      }
    }
    return;
  }
  // 2x2 matrices with real (RY, H) or real-diagonal / imaginary off-diagonal
  // (RX) entries: the zero parts of the complex products are left out (half
  // the multiply-adds; at complex128 these run on the narrow FP64 pipe)
  const R s1 = inverse ? -gs : gs;
  if (kind == B_RX) {
    // [[c, -i s], [-i s, c]]: y0 = c x0 - i s x1, y1 = -i s x0 + c x1
#pragma unroll kU
    for (uint32_t p = threadIdx.x; p < (L >> 1); p += kBatchThreads) {
      const uint32_t i0 = ins1(p, a), i1 = i0 | (1u << a);
      const T x0 = tile[i0], x1 = tile[i1];
      T y0, y1;
      y0.x = rfma(s1, x1.y, gc * x0.x);
      y0.y = rfma(-s1, x1.x, gc * x0.y);
      y1.x = rfma(s1, x0.y, gc * x1.x);
      y1.y = rfma(-s1, x0.x, gc * x1.y);
      tile[i0] = y0;
      tile[i1] = y1;
    }
    return;
  }
  R m00, m01, m10, m11;  // RY [[c, -s], [s, c]], H [[h, h], [h, -h]]
  if (kind == B_RY) {
    m00 = gc; m01 = -s1; m10 = s1; m11 = gc;
  } else {
    const R h = from_d<R>(0.70710678118654752440);
    m00 = h; m01 = h; m10 = h; m11 = -h;
  }
#pragma unroll kU
  for (uint32_t p = threadIdx.x; p < (L >> 1); p += kBatchThreads) {
    const uint32_t i0 = ins1(p, a), i1 = i0 | (1u << a);
    const T x0 = tile[i0], x1 = tile[i1];
    T y0, y1;
    y0.x = rfma(m01, x1.x, m00 * x0.x);
    y0.y = rfma(m01, x1.y, m00 * x0.y);
    y1.x = rfma(m11, x1.x, m10 * x0.x);
    y1.y = rfma(m11, x1.y, m10 * x0.y);
    tile[i0] = y0;
    tile[i1] = y1;
  }
}

// This thread's part of Im <lam| P |psi> over a tile for the generator of a
// rotation gate on local bit a, summed in the data precision (at most 2^m /
// blockDim terms per thread; the caller sums the warp and then accumulates
// in double).
template <typename T, int MT>
__device__ __forceinline__ decltype(T::x) tile_generator(const T *lam, const T *psi, int m, int kind, int a) {
  using R = decltype(T::x);
  const uint32_t L = MT ? (1u << MT) : (1u << m), bit = 1u << a;
  constexpr int kU = MT ? 16 : 1;
  R acc = R(0.0f);
#pragma unroll kU
  for (uint32_t l = threadIdx.x; l < L; l += kBatchThreads) {
    const T lv = lam[l];
    T pv;
    if (kind == B_RZ) {
      pv = psi[l];
      if (l & bit) { pv.x = -pv.x; pv.y = -pv.y; }
    } else if (kind == B_RX) {
      pv = psi[l ^ bit];
    } else {  // Y = -i X Z in the (x, z) form: phase -i, sign (-1)^{bit of l}
      const T v = psi[l ^ bit];
      const R sg = (l & bit) ? R(-1.0f) : R(1.0f);
      pv.x = sg * v.y;   // -i * v = (v.y, -v.x)
      pv.y = -sg * v.x;
    }
    // Im(conj(lv) * pv)
    acc += lv.x * pv.y - lv.y * pv.x;
  }
  return acc;
}

template <typename T, int M>
__global__ void __launch_bounds__(kBatchThreads) k_batch(const InstDev *__restrict__ insts, int ninst,
                                                         const GateDev *__restrict__ gates,
                                                         const RunDev *__restrict__ runs,
                                                         const TermDevB *__restrict__ terms, T *__restrict__ arena,
                                                         const double *__restrict__ rnds, uint64_t *__restrict__ samples,
                                                         double *__restrict__ energy, double *__restrict__ grads,
                                                         unsigned long long *__restrict__ t_start,
                                                         unsigned long long *__restrict__ t_end, int *queue, int want_grad,
                                                         const int2 *__restrict__ items, int nitems,
                                                         unsigned *__restrict__ team_bar, int *__restrict__ team_err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *tp = reinterpret_cast<T *>(smem_raw);
  T *tl = tp + (1u << M);
  uint64_t *pd_lo = reinterpret_cast<uint64_t *>(tl + (1u << M));
  uint64_t *pd_hi = pd_lo + 64;
  __shared__ double red[32];
  // per run: its gates with their tile-local bits, and per-warp sums of the
  // generator inner products (reduced over warps once per run)
  __shared__ GateDev s_g[kBatchMaxRunOps];
  __shared__ uint8_t s_a[kBatchMaxRunOps], s_b[kBatchMaxRunOps];
  __shared__ decltype(T::x) s_c[kBatchMaxRunOps], s_s[kBatchMaxRunOps];
  __shared__ double gacc[kBatchMaxRunOps][kBatchThreads / 32];
  __shared__ decltype(T::x) gaccf[kBatchMaxRunOps][kBatchThreads / 32];  // this tile group's sums, data precision
  __shared__ uint64_t s_tx[kTermCache], s_tz[kTermCache];
  __shared__ decltype(T::x) s_tc[kTermCache][2];
  __shared__ int s_idx, s_member, s_abort;
  __shared__ unsigned s_nsync;
  __shared__ int s_T[64];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int q = atomicAdd(queue, 1);
      s_idx = q < nitems ? items[q].x : ninst;
      s_member = q < nitems ? items[q].y : 0;
      s_nsync = 0;
      s_abort = 0;
    }
    __syncthreads();
    const int idx = s_idx;
    if (idx >= ninst) break;
    const int member = s_member;
    const InstDev I = insts[idx];
    const int TM = I.team;
    // Barrier of the instance's team (its members are consecutive queue
    // items, taken at about the same time): every member arrives, then all
    // go on.  Bounded: after 2 s, or when another CTA gave up, the team's
    // CTAs raise *team_err and leave the kernel; the host reports it.
    auto team_sync = [&]() -> bool {
      __syncthreads();
      if (TM == 1) return true;
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&team_bar[idx], 1u);
        const unsigned target = (unsigned)TM * (++s_nsync);
        unsigned long long t0, t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        int bad = 0;
        while (atomicAdd(&team_bar[idx], 0u) < target) {
          __nanosleep(256);
          if (*(volatile int *)team_err) { bad = 1; break; }
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
          if (t1 - t0 > 2000000000ULL) { atomicExch(team_err, 1); bad = 1; break; }
        }
        __threadfence();
        s_abort = bad;
      }
      __syncthreads();
      return !s_abort;
    };
    if (threadIdx.x == 0 && member == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      t_start[idx] = t;
    }
    T *psi = arena + I.psi_off;
    T *lam = arena + I.lam_off;
    const uint64_t N = 1ULL << I.n;
    const uint64_t tstride = (uint64_t)blockDim.x * TM;  // thread stride over the team
    const uint64_t tbase = (uint64_t)member * blockDim.x + threadIdx.x;
    for (uint64_t i = tbase; i < N; i += tstride) psi[i] = cplx<T>(i == 0 ? 1.0 : 0.0, 0.0);
    if (!team_sync()) return;
    // ---------------- runs: forward (dir = 0) and backward (dir = 1) ----------------
    for (int dir = 0; dir < 2; ++dir) {
      if (dir == 1) {
        // sampling on the final state, before the sweep uncomputes it, in
        // the reference's order of operations (QubitVector::sample_measure,
        // qubitvector.hpp:2148-2228): sequential block totals over 2^10
        // blocks, their running prefix P, then per shot the block with
        // r < P[j + 1] and the walk p = P[j] + prob(k) ... until r < p; the
        // probabilities as std::real(z * conj(z)), no contraction
        auto prob = [&](uint64_t k) -> double {
          const T a = psi[k];
          if constexpr (sizeof(T) == 8) {
            return (double)__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y));
          } else {
            const double re = to_d(a.x), im = to_d(a.y);
            return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
          }
        };
        const bool blocks = I.n >= kSampleBits;
        const uint64_t nb = blocks ? 1ULL << kSampleBits : 0, L = blocks ? N >> kSampleBits : 0;
        double *cdf = reinterpret_cast<double *>(lam);  // P[j + 1] at cdf[j]; lam is free until H psi
        if (blocks) {
          for (uint64_t j = tbase; j < nb; j += tstride) {
            double sacc = 0.0;
            for (uint64_t t = 0; t < L; ++t) sacc = __dadd_rn(sacc, prob(j * L + t));
            cdf[j] = sacc;
          }
          if (!team_sync()) return;
          if (threadIdx.x == 0 && member == 0) {
            double run = 0.0;
            for (uint64_t j = 0; j < nb; ++j) {
              run = __dadd_rn(run, cdf[j]);
              cdf[j] = run;
            }
          }
          if (!team_sync()) return;
        }
        for (uint64_t sh = tbase; sh < I.shots; sh += tstride) {
          const double r = rnds[I.rnd_off + sh];
          double p = 0.0;
          uint64_t k = 0;
          if (blocks) {
            uint64_t lo = 0, hi = nb;
            while (lo < hi) {
              const uint64_t mid = (lo + hi) >> 1;
              if (r < cdf[mid]) hi = mid; else lo = mid + 1;
            }
            if (lo == nb) {  // at or above the total: the reference's walk ends at 2^n
              samples[I.smp_off + sh] = N;
              continue;
            }
            p = lo ? cdf[lo - 1] : 0.0;
            k = lo * L;
          }
          for (; k < N - 1; ++k) {
            p = __dadd_rn(p, prob(k));
            if (r < p) break;
          }
          samples[I.smp_off + sh] = k;
        }
        if (!team_sync()) return;  // the CDF (in lambda's space) is read until here
        // lambda = H psi and <H> = Re <psi|lambda>: lambda in the data
        // precision (complex64 sums its terms in float: the FP64 pipe is
        // far narrower), <H> accumulated in double
        using Rt = decltype(T::x);
        // the coefficients in the data precision, converted once per
        // instance (a conversion from double runs on the FP64 pipe)
        const bool staged = I.nterms <= kTermCache;
        if (staged)
          for (int t = threadIdx.x; t < I.nterms; t += blockDim.x) {
            const TermDevB h = terms[I.term_off + t];
            s_tx[t] = h.x_mask;
            s_tz[t] = h.z_mask;
            s_tc[t][0] = from_d<Rt>(h.re);
            s_tc[t][1] = from_d<Rt>(h.im);
          }
        __syncthreads();
        double e_acc = 0.0;
        for (uint64_t i = tbase; i < N; i += tstride) {
          Rt ar = Rt(0.0f), ai = Rt(0.0f);
          for (int t = 0; t < I.nterms; ++t) {
            uint64_t xm, zm;
            Rt cr, ci;
            if (staged) {
              xm = s_tx[t];
              zm = s_tz[t];
              cr = s_tc[t][0];
              ci = s_tc[t][1];
            } else {
              const TermDevB h = terms[I.term_off + t];
              xm = h.x_mask;
              zm = h.z_mask;
              cr = from_d<Rt>(h.re);
              ci = from_d<Rt>(h.im);
            }
            const T a = psi[i ^ xm];
            if (__popcll(i & zm) & 1) { cr = -cr; ci = -ci; }
            ar += cr * a.x - ci * a.y;
            ai += cr * a.y + ci * a.x;
          }
          const T p = psi[i];
          e_acc += to_d(p.x * ar + p.y * ai);
          T l;
          l.x = ar;
          l.y = ai;
          lam[i] = l;
        }
        const double e = bsum(e_acc, red);
        if (threadIdx.x == 0) {
          if (TM == 1)
            energy[idx] = e;
          else
            atomicAdd(&energy[idx], e);  // zeroed before the launch
        }
        if (TM == 1)
          for (int pi = threadIdx.x; pi < I.nparams; pi += blockDim.x) grads[I.grad_off + pi] = 0.0;
        if (!team_sync()) return;
        if (!want_grad) break;
      }
      for (int rr = 0; rr < I.nruns; ++rr) {
        const RunDev R = runs[I.run_off + (dir == 0 ? rr : I.nruns - 1 - rr)];
        // tile geometry
        if (threadIdx.x == 0) {
          int j = 0;
          for (int q = 0; q < I.n; ++q)
            if ((R.tmask >> q) & 1) s_T[j++] = q;
        }
        for (int i = threadIdx.x; i < kBatchMaxRunOps * (kBatchThreads / 32); i += blockDim.x) {
          gacc[i / (kBatchThreads / 32)][i % (kBatchThreads / 32)] = 0.0;
          gaccf[i / (kBatchThreads / 32)][i % (kBatchThreads / 32)] = decltype(T::x)(0.0f);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < R.count; k += blockDim.x) {
          const GateDev g = gates[I.op_off + R.first + k];
          int a = 0, b = 0;
          for (int j = 0; j < __popcll(R.tmask); ++j) {
            if (s_T[j] == g.q0) a = j;
            if (s_T[j] == g.q1) b = j;
          }
          s_g[k] = g;
          s_a[k] = (uint8_t)a;
          s_b[k] = (uint8_t)b;
          s_c[k] = from_d<decltype(T::x)>(g.c);
          s_s[k] = from_d<decltype(T::x)>(g.s);
        }
        __syncthreads();
        const int m = __popcll(R.tmask);
        const int lo_bits = min(m, 6), hi_bits = m - lo_bits;
        for (int h = threadIdx.x; h < 64; h += blockDim.x) {
          uint64_t a = 0;
          for (int j = 0; j < lo_bits; ++j)
            if ((h >> j) & 1) a |= 1ULL << s_T[j];
          pd_lo[h] = a;
        }
        for (int h = threadIdx.x; h < (1 << hi_bits); h += blockDim.x) {
          uint64_t a = 0;
          for (int j = 0; j < hi_bits; ++j)
            if ((h >> j) & 1) a |= 1ULL << s_T[lo_bits + j];
          pd_hi[h] = a;
        }
        __syncthreads();
        const uint64_t ntiles = 1ULL << (I.n - m);
        const uint32_t L = 1u << m;
        uint64_t lt = 0;  // tiles this CTA has processed in the run
        for (uint64_t t = member; t < ntiles; t += TM, ++lt) {
          // deposit the tile id into the bits outside the tile
          uint64_t base = 0, tt = t;
          for (int q = 0; q < I.n && tt; ++q)
            if (!((R.tmask >> q) & 1)) {
              base |= (tt & 1) << q;
              tt >>= 1;
            }
          if (m == M) {  // every load of the thread issued before the first store
            constexpr int kPer = (1 << M) / kBatchThreads;
            T vp[kPer], vl[kPer];
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
              const uint32_t l = threadIdx.x + j * kBatchThreads;
              const uint64_t gi = base | pd_lo[l & 63] | pd_hi[l >> 6];
              vp[j] = psi[gi];
              if (dir == 1) vl[j] = lam[gi];
            }
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
              const uint32_t l = threadIdx.x + j * kBatchThreads;
              tp[l] = vp[j];
              if (dir == 1) tl[l] = vl[j];
            }
          } else {
            for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) {
              const uint64_t gi = base | pd_lo[l & 63] | pd_hi[l >> 6];
              tp[l] = psi[gi];
              if (dir == 1) tl[l] = lam[gi];
            }
          }
          __syncthreads();
          for (int k = 0; k < R.count; ++k) {
            const int oi = dir == 0 ? k : R.count - 1 - k;
            const GateDev &g = s_g[oi];
            const int a = s_a[oi], b = s_b[oi];
            if (dir == 1 && g.param >= 0) {
              // the warp's sum in the data precision (32 terms), then into the
              // double accumulator of the warp
              auto part = m == M ? tile_generator<T, M>(tl, tp, m, g.kind, a)
                                 : tile_generator<T, 0>(tl, tp, m, g.kind, a);
              for (int o = 16; o > 0; o >>= 1) part += shfl_xor_r(part, o);
              if ((threadIdx.x & 31) == 0) {
                // 16 tiles' warp sums in the data precision, then into double
                auto &f = gaccf[oi][threadIdx.x >> 5];
                f += part;
                if ((lt & 15) == 15) {
                  gacc[oi][threadIdx.x >> 5] += to_d(f);
                  f = decltype(T::x)(0.0f);
                }
              }
            }
            const auto gc = s_c[oi], gs = s_s[oi];
            if (m == M) {
              tile_gate<T, M>(tp, m, g.kind, gc, gs, a, b, dir == 1);
              if (dir == 1) tile_gate<T, M>(tl, m, g.kind, gc, gs, a, b, true);
            } else {
              tile_gate<T, 0>(tp, m, g.kind, gc, gs, a, b, dir == 1);
              if (dir == 1) tile_gate<T, 0>(tl, m, g.kind, gc, gs, a, b, true);
            }
            __syncthreads();
          }
#pragma unroll 8
          for (uint32_t l = threadIdx.x; l < L; l += kBatchThreads) {
            const uint64_t gi = base | pd_lo[l & 63] | pd_hi[l >> 6];
            psi[gi] = tp[l];
            if (dir == 1) lam[gi] = tl[l];
          }
          __syncthreads();
        }
        if (dir == 1 && threadIdx.x == 0)
          for (int k = 0; k < R.count; ++k) {
            const GateDev &g = s_g[k];
            if (g.param < 0) continue;
            double sum = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += gacc[k][w] + to_d(gaccf[k][w]);
            if (TM == 1)
              grads[I.grad_off + g.param] += sum;
            else
              atomicAdd(&grads[I.grad_off + g.param], sum);  // zeroed before the launch
          }
        if (!team_sync()) return;
      }
    }
    if (threadIdx.x == 0 && member == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      t_end[idx] = t;
    }
  }
}

}  // namespace
}  // namespace gbqv

using namespace gbqv;

// ------------------------------- host side -------------------------------

struct BatchInstHost {
  int n, nparams;
  std::vector<GateDev> gates;
  std::vector<RunDev> runs;
  std::vector<TermDevB> terms;
  uint64_t shots, seed;
};

struct gbqv_batch {
  bool dbl = true;
  bool fp64 = false;  // complex128 gates on the FP64 pipe instead of float pairs
  std::vector<BatchInstHost> inst;
  // device buffers
  cudaStream_t stream = nullptr;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  void *dev_blob = nullptr;
  size_t blob_bytes = 0;
  std::vector<double> energy, grads;
  std::vector<uint64_t> samples, t0, t1;
  std::vector<size_t> grad_off, smp_off;
  std::vector<size_t> order;  // device position -> instance index
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_def = nullptr;
  bool built = false;
  std::string err;
  // teams: the costliest instances (up to team_max instances whose cost is
  // at least team_frac of the largest) run on two CTAs each
  int team_max = 64;
  double team_frac = 0.5;
  void *team_blob = nullptr;  // queue items (int2), per-instance barrier counters, error word
  int nitems = 0;
};

namespace {

thread_local std::string g_berr;

template <typename F>
int bguard(F &&f) {
  try {
    f();
    return GBQV_OK;
  } catch (const Error &e) {
    set_last_error(nullptr, e.what());
    return e.code;
  } catch (const std::exception &e) {
    set_last_error(nullptr, e.what());
    return GBQV_ERR_ARG;
  }
}

int tile_bits_for(bool dbl) { return dbl ? 11 : 12; }

// Greedy run builder (same rule as the single-state scheduler): take later
// gates that touch no qubit of a skipped gate while the tile has room.  The
// gate list is rewritten in run order; runs index into it.
std::vector<RunDev> build_runs(std::vector<GateDev> &g, int n, int m) {
  std::vector<RunDev> runs;
  std::vector<char> done(g.size(), 0);
  std::vector<GateDev> out;
  size_t first = 0;
  while (true) {
    while (first < g.size() && done[first]) ++first;
    if (first >= g.size()) break;
    uint64_t T = 0;
    for (int q = 0; q < std::min(4, n); ++q) T |= 1ULL << q;
    uint64_t blocked = 0;
    RunDev r{(int)out.size(), 0, 0};
    for (size_t i = first; i < g.size(); ++i) {
      if (done[i]) continue;
      uint64_t qm = 1ULL << g[i].q0;
      if (g[i].kind == B_CX || g[i].kind == B_CZ) qm |= 1ULL << g[i].q1;
      if (qm & blocked) {
        blocked |= qm;
        continue;
      }
      const uint64_t T2 = T | qm;
      if (__builtin_popcountll(T2) <= m && r.count < kBatchMaxRunOps) {
        T = T2;
        out.push_back(g[i]);
        ++r.count;
        done[i] = 1;
      } else {
        blocked |= qm;
      }
      if (__builtin_popcountll(blocked) >= n) break;
    }
    for (int q = 0; q < n && __builtin_popcountll(T) < m; ++q) T |= 1ULL << q;
    r.tmask = T;
    runs.push_back(r);
  }
  g = out;
  return runs;
}

}  // namespace

extern "C" int gbqv_batch_create(int precision, gbqv_batch_t *out) {
  return bguard([&] {
    if (!out || (precision != GBQV_C64 && precision != GBQV_C128)) throw Error(GBQV_ERR_ARG, "bad arguments");
    auto *b = new gbqv_batch;
    b->dbl = precision == GBQV_C128;
    *out = b;
  });
}

extern "C" int gbqv_batch_destroy(gbqv_batch_t b) {
  if (!b) return GBQV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_def) cudaGraphDestroy(b->graph_def);
  if (b->arena) cudaFree(b->arena);
  if (b->dev_blob) cudaFree(b->dev_blob);
  if (b->team_blob) cudaFree(b->team_blob);
  if (b->stream) cudaStreamDestroy(b->stream);
  cudaGetLastError();
  delete b;
  return GBQV_OK;
}

extern "C" int gbqv_batch_set_teams(gbqv_batch_t b, int max_team_instances, double min_cost_fraction) {
  return bguard([&] {
    if (!b) throw Error(GBQV_ERR_ARG, "null batch");
    if (b->built) throw Error(GBQV_ERR_ARG, "teams are fixed once the batch has run");
    if (max_team_instances < 0 || max_team_instances > 64 || !(min_cost_fraction >= 0.0))
      throw Error(GBQV_ERR_ARG, "team settings out of range (at most 64 team instances)");
    b->team_max = max_team_instances;
    b->team_frac = min_cost_fraction;
  });
}

extern "C" int gbqv_batch_set_fp64(gbqv_batch_t b, int on) {
  return bguard([&] {
    if (!b) throw Error(GBQV_ERR_ARG, "null batch");
    if (b->graph) throw Error(GBQV_ERR_ARG, "the arithmetic is fixed once the batch has run");
    b->fp64 = on != 0;
  });
}

extern "C" int gbqv_batch_add(gbqv_batch_t b, int num_qubits, int ngates, const int *kinds, const uint64_t *qubits,
                              const int *param_of_gate, const double *params, int nparams, int nterms,
                              const uint64_t *tq, const int *toffsets, const char *const *labels,
                              const double *coeffs, uint64_t shots, uint64_t seed, int *index) {
  return bguard([&] {
    if (!b || b->built) throw Error(GBQV_ERR_ARG, "batch is null or already run");
    if (num_qubits < 1 || num_qubits > 30) throw Error(GBQV_ERR_ARG, "instance qubits must be 1..30");
    if (ngates < 0 || (ngates && (!kinds || !qubits || !param_of_gate))) throw Error(GBQV_ERR_ARG, "bad gate arrays");
    if (nterms < 1 || !toffsets || !labels) throw Error(GBQV_ERR_ARG, "an instance needs a Hamiltonian");
    BatchInstHost h;
    h.n = num_qubits;
    h.nparams = nparams;
    h.shots = shots;
    h.seed = seed;
    for (int i = 0; i < ngates; ++i) {
      GateDev g{kinds[i], (int)qubits[2 * i], (int)qubits[2 * i + 1], param_of_gate[i], 1.0, 0.0};
      if (g.kind < B_RX || g.kind > B_H) throw Error(GBQV_ERR_ARG, "unknown batch gate kind");
      const bool two = g.kind == B_CX || g.kind == B_CZ;
      if (g.q0 < 0 || g.q0 >= num_qubits || (two && (g.q1 < 0 || g.q1 >= num_qubits || g.q1 == g.q0)))
        throw Error(GBQV_ERR_QUBIT, "gate qubit out of range");
      if (!two) g.q1 = g.q0;
      if (g.kind <= B_RZ) {
        if (g.param < 0 || g.param >= nparams || !params) throw Error(GBQV_ERR_ARG, "rotation gates need a parameter");
        g.c = std::cos(0.5 * params[g.param]);
        g.s = std::sin(0.5 * params[g.param]);
      } else {
        g.param = -1;
      }
      h.gates.push_back(g);
    }
    for (int t = 0; t < nterms; ++t) {
      const int k = toffsets[t + 1] - toffsets[t];
      reg_t q(tq + toffsets[t], tq + toffsets[t] + k);
      for (auto x : q)
        if (x >= (uint64_t)num_qubits) throw Error(GBQV_ERR_QUBIT, "Hamiltonian qubit out of range");
      if (!labels[t] || (int)std::strlen(labels[t]) != k) throw Error(GBQV_ERR_ARG, "bad Pauli label");
      PauliMasks mk = pauli_masks(q, labels[t]);
      const cd ph = add_y_phase(mk.num_y, cd(coeffs ? coeffs[t] : 1.0, 0.0));
      h.terms.push_back(TermDevB{mk.x_mask, mk.z_mask, ph.real(), ph.imag()});
    }
    const int m = std::min(num_qubits, tile_bits_for(b->dbl));
    h.runs = build_runs(h.gates, num_qubits, m);
    if (index) *index = (int)b->inst.size();
    b->inst.push_back(std::move(h));
  });
}

namespace {

void batch_build(gbqv_batch *b) {
  const size_t ninst = b->inst.size();
  if (!ninst) throw Error(GBQV_ERR_ARG, "empty batch");
  cuda_check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
  // costliest instances first (gates x amplitudes), so the long ones start early
  auto cost = [&](size_t i) { return (double)std::max<size_t>(b->inst[i].gates.size(), 1) * std::ldexp(1.0, b->inst[i].n); };
  std::vector<size_t> order(ninst);
  for (size_t i = 0; i < ninst; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) { return cost(a) > cost(c); });
  // teams of two CTAs for the costliest instances that span at least two tiles
  const int tile_bits = b->dbl ? 11 : 12;
  std::vector<int> team(ninst, 1);
  int nteams = 0;
  for (size_t k = 0; k < ninst && nteams < b->team_max; ++k) {
    const size_t i = order[k];
    if (cost(i) < b->team_frac * cost(order[0])) break;
    if (b->inst[i].n <= tile_bits) continue;
    team[k] = 2;
    ++nteams;
  }
  std::vector<int2> items;
  for (size_t k = 0; k < ninst; ++k)
    for (int m = 0; m < team[k]; ++m) items.push_back(make_int2((int)k, m));
  b->nitems = (int)items.size();
  std::vector<InstDev> idev(ninst);
  std::vector<GateDev> gates;
  std::vector<RunDev> runs;
  std::vector<TermDevB> terms;
  std::vector<double> rnds;
  const size_t amp = b->dbl ? 16 : 8;
  uint64_t off = 0;
  size_t goff = 0, soff = 0;
  b->grad_off.assign(ninst, 0);
  b->smp_off.assign(ninst, 0);
  for (size_t k = 0; k < ninst; ++k) {
    const size_t i = order[k];
    BatchInstHost &h = b->inst[i];
    InstDev &d = idev[k];
    d.n = h.n;
    d.team = team[k];
    d.nops = (int)h.gates.size();
    d.nruns = (int)h.runs.size();
    d.nterms = (int)h.terms.size();
    d.nparams = h.nparams;
    d.op_off = (int)gates.size();
    d.run_off = (int)runs.size();
    d.term_off = (int)terms.size();
    d.grad_off = (int)goff;
    b->grad_off[i] = goff;
    goff += h.nparams;
    gates.insert(gates.end(), h.gates.begin(), h.gates.end());
    runs.insert(runs.end(), h.runs.begin(), h.runs.end());
    terms.insert(terms.end(), h.terms.begin(), h.terms.end());
    const uint64_t N = 1ULL << h.n;
    // lambda doubles as the sampling CDF: it needs >= N / 2^10 doubles
    d.psi_off = off;
    off += N;
    d.lam_off = off;
    off += std::max<uint64_t>(N, 64);
    d.shots = h.shots;
    d.rnd_off = rnds.size();
    d.smp_off = soff;
    b->smp_off[i] = soff;
    soff += h.shots;
    std::mt19937_64 rng(h.seed);
    std::uniform_real_distribution<double> dist(0.0, 1.0);
    for (uint64_t s = 0; s < h.shots; ++s) rnds.push_back(dist(rng));
  }
  b->arena_bytes = off * amp;
  cuda_check(cudaMalloc(&b->arena, b->arena_bytes), "batch state arena");
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t s_inst = al(sizeof(InstDev) * ninst), s_gates = al(sizeof(GateDev) * std::max<size_t>(gates.size(), 1)),
               s_runs = al(sizeof(RunDev) * std::max<size_t>(runs.size(), 1)),
               s_terms = al(sizeof(TermDevB) * terms.size()), s_rnds = al(sizeof(double) * std::max<size_t>(rnds.size(), 1)),
               s_smp = al(sizeof(uint64_t) * std::max<size_t>(soff, 1)), s_e = al(sizeof(double) * ninst),
               s_g = al(sizeof(double) * std::max<size_t>(goff, 1)), s_t = al(sizeof(unsigned long long) * ninst),
               s_q = 256;
  b->blob_bytes = s_inst + s_gates + s_runs + s_terms + s_rnds + s_smp + s_e + s_g + 2 * s_t + s_q;
  cuda_check(cudaMalloc(&b->dev_blob, b->blob_bytes), "batch buffers");
  char *p = static_cast<char *>(b->dev_blob);
  auto up = [&](const void *src, size_t bytes, size_t slot) {
    if (bytes) cuda_check(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice), "batch upload");
    char *r = p;
    p += slot;
    return r;
  };
  up(idev.data(), sizeof(InstDev) * ninst, s_inst);
  up(gates.data(), sizeof(GateDev) * gates.size(), s_gates);
  up(runs.data(), sizeof(RunDev) * runs.size(), s_runs);
  up(terms.data(), sizeof(TermDevB) * terms.size(), s_terms);
  up(rnds.data(), sizeof(double) * rnds.size(), s_rnds);
  b->samples.assign(soff, 0);
  b->energy.assign(ninst, 0.0);
  b->grads.assign(goff, 0.0);
  b->t0.assign(ninst, 0);
  b->t1.assign(ninst, 0);
  b->order = order;
  // team buffers: items, one barrier counter per instance, the error word
  const size_t s_items = (sizeof(int2) * items.size() + 255) & ~size_t(255);
  cuda_check(cudaMalloc(&b->team_blob, s_items + sizeof(unsigned) * ninst + 256), "batch team buffers");
  cuda_check(cudaMemcpy(b->team_blob, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice),
             "batch upload");
  b->built = true;
}

struct BatchLayout {
  InstDev *inst;
  GateDev *gates;
  RunDev *runs;
  TermDevB *terms;
  double *rnds;
  uint64_t *samples;
  double *energy, *grads;
  unsigned long long *t0, *t1;
  int *queue;
  size_t ngrad;
};

BatchLayout layout(gbqv_batch *b, size_t ngates, size_t nruns, size_t nterms, size_t nrnds, size_t nsmp, size_t ngrad) {
  const size_t ninst = b->inst.size();
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  char *p = static_cast<char *>(b->dev_blob);
  BatchLayout L;
  L.inst = reinterpret_cast<InstDev *>(p); p += al(sizeof(InstDev) * ninst);
  L.gates = reinterpret_cast<GateDev *>(p); p += al(sizeof(GateDev) * std::max<size_t>(ngates, 1));
  L.runs = reinterpret_cast<RunDev *>(p); p += al(sizeof(RunDev) * std::max<size_t>(nruns, 1));
  L.terms = reinterpret_cast<TermDevB *>(p); p += al(sizeof(TermDevB) * nterms);
  L.rnds = reinterpret_cast<double *>(p); p += al(sizeof(double) * std::max<size_t>(nrnds, 1));
  L.samples = reinterpret_cast<uint64_t *>(p); p += al(sizeof(uint64_t) * std::max<size_t>(nsmp, 1));
  L.energy = reinterpret_cast<double *>(p); p += al(sizeof(double) * ninst);
  L.grads = reinterpret_cast<double *>(p); p += al(sizeof(double) * std::max<size_t>(ngrad, 1));
  L.t0 = reinterpret_cast<unsigned long long *>(p); p += al(sizeof(unsigned long long) * ninst);
  L.t1 = reinterpret_cast<unsigned long long *>(p); p += al(sizeof(unsigned long long) * ninst);
  L.queue = reinterpret_cast<int *>(p);
  L.ngrad = ngrad;
  return L;
}

template <typename T, int M>
void launch_batch(gbqv_batch *b, const BatchLayout &L, int want_grad) {
  const size_t smem = sizeof(T) * 2 * (1u << M) + sizeof(uint64_t) * (64 + (1u << (M - 6)));
  static bool attr = false;
  if (!attr) {
    cuda_check(cudaFuncSetAttribute(k_batch<T, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
    attr = true;
  }
  int per_sm = 1;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<T, M>, kBatchThreads, smem), "occupancy");
  // every CTA resident at once (a team member waits for its partner, the next queue item)
  const int grid = (int)std::min<size_t>((size_t)b->nitems, (size_t)sm_count() * std::max(per_sm, 1));
  const size_t ninst = b->inst.size();
  char *tb = static_cast<char *>(b->team_blob);
  const size_t s_items = (sizeof(int2) * b->nitems + 255) & ~size_t(255);
  unsigned *bar = reinterpret_cast<unsigned *>(tb + s_items);
  int *err = reinterpret_cast<int *>(tb + s_items + sizeof(unsigned) * ninst);
  cuda_check(cudaMemsetAsync(L.queue, 0, sizeof(int), b->stream), "queue reset");
  cuda_check(cudaMemsetAsync(bar, 0, sizeof(unsigned) * ninst + sizeof(int), b->stream), "team reset");
  cuda_check(cudaMemsetAsync(L.energy, 0, sizeof(double) * ninst, b->stream), "energy reset");
  if (L.ngrad) cuda_check(cudaMemsetAsync(L.grads, 0, sizeof(double) * L.ngrad, b->stream), "gradient reset");
  k_batch<T, M><<<grid, kBatchThreads, smem, b->stream>>>(L.inst, (int)ninst, L.gates, L.runs, L.terms,
                                                          static_cast<T *>(b->arena), L.rnds, L.samples, L.energy,
                                                          L.grads, L.t0, L.t1, L.queue, want_grad,
                                                          reinterpret_cast<const int2 *>(tb), b->nitems, bar, err);
  cuda_check(cudaGetLastError(), "batch kernel");
}

int team_error(gbqv_batch *b) {
  const size_t s_items = (sizeof(int2) * b->nitems + 255) & ~size_t(255);
  int e = 0;
  cuda_check(cudaMemcpy(&e, static_cast<char *>(b->team_blob) + s_items + sizeof(unsigned) * b->inst.size(),
                        sizeof(int), cudaMemcpyDeviceToHost),
             "team status");
  return e;
}

}  // namespace

extern "C" int gbqv_batch_run(gbqv_batch_t b, int want_grad, double *elapsed_ms) {
  return bguard([&] {
    if (!b) throw Error(GBQV_ERR_ARG, "null batch");
    if (!b->built) batch_build(b);
    size_t ng = 0, nr = 0, nt = 0, nrnd = 0, ngrad = 0;
    for (auto &h : b->inst) {
      ng += h.gates.size();
      nr += h.runs.size();
      nt += h.terms.size();
      nrnd += h.shots;
      ngrad += h.nparams;
    }
    BatchLayout L = layout(b, ng, nr, nt, nrnd, nrnd, ngrad);
    // one persistent launch (plus the queue reset), captured once as a CUDA graph
    if (!b->graph) {
      cuda_check(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
      if (b->dbl && b->fp64)
        launch_batch<double2, 11>(b, L, want_grad);
      else if (b->dbl)
        launch_batch<fcx, 11>(b, L, want_grad);
      else
        launch_batch<float2, 12>(b, L, want_grad);
      cuda_check(cudaStreamEndCapture(b->stream, &b->graph_def), "graph capture");
      cuda_check(cudaGraphInstantiate(&b->graph, b->graph_def, 0), "graph instantiate");
    }
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    cuda_check(cudaEventRecord(e0, b->stream), "event");
    cuda_check(cudaGraphLaunch(b->graph, b->stream), "graph launch");
    cuda_check(cudaEventRecord(e1, b->stream), "event");
    cuda_check(cudaEventSynchronize(e1), "batch run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (elapsed_ms) *elapsed_ms = ms;
    if (team_error(b)) throw Error(GBQV_ERR_TIMEOUT, "a team barrier of the batched kernel gave up after 2 s");
    // results back, in instance order
    const size_t ninst = b->inst.size();
    std::vector<double> energy(ninst);
    std::vector<unsigned long long> t0(ninst), t1(ninst);
    std::vector<double> grads(ngrad);
    std::vector<uint64_t> samples(nrnd);
    cuda_check(cudaMemcpy(energy.data(), L.energy, sizeof(double) * ninst, cudaMemcpyDeviceToHost), "copy");
    cuda_check(cudaMemcpy(t0.data(), L.t0, sizeof(unsigned long long) * ninst, cudaMemcpyDeviceToHost), "copy");
    cuda_check(cudaMemcpy(t1.data(), L.t1, sizeof(unsigned long long) * ninst, cudaMemcpyDeviceToHost), "copy");
    if (ngrad) cuda_check(cudaMemcpy(grads.data(), L.grads, sizeof(double) * ngrad, cudaMemcpyDeviceToHost), "copy");
    if (nrnd) cuda_check(cudaMemcpy(samples.data(), L.samples, sizeof(uint64_t) * nrnd, cudaMemcpyDeviceToHost), "copy");
    // device position k held instance order[k]; grads / samples were laid out per instance already
    b->energy.assign(ninst, 0.0);
    b->t0.assign(ninst, 0);
    b->t1.assign(ninst, 0);
    for (size_t k = 0; k < ninst; ++k) {
      const size_t i = b->order[k];
      b->energy[i] = energy[k];
      b->t0[i] = t0[k];
      b->t1[i] = t1[k];
    }
    b->grads = grads;
    b->samples = samples;
  });
}

extern "C" int gbqv_batch_result(gbqv_batch_t b, int i, double *energy, double *grad, int nparams, uint64_t *samples,
                                 uint64_t shots, double *latency_ms) {
  return bguard([&] {
    if (!b || i < 0 || i >= (int)b->inst.size()) throw Error(GBQV_ERR_ARG, "instance index out of range");
    const BatchInstHost &h = b->inst[i];
    if (energy) *energy = b->energy[i];
    if (grad) {
      if (nparams != h.nparams) throw Error(GBQV_ERR_ARG, "parameter count mismatch");
      std::copy(b->grads.begin() + b->grad_off[i], b->grads.begin() + b->grad_off[i] + nparams, grad);
    }
    if (samples) {
      if (shots != h.shots) throw Error(GBQV_ERR_ARG, "shot count mismatch");
      std::copy(b->samples.begin() + b->smp_off[i], b->samples.begin() + b->smp_off[i] + shots, samples);
    }
    if (latency_ms) *latency_ms = (double)(b->t1[i] - b->t0[i]) * 1e-6;
  });
}
