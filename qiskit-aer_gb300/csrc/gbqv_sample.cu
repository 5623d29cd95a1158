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
// The sequential sums are 2^isz dependent chains (1024 by default), far too
// few threads to cover HBM latency with ordinary loads.  So the
// probabilities are first written out in one parallel pass (8 bytes per
// outcome), and each CTA then streams the probabilities of 8 chains through
// a 3-stage shared-memory ring filled by bulk copies (cp.async.bulk, 8 KB
// per chain per stage), the 8 chain threads adding from shared memory.
// Every wait is bounded; a stalled ring raises the device status word that
// the host reports as GBQV_ERR_TIMEOUT.  When the probability buffer cannot
// be allocated, or the blocks are short, the chains read the state itself.
#include <algorithm>
#include <cstdint>

#include "gbqv_internal.h"
#include "gbqv_tc.cuh"

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

// Every outcome's probability, in the reference's rounding.
template <typename T>
__global__ void __launch_bounds__(256) k_probs_exact(const T *__restrict__ psi, uint64_t count, uint64_t diag_stride,
                                                     double *__restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = prob_exact<T>(psi, i, diag_stride);
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

// The staged form over the probability buffer: CTA = kChains chain threads
// (warp 0) + one loader thread (warp 1); blocks of L >= kChunk doubles.
constexpr int kChains = 8;
constexpr int kChunk = 1024;                     // doubles per chain per stage, one checkpoint each
constexpr int kStages = 3;
constexpr int kRowBytes = kChunk * 8 + 16;       // row pitch: chain b's row starts 4 banks after b - 1's
constexpr int kStageBytes = kChains * kRowBytes;
constexpr int kSeqSmem = kStages * kStageBytes + 2 * kStages * 8 + 16;

template <bool WALK>
__global__ void __launch_bounds__(64) k_seq_chains(const double *__restrict__ probs, uint64_t nblocks, uint64_t L,
                                                   const double *__restrict__ P, double *__restrict__ out,
                                                   int *status) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kStages * kStageBytes);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kStages * kStageBytes + 2 * kStages * 8);
  const uint32_t bar0 = tc::smem_u32(bars);
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (kStages + s); };
  const uint64_t chain0 = (uint64_t)blockIdx.x * kChains;
  const int active = (int)std::min<uint64_t>(kChains, nblocks - chain0);
  const uint64_t nchunks = L / kChunk;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(full(s), 1);
      tc::mbar_init(empty(s), (uint32_t)active);
    }
    *abort_flag = 0;
    tc::mbar_init_fence();
  }
  __syncthreads();
  if (tid < active) {
    const uint64_t j = chain0 + tid;
    double acc = WALK ? P[j] : 0.0;
    bool ok = true;
    for (uint64_t c = 0; c < nchunks; ++c) {
      const int s = (int)(c % kStages);
      if (!tc::mbar_wait(full(s), (uint32_t)((c / kStages) & 1), abort_flag)) {
        ok = false;
        break;
      }
      const double *row = reinterpret_cast<const double *>(smem + s * kStageBytes + tid * kRowBytes);
      for (int t = 0; t < kChunk; t += 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = row[t + u];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc = __dadd_rn(acc, v[u]);
      }
      if (WALK) out[j * nchunks + c] = acc;
      // these generic-proxy reads come before the loader's next bulk
      // (async-proxy) write into the stage
      tc::fence_async_smem();
      tc::mbar_arrive(empty(s));
    }
    if (ok && !WALK) out[j] = acc;
  } else if (tid == 32) {
    // loader: chunk c of every active chain into stage c % kStages
    uint64_t issued = 0;
    for (uint64_t c = 0; c < nchunks; ++c) {
      const int s = (int)(c % kStages);
      if (c >= kStages && !tc::mbar_wait(empty(s), (uint32_t)((c / kStages - 1) & 1), abort_flag, 64)) break;
      tc::mbar_arrive_expect_tx(full(s), (uint32_t)(active * kChunk * 8));
      for (int b = 0; b < active; ++b)
        tc::bulk_g2s(tc::smem_u32(smem + s * kStageBytes + b * kRowBytes), probs + (chain0 + b) * L + c * kChunk,
                     kChunk * 8, full(s));
      issued = c + 1;
    }
    // copies in flight after an abort land before the CTA exits
    int never = 0;
    for (uint64_t c = issued > kStages ? issued - kStages : 0; c < issued; ++c)
      tc::mbar_wait(full((int)(c % kStages)), (uint32_t)((c / kStages) & 1), &never);
  }
  __syncthreads();
  if (tid == 0 && *abort_flag) atomicExch(status, 1);
}

// P[0] = 0, P[j + 1] = fl(P[j] + idxs[j]): the reference's running sum.
__global__ void k_seq_prefix(const double *__restrict__ idxs, uint64_t nblocks, double *__restrict__ P) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double p = 0.0;
  P[0] = 0.0;
  for (uint64_t j = 0; j < nblocks; ++j) {
    p = __dadd_rn(p, idxs[j]);
    P[j + 1] = p;
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
  const uint64_t ck = kChunk;
  // blocks of up to 1024 amplitudes are walked from P[j] by each shot;
  // longer blocks keep every 1024th partial sum of the walk
  const bool use_cps = L > ck;
  const uint64_t ncps = use_cps ? END / ck : 0;
  // idxs[nblocks], P[nblocks + 1], checkpoints[END / ck]
  grow(dev.aux, dev.aux_cap, sizeof(double) * (2 * nblocks + 1 + ncps + 1));
  double *idxs = reinterpret_cast<double *>(dev.aux);
  double *P = idxs + nblocks;
  double *cps = use_cps ? P + nblocks + 1 : nullptr;
  // the probability buffer, for the staged chains (long blocks) and the walks
  double *probs = nullptr;
  if (use_cps) {
    try {
      probs = static_cast<double *>(grow(dev.probs, dev.probs_cap, sizeof(double) * END));
    } catch (const Error &) {
      cudaGetLastError();  // no room for 8 bytes per outcome: the chains read the state
      probs = nullptr;
    }
  }
  if (probs) {
    k_probs_exact<T><<<(unsigned)std::min<uint64_t>((END + 255) / 256, (uint64_t)sm_count() * 16), 256, 0,
                       dev.stream>>>(psi, END, ds, probs);
    check_launch("sampling probabilities");
  }
  if (nblocks) {
    if (probs) {
      static bool attr = false;
      if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_seq_chains<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSeqSmem),
                   "sampling chain attribute");
        cuda_check(cudaFuncSetAttribute(k_seq_chains<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSeqSmem),
                   "sampling chain attribute");
        attr = true;
      }
      int *status = tc_status_word(dev);
      const unsigned g = (unsigned)((nblocks + kChains - 1) / kChains);
      k_seq_chains<false><<<g, 64, kSeqSmem, dev.stream>>>(probs, nblocks, L, nullptr, idxs, status);
      check_launch("sampling block sums");
      k_seq_prefix<<<1, 32, 0, dev.stream>>>(idxs, nblocks, P);
      check_launch("sampling block prefix");
      k_seq_chains<true><<<g, 64, kSeqSmem, dev.stream>>>(probs, nblocks, L, P, cps, status);
      check_launch("sampling block walk");
    } else {
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
  }
  const unsigned g2 = (unsigned)std::min<uint64_t>((shots + 255) / 256, (uint64_t)sm_count() * 16);
  k_sample_exact<T><<<std::max(g2, 1u), 256, 0, dev.stream>>>(psi, probs, END, nblocks, L, ds, P, cps, ck, d_rnds,
                                                              shots, d_out);
  check_launch("sampling search");
  // a large probability buffer is not kept between calls (cudaFree waits
  // for the kernels above)
  if (dev.probs && dev.probs_cap > (1ULL << 30)) {
    cuda_check(cudaFree(dev.probs), "sampling buffer release");
    dev.probs = nullptr;
    dev.probs_cap = 0;
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
