// gbqv_noalloc.cu — gbqv_expval_pauli_many_noalloc: Pauli expectation values
// of a caller-owned device state that allocate no memory at all.
//
// Who needs it: callers that cannot call cudaMalloc — a framework whose
// caching allocator already owns the device's memory (the statevector was
// placed in its pool and a cudaMalloc next to it would fail or fragment it),
// or a latency-critical loop that must not pay the device synchronisation
// cudaMalloc / cudaFree imply.  Every other reduction in this library keeps
// its partial sums in per-handle scratch that grows with cudaMalloc; this
// entry point keeps them in one file-scope __device__ array instead.
//
// Limits and sharing: at most kNoAllocMaxTerms terms per call.  The array is
// allocated when the library is loaded on a device and stays allocated until
// the process exits.  Every call on a device uses the same array, so calls
// whose kernels overlap on the GPU (different streams, different threads)
// race on it; serialise them.  The array keeps the last call's partial sums;
// each call writes every slot it later reads, so nothing needs clearing.
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current); make that first call
// before any stream capture.
#include <cstring>
#include <mutex>

#include "../../include/gbqv.h"
#include "gbqv_gates.h"
#include "gbqv_internal.h"

namespace gbqv {
namespace {

constexpr int kNoAllocMaxTerms = 64;
constexpr int kNoAllocBlocks = 152;  // one CTA per SM of a GB300
constexpr int kNoAllocThreads = 256;
constexpr size_t kNoAllocDoubles = (size_t)kNoAllocBlocks * kNoAllocMaxTerms + kNoAllocMaxTerms;

// partial sums [term][block], then the per-term results
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

struct NoAllocTerm {
  uint64_t x_mask, z_mask, x_max;
  double ph_re;
  double ph_im;
};

struct NoAllocTerms {
  NoAllocTerm t[kNoAllocMaxTerms];
};

__device__ __forceinline__ double na_block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;
}

// The expval reduction of QubitVector::expval_pauli (qubitvector.hpp:2299-2347),
// terms by value (kernel parameters), one row of CTAs per term.
template <typename T>
__global__ void __launch_bounds__(kNoAllocThreads) k_expval_static(const T *__restrict__ psi, int n,
                                                                   const __grid_constant__ NoAllocTerms terms,
                                                                   double *__restrict__ scratch) {
  const NoAllocTerm t = terms.t[blockIdx.y];
  using R = decltype(T::x);
  const R pr = (R)t.ph_re, pi = (R)t.ph_im;
  double acc = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (!t.x_mask) {
    const uint64_t count = 1ULL << n;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
      const T a = psi[i];
      R v = pr * (a.x * a.x + a.y * a.y);
      if (t.z_mask && (__popcll(i & t.z_mask) & 1)) v = -v;
      acc += (double)v;
    }
  } else {
    const uint64_t count = 1ULL << (n - 1);
    const uint64_t mask_l = (1ULL << t.x_max) - 1;
    const uint64_t mask_u = ~((1ULL << (t.x_max + 1)) - 1);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
      const uint64_t i0 = ((i << 1) & mask_u) | (i & mask_l);
      const uint64_t i1 = i0 ^ t.x_mask;
      const T a0 = psi[i0], a1 = psi[i1];
      const R zr = a1.x * a0.x + a1.y * a0.y;
      const R zi = a1.y * a0.x - a1.x * a0.y;
      R v0 = pr * zr - pi * zi;
      R v1 = pr * zr + pi * zi;
      if (t.z_mask && (__popcll(i0 & t.z_mask) & 1)) v0 = -v0;
      if (t.z_mask && (__popcll(i1 & t.z_mask) & 1)) v1 = -v1;
      acc += (double)v0;
      acc += (double)v1;
    }
  }
  acc = na_block_sum(acc);
  if (threadIdx.x == 0) scratch[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

// Per-term sum of the CTA partials in a fixed order, into the results slots.
__global__ void k_finish_static(double *__restrict__ scratch, int nblocks, int nterms) {
  for (int v = blockIdx.x; v < nterms; v += gridDim.x) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += scratch[(size_t)v * nblocks + b];
    s = na_block_sum(s);
    if (threadIdx.x == 0) scratch[(size_t)kNoAllocBlocks * kNoAllocMaxTerms + v] = s;
  }
}

std::mutex g_noalloc_mu;
double *g_noalloc_ptr[64] = {nullptr};

// Device address of the static array on the current device (resolved once
// per device, with that device current).  The address is cached for the
// life of the process: after cudaDeviceReset (or any reset of the device's
// primary context) the module is loaded again and the array may move, so a
// process that resets a device must not call the allocation-free entry point
// on that device afterwards.
double *noalloc_scratch() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= 64) throw Error(GBQV_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress of the static scratch");
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  return g_noalloc_ptr[dev];
}

}  // namespace
}  // namespace gbqv

using namespace gbqv;

extern "C" int gbqv_expval_pauli_many_noalloc(const void *state, int num_qubits, int precision, int nterms,
                                              const uint64_t *qubits, const int *offsets,
                                              const char *const *labels, const double *coeffs, void *stream,
                                              double *out, double *total) {
  try {
    if (!state) throw Error(GBQV_ERR_ARG, "null device state");
    if (precision != GBQV_C64 && precision != GBQV_C128) throw Error(GBQV_ERR_ARG, "bad precision");
    if (num_qubits < 1 || num_qubits > kMaxQubits) throw Error(GBQV_ERR_ARG, "number of qubits out of range");
    if (nterms < 1 || nterms > kNoAllocMaxTerms)
      throw Error(GBQV_ERR_ARG, "expval_pauli_many_noalloc takes 1.." + std::to_string(kNoAllocMaxTerms) +
                                    " terms per call (static scratch of " +
                                    std::to_string(kNoAllocDoubles * sizeof(double)) + " bytes); got " +
                                    std::to_string(nterms));
    if (!offsets || !labels) throw Error(GBQV_ERR_ARG, "null term arrays");
    if (offsets[0] != 0) throw Error(GBQV_ERR_ARG, "bad term offsets: offsets[0] must be 0");
    NoAllocTerms terms{};
    for (int t = 0; t < nterms; ++t) {
      const int k = offsets[t + 1] - offsets[t];
      if (k < 0 || k > num_qubits || (k > 0 && !qubits)) throw Error(GBQV_ERR_ARG, "bad term offsets");
      const uint64_t *q = qubits + offsets[t];
      if (!labels[t] || (int)std::strlen(labels[t]) != k)
        throw Error(GBQV_ERR_ARG, "Pauli label length must equal qubit count");
      // pauli_masks_and_phase (qubitvector.hpp:2235-2272) on fixed storage
      uint64_t x_mask = 0, z_mask = 0, num_y = 0, x_max = 0, seen = 0;
      for (int i = 0; i < k; ++i) {
        if (q[i] >= (uint64_t)num_qubits) throw Error(GBQV_ERR_QUBIT, "qubit index out of range");
        const uint64_t bit = 1ULL << q[i];
        if (seen & bit) throw Error(GBQV_ERR_QUBIT, "repeated qubit");
        seen |= bit;
        switch (labels[t][k - 1 - i]) {
          case 'I': break;
          case 'X': x_mask |= bit; x_max = q[i] > x_max ? q[i] : x_max; break;
          case 'Z': z_mask |= bit; break;
          case 'Y': x_mask |= bit; z_mask |= bit; x_max = q[i] > x_max ? q[i] : x_max; ++num_y; break;
          default: throw Error(GBQV_ERR_ARG, "invalid Pauli letter");
        }
      }
      const cd ph = add_y_phase(num_y, cd(1.0, 0.0));
      terms.t[t] = NoAllocTerm{x_mask, z_mask, x_max, ph.real(), ph.imag()};
    }
    double *scratch = noalloc_scratch();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 grid(kNoAllocBlocks, (unsigned)nterms);
    if (precision == GBQV_C128)
      k_expval_static<double2><<<grid, kNoAllocThreads, 0, s>>>(static_cast<const double2 *>(state), num_qubits, terms,
                                                                scratch);
    else
      k_expval_static<float2><<<grid, kNoAllocThreads, 0, s>>>(static_cast<const float2 *>(state), num_qubits, terms,
                                                               scratch);
    cuda_check(cudaGetLastError(), "expval kernel (static scratch)");
    k_finish_static<<<std::min(nterms, 64), 256, 0, s>>>(scratch, kNoAllocBlocks, nterms);
    cuda_check(cudaGetLastError(), "reduction finish (static scratch)");
    double vals[kNoAllocMaxTerms];
    cuda_check(cudaMemcpyAsync(vals, scratch + (size_t)kNoAllocBlocks * kNoAllocMaxTerms, sizeof(double) * nterms,
                               cudaMemcpyDeviceToHost, s),
               "result copy");
    cuda_check(cudaStreamSynchronize(s), "stream synchronize");
    double sum = 0.0;
    for (int t = 0; t < nterms; ++t) {
      if (out) out[t] = vals[t];
      sum += (coeffs ? coeffs[t] : 1.0) * vals[t];
    }
    if (total) *total = sum;
    return GBQV_OK;
  } catch (const Error &e) {
    set_last_error(nullptr, e.what());
    return e.code;
  } catch (const std::exception &e) {
    set_last_error(nullptr, e.what());
    return GBQV_ERR_ARG;
  }
}
