// gbqv_kernels.cu — sm_103a kernels of the GB300 statevector / density-matrix
// engine and their launchers.
//
// Layout in HBM: one contiguous array of 2^n interleaved complex amplitudes
// (complex<double>: 16 B, complex<float>: 8 B), amplitude index bit q = qubit
// q, 256-byte aligned (cudaMalloc).  A density matrix is vec(rho) over 2n
// vector qubits, column-stacked (rho[i,j] at i + 2^n j), as the reference
// stores it (src/simulators/density_matrix/densitymatrix.hpp:265-323).
//
// Every kernel is a grid-stride loop sized to a multiple of the 152 SMs.
// A thread owns one "group": the 2^k amplitudes that a k-qubit op mixes,
// found by inserting zero bits at the sorted target positions of the group
// number (src/simulators/statevector/indexes.hpp:212-258).  Consecutive
// threads own consecutive groups, so every load of a group member is
// coalesced across the warp whenever the targets sit above the 16-byte
// word; low targets are served from L1 (the partner amplitude is in the
// same 128-byte line).
//
// Reductions accumulate in FP64 in every precision, reduce each CTA with
// warp shuffles, and combine the CTA partials in a fixed order in a second
// launch, so results are deterministic run to run.
#include "gbqv_internal.h"
#include "gbqv_ozaki.h"

#include <algorithm>
#include <type_traits>
#include <cstring>
#include <memory>
#include <atomic>

namespace gbqv {

namespace {

#include "gbqv_fpair.cuh"

template <typename R> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
  T r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// acc += a * b (four FMAs)
template <typename T>
__device__ __forceinline__ void cfma(T &acc, T a, T b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

template <typename T>
__device__ __forceinline__ bool is_one(T a) { return a.x == 1 && a.y == 0; }

__device__ __forceinline__ uint64_t insert_zeros(uint64_t i, const uint64_t *lowmask, int k) {
  for (int j = 0; j < k; ++j) {
    const uint64_t m = lowmask[j];
    i = ((i & ~m) << 1) | (i & m);
  }
  return i;
}

template <int K>
__device__ __forceinline__ uint64_t insert_zeros_k(uint64_t i, const uint64_t *lowmask) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const uint64_t m = lowmask[j];
    i = ((i & ~m) << 1) | (i & m);
  }
  return i;
}

inline int grid_for(uint64_t work, int threads, int per_sm = 8) {
  uint64_t blocks = (work + threads - 1) / threads;
  uint64_t cap = 152ULL * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

}  // namespace

void sorted_masks(const reg_t &qubits, uint64_t *lowmask) {
  reg_t s = qubits;
  std::sort(s.begin(), s.end());
  for (size_t j = 0; j < s.size(); ++j) lowmask[j] = (1ULL << s[j]) - 1;
}

void local_offsets(const reg_t &qubits, uint64_t *offs) {
  const int k = (int)qubits.size();
  offs[0] = 0;
  for (int j = 0; j < k; ++j) {
    const uint64_t n = 1ULL << j, bit = 1ULL << qubits[j];
    for (uint64_t m = 0; m < n; ++m) offs[n + m] = offs[m] | bit;
  }
}

namespace {

template <typename T> T to_dev(const cd &z);
template <> double2 to_dev<double2>(const cd &z) { return make_double2(z.real(), z.imag()); }
template <> float2 to_dev<float2>(const cd &z) { return make_float2((float)z.real(), (float)z.imag()); }

std::atomic<uint64_t> g_launches{0};

}  // namespace

void check_launch(const char *what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cuda_check(cudaGetLastError(), what);
}

namespace {

// -------------------------------------------------------------------------
// Dense k-qubit matrix, k <= 5: the matrix rides in the kernel parameters
// (constant bank, broadcast to the warp), the group in registers.
// Transformer::apply_matrix_n (transformer.hpp:151-171).
// -------------------------------------------------------------------------
template <typename T, int K>
struct DenseParams {
  T mat[1 << (2 * K)];
  uint64_t offs[1 << K];
  uint64_t lowmask[K];
  uint64_t ngroups;
};

// (Capping complex64 k <= 4 at 3 CTAs per SM spills and measured slower
// than 2 CTAs per SM; an explicit minimum of 1 CTA per SM lets the compiler
// take 130 registers for complex64 k = 4, which allows only one CTA per SM
// and cost 35% at 30 qubits.  The plain bound gives 118 registers, 2 CTAs.)
template <typename T, int K, bool NORM>
__global__ void __launch_bounds__(256) k_dense(T *__restrict__ psi, const __grid_constant__ DenseParams<T, K> p,
                                               double *__restrict__ partials) {
  constexpr int D = 1 << K;
  double nacc = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.ngroups; g += stride) {
    const uint64_t base = insert_zeros_k<K>(g, p.lowmask);
    T v[D];
#pragma unroll
    for (int a = 0; a < D; ++a) v[a] = psi[base + p.offs[a]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      T acc;
      acc.x = 0;
      acc.y = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) cfma(acc, p.mat[r + D * c], v[c]);
      if (NORM)
        nacc += (double)(acc.x * acc.x + acc.y * acc.y);
      else
        psi[base + p.offs[r]] = acc;
    }
  }
  if (NORM) {
    for (int o = 16; o > 0; o >>= 1) nacc += __shfl_xor_sync(0xffffffffu, nacc, o);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nacc;
    __syncthreads();
    if (threadIdx.x < 32) {
      double s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
  }
}

// Dense k-qubit matrix, 6 <= k <= 13: one CTA per group, the group staged in
// shared memory, the matrix read from device memory (L2 resident up to
// k = 11 at complex128); thread r computes output rows r, r + blockDim.x, ...
// MatrixMultNxN (chunk/thrust_kernels.hpp:900-933).  NORM: ||M psi||^2
// (QubitVector::norm(qubits, mat), qubitvector.hpp:1878-2082) into one FP64
// partial per CTA, the state left as it is.
template <typename T, bool NORM>
__global__ void k_dense_big(T *__restrict__ psi, const T *__restrict__ mat, int k, uint64_t ngroups,
                            const uint64_t *__restrict__ meta, double *__restrict__ partials) {
  extern __shared__ unsigned char smem_raw[];
  T *cache = reinterpret_cast<T *>(smem_raw);
  const int D = 1 << k;
  const uint64_t *offs = meta;
  const uint64_t *lowmask = meta + D;
  double nacc = 0.0;
  for (uint64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const uint64_t base = insert_zeros(g, lowmask, k);
    for (int a = threadIdx.x; a < D; a += blockDim.x) cache[a] = psi[base + offs[a]];
    __syncthreads();
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
      T acc;
      acc.x = 0;
      acc.y = 0;
      for (int c = 0; c < D; ++c) cfma(acc, mat[r + (uint64_t)D * c], cache[c]);
      if (NORM)
        nacc += (double)acc.x * (double)acc.x + (double)acc.y * (double)acc.y;
      else
        psi[base + offs[r]] = acc;
    }
    __syncthreads();
  }
  if (NORM) {
    for (int o = 16; o > 0; o >>= 1) nacc += __shfl_xor_sync(0xffffffffu, nacc, o);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nacc;
    __syncthreads();
    if (threadIdx.x < 32) {
      double s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
  }
}

template <typename T, int K>
void dense_small(Device &dev, const reg_t &qubits, const cd *mat, bool norm) {
  DenseParams<T, K> p;
  constexpr int D = 1 << K;
  for (int i = 0; i < D * D; ++i) p.mat[i] = to_dev<T>(mat[i]);
  local_offsets(qubits, p.offs);
  sorted_masks(qubits, p.lowmask);
  p.ngroups = dev.amps() >> K;
  const int threads = 256;
  if (norm) {
    const int grid = kReduceBlocks;
    k_dense<T, K, true><<<grid, threads, 0, dev.stream>>>(reinterpret_cast<T *>(dev.state), p, dev.partials);
  } else {
    const int grid = grid_for(p.ngroups, threads);
    k_dense<T, K, false><<<grid, threads, 0, dev.stream>>>(reinterpret_cast<T *>(dev.state), p, nullptr);
  }
  check_launch("dense matrix kernel");
}

template <typename T>
void dense_any(Device &dev, const reg_t &qubits, const cd *mat, bool norm) {
  const int k = (int)qubits.size();
  switch (k) {
    case 1: return dense_small<T, 1>(dev, qubits, mat, norm);
    case 2: return dense_small<T, 2>(dev, qubits, mat, norm);
    case 3: return dense_small<T, 3>(dev, qubits, mat, norm);
    case 4: return dense_small<T, 4>(dev, qubits, mat, norm);
    case 5: return dense_small<T, 5>(dev, qubits, mat, norm);
    default: break;
  }
  const int D = 1 << k;
  const size_t smem = sizeof(T) * (size_t)D;
  if (k > kMaxDenseK || smem > 227 * 1024)
    throw Error(1, "dense matrix supports at most " + std::to_string(kMaxDenseK) + " qubits");
  // matrix + offsets + masks in one device buffer
  const size_t mat_bytes = sizeof(T) * (size_t)D * D;
  const size_t meta_bytes = sizeof(uint64_t) * (D + k);
  grow(dev.mat, dev.mat_cap, mat_bytes + meta_bytes);
  std::vector<T> hm((size_t)D * D);
  for (size_t i = 0; i < hm.size(); ++i) hm[i] = to_dev<T>(mat[i]);
  std::vector<uint64_t> meta(D + k);
  local_offsets(qubits, meta.data());
  sorted_masks(qubits, meta.data() + D);
  cuda_check(cudaMemcpyAsync(dev.mat, hm.data(), mat_bytes, cudaMemcpyHostToDevice, dev.stream), "matrix upload");
  uint64_t *d_meta = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(dev.mat) + mat_bytes);
  cuda_check(cudaMemcpyAsync(d_meta, meta.data(), meta_bytes, cudaMemcpyHostToDevice, dev.stream), "matrix upload");
  // the host copies above are from pageable memory: cudaMemcpyAsync returns
  // only once the source has been consumed, so hm/meta may go out of scope.
  const uint64_t ngroups = dev.amps() >> k;
  const int threads = std::min(D, 1024);
  // norm: one partial per CTA, at most kReduceBlocks of them
  const int grid = (int)std::min<uint64_t>(ngroups, norm ? (uint64_t)kReduceBlocks : 152ULL * 16);
  auto kern = norm ? k_dense_big<T, true> : k_dense_big<T, false>;
  if (smem > 48 * 1024)
    cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "dense matrix kernel attribute");
  kern<<<grid, threads, smem, dev.stream>>>(reinterpret_cast<T *>(dev.state), reinterpret_cast<const T *>(dev.mat), k,
                                            ngroups, d_meta, dev.partials);
  if (norm) {
    // partials past the last CTA are zero for finish()'s fixed block count
    if (grid < kReduceBlocks)
      cuda_check(cudaMemsetAsync(dev.partials + grid, 0, sizeof(double) * (kReduceBlocks - grid), dev.stream),
                 "norm partials");
  }
  check_launch("dense matrix kernel (k > 5)");
}

// -------------------------------------------------------------------------
// Diagonal matrix: Transformer::apply_diagonal_matrix (transformer.hpp:234-258)
// -------------------------------------------------------------------------
template <typename T>
struct DiagParams {
  T diag[1 << kMaxDiagK];
  uint64_t qbit[kMaxDiagK];
  int k;
  uint64_t n_amps;
};

template <typename T>
__global__ void __launch_bounds__(256) k_diag(T *__restrict__ psi, const __grid_constant__ DiagParams<T> p) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_amps; i += stride) {
    uint32_t iv = 0;
    for (int j = 0; j < p.k; ++j) iv |= ((i & p.qbit[j]) != 0) << j;
    const T d = p.diag[iv];
    if (!is_one(d)) psi[i] = cmul(psi[i], d);
  }
}

template <typename T>
void diag_any(Device &dev, const reg_t &qubits, const cd *diag) {
  const int k = (int)qubits.size();
  if (k > kMaxDiagK) throw Error(1, "diagonal matrix supports at most 10 qubits per call");
  DiagParams<T> p;
  for (int i = 0; i < (1 << k); ++i) p.diag[i] = to_dev<T>(diag[i]);
  for (int j = 0; j < k; ++j) p.qbit[j] = 1ULL << qubits[j];
  p.k = k;
  p.n_amps = dev.amps();
  k_diag<T><<<grid_for(p.n_amps, 256), 256, 0, dev.stream>>>(reinterpret_cast<T *>(dev.state), p);
  check_launch("diagonal kernel");
}

// -------------------------------------------------------------------------
// Multi-controlled gates (qubitvector.hpp:1446-1720)
// -------------------------------------------------------------------------
template <typename T>
struct McParams {
  uint64_t lowmask[kMaxQubits];
  int nq;
  int kind;
  uint64_t p0, p1;
  uint64_t ngroups;
  T m[4];
};

template <typename T>
__global__ void __launch_bounds__(256) k_mc(T *__restrict__ psi, const __grid_constant__ McParams<T> p) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.ngroups; g += stride) {
    const uint64_t b = insert_zeros(g, p.lowmask, p.nq);
    const uint64_t i0 = b | p.p0, i1 = b | p.p1;
    switch (p.kind) {
      case 0:
      case 5: {  // X / SWAP: exchange
        const T a = psi[i0];
        psi[i0] = psi[i1];
        psi[i1] = a;
        break;
      }
      case 1: {  // Y: (i0, i1) <- (-i a1, i a0)
        const T a0 = psi[i0], a1 = psi[i1];
        T r0, r1;
        r0.x = a1.y;
        r0.y = -a1.x;
        r1.x = -a0.y;
        r1.y = a0.x;
        psi[i0] = r0;
        psi[i1] = r1;
        break;
      }
      case 2:  // phase on the all-ones entry
        psi[i1] = cmul(psi[i1], p.m[0]);
        break;
      case 3: {  // 2x2 column-major
        const T a0 = psi[i0], a1 = psi[i1];
        T r0 = cmul(p.m[0], a0), r1 = cmul(p.m[1], a0);
        cfma(r0, p.m[2], a1);
        cfma(r1, p.m[3], a1);
        psi[i0] = r0;
        psi[i1] = r1;
        break;
      }
      case 4:  // diagonal 2x2
        psi[i0] = cmul(p.m[0], psi[i0]);
        psi[i1] = cmul(p.m[1], psi[i1]);
        break;
    }
  }
}

template <typename T>
void mc_any(Device &dev, const reg_t &qubits, int kind, const cd *mat) {
  McParams<T> p;
  const int N = (int)qubits.size();
  sorted_masks(qubits, p.lowmask);
  p.nq = N;
  p.kind = kind;
  uint64_t ctrl = 0;
  if (kind == 5) {
    for (int j = 0; j < N - 2; ++j) ctrl |= 1ULL << qubits[j];
    p.p0 = ctrl | (1ULL << qubits[N - 2]);
    p.p1 = ctrl | (1ULL << qubits[N - 1]);
  } else {
    for (int j = 0; j < N - 1; ++j) ctrl |= 1ULL << qubits[j];
    p.p0 = ctrl;
    p.p1 = ctrl | (1ULL << qubits[N - 1]);
  }
  p.ngroups = dev.amps() >> N;
  const int nm = kind == 2 ? 1 : kind == 3 ? 4 : kind == 4 ? 2 : 0;
  for (int i = 0; i < 4; ++i) p.m[i] = to_dev<T>(i < nm ? mat[i] : cd(0, 0));
  k_mc<T><<<grid_for(p.ngroups, 256), 256, 0, dev.stream>>>(reinterpret_cast<T *>(dev.state), p);
  check_launch("multi-controlled gate kernel");
}

// -------------------------------------------------------------------------
// Ordered pair swaps inside each group: apply_permutation_matrix
// (qubitvector.hpp:1349-1434); the density-matrix cnot / swap / toffoli / x
// are such permutations on (q, q+n) (densitymatrix.hpp:331-440).
// -------------------------------------------------------------------------
struct SwapParams {
  uint64_t offs[1 << 10];
  uint64_t lowmask[10];
  uint32_t pairs[2 * kMaxPermPairs];
  int k, npairs;
  uint64_t ngroups;
};

template <typename T>
__global__ void __launch_bounds__(256) k_swaps(T *__restrict__ psi, const SwapParams *__restrict__ p) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p->ngroups; g += stride) {
    const uint64_t b = insert_zeros(g, p->lowmask, p->k);
    for (int j = 0; j < p->npairs; ++j) {
      const uint64_t i0 = b + p->offs[p->pairs[2 * j]], i1 = b + p->offs[p->pairs[2 * j + 1]];
      const T a = psi[i0];
      psi[i0] = psi[i1];
      psi[i1] = a;
    }
  }
}

template <typename T>
void swaps_any(Device &dev, const reg_t &qubits, const std::vector<std::pair<uint32_t, uint32_t>> &pairs) {
  const int k = (int)qubits.size();
  if (k > 10) throw Error(1, "permutation matrix supports at most 10 qubits");
  if (pairs.size() > (size_t)kMaxPermPairs) throw Error(1, "too many permutation pairs");
  auto p = std::make_unique<SwapParams>();
  local_offsets(qubits, p->offs);
  sorted_masks(qubits, p->lowmask);
  for (size_t j = 0; j < pairs.size(); ++j) {
    p->pairs[2 * j] = pairs[j].first;
    p->pairs[2 * j + 1] = pairs[j].second;
  }
  p->k = k;
  p->npairs = (int)pairs.size();
  p->ngroups = dev.amps() >> k;
  grow(dev.mat, dev.mat_cap, sizeof(SwapParams));
  cuda_check(cudaMemcpyAsync(dev.mat, p.get(), sizeof(SwapParams), cudaMemcpyHostToDevice, dev.stream),
             "permutation upload");
  k_swaps<T><<<grid_for(p->ngroups, 256), 256, 0, dev.stream>>>(reinterpret_cast<T *>(dev.state),
                                                                   reinterpret_cast<const SwapParams *>(dev.mat));
  check_launch("permutation kernel");
}

// -------------------------------------------------------------------------
// Pauli string: QubitVector::apply_pauli (qubitvector.hpp:2392-2433)
// -------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_pauli(T *__restrict__ psi, uint64_t x_mask, uint64_t z_mask, uint64_t x_max,
                                               T phase, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t mask_l = (1ULL << x_max) - 1;
  const uint64_t mask_u = ~((1ULL << (x_max + 1)) - 1);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    if (!x_mask) {
      T a = psi[i];
      if (z_mask && (__popcll(i & z_mask) & 1)) {
        a.x = -a.x;
        a.y = -a.y;
      }
      psi[i] = cmul(a, phase);
    } else {
      const uint64_t i0 = ((i << 1) & mask_u) | (i & mask_l);
      const uint64_t i1 = i0 ^ x_mask;
      T a0 = psi[i1], a1 = psi[i0];  // swapped
      if (z_mask && (__popcll(i0 & z_mask) & 1)) {
        a0.x = -a0.x;
        a0.y = -a0.y;
      }
      if (z_mask && (__popcll(i1 & z_mask) & 1)) {
        a1.x = -a1.x;
        a1.y = -a1.y;
      }
      psi[i0] = cmul(a0, phase);
      psi[i1] = cmul(a1, phase);
    }
  }
}

// DensityMatrix Y superoperator (densitymatrix.hpp:415-428) on (q, q+n):
// swap(0,3); (1,2) <- (-a2, -a1).
template <typename T>
__global__ void k_dm_y(T *__restrict__ psi, uint64_t m0, uint64_t m1, uint64_t b0, uint64_t b1, uint64_t ngroups) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
    uint64_t b = ((g & ~m0) << 1) | (g & m0);
    b = ((b & ~m1) << 1) | (b & m1);
    const T a0 = psi[b], a1 = psi[b | b0], a2 = psi[b | b1], a3 = psi[b | b0 | b1];
    T n1, n2;
    n1.x = -a2.x;
    n1.y = -a2.y;
    n2.x = -a1.x;
    n2.y = -a1.y;
    psi[b] = a3;
    psi[b | b0 | b1] = a0;
    psi[b | b0] = n1;
    psi[b | b1] = n2;
  }
}

template <typename T>
__global__ void k_scale(T *__restrict__ psi, T s, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) psi[i] = cmul(psi[i], s);
}

template <typename T>
__global__ void k_set_basis(T *__restrict__ psi, uint64_t index, T value, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    T z;
    z.x = 0;
    z.y = 0;
    psi[i] = i == index ? value : z;
  }
}

// complex128 <-> complex64 copies between a staging slice and the state, so
// that a complex64 state is filled from (and read back to) the ABI's
// complex128 host vectors at HBM speed.  Narrowing rounds to nearest, the
// same value as a C++ double -> float conversion on the host.
__global__ void k_narrow(const double2 *__restrict__ src, float2 *__restrict__ dst, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const double2 v = src[i];
    dst[i] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
  }
}
__global__ void k_copy_c128(const double2 *__restrict__ src, double2 *__restrict__ dst, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) dst[i] = src[i];
}
__global__ void k_widen(const float2 *__restrict__ src, double2 *__restrict__ dst, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const float2 v = src[i];
    dst[i] = make_double2(v.x, v.y);
  }
}

// -------------------------------------------------------------------------
// Reductions
// -------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v) {
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
  return s;  // valid in thread 0
}

// partials laid out [value][block]; out[v] = sum over blocks in order.
__global__ void k_finish(const double *__restrict__ partials, int nblocks, int nvalues, double *__restrict__ out) {
  for (int v = blockIdx.x; v < nvalues; v += gridDim.x) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(size_t)v * nblocks + b];
    s = block_sum(s);
    if (threadIdx.x == 0) out[v] = s;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_norm(const T *__restrict__ psi, uint64_t count, double *__restrict__ partials) {
  double acc = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const T a = psi[i];
    acc += (double)(a.x * a.x + a.y * a.y);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// Expectation values of many Pauli strings, term = blockIdx.y
// (QubitVector::expval_pauli, qubitvector.hpp:2299-2347).
struct TermDev {
  uint64_t x_mask, z_mask, x_max;
  double ph_re, ph_im;
  int diag_only;
};

template <typename T>
__global__ void __launch_bounds__(256) k_expval(const T *__restrict__ psi, int n, const TermDev *__restrict__ terms,
                                                double *__restrict__ partials) {
  const TermDev t = terms[blockIdx.y];
  using R = decltype(T::x);
  const R pr = (R)t.ph_re, pi = (R)t.ph_im;
  // complex64: short sums in float before the double accumulator (one FP64
  // add per 8 amplitudes instead of one per amplitude)
  constexpr int kChunk = sizeof(R) == 4 ? 8 : 1;
  double acc = 0.0;
  R part = 0;
  int cnt = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (!t.x_mask) {
    const uint64_t count = 1ULL << n;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
      const T a = psi[i];
      // real(phase * a * conj(a)) = Re(phase) * |a|^2 in the data precision
      R v = pr * (a.x * a.x + a.y * a.y);
      if (t.z_mask && (__popcll(i & t.z_mask) & 1)) v = -v;
      part += v;
      if (++cnt == kChunk) { acc += (double)part; part = 0; cnt = 0; }
    }
  } else {
    const uint64_t count = 1ULL << (n - 1);
    const uint64_t mask_l = (1ULL << t.x_max) - 1;
    const uint64_t mask_u = ~((1ULL << (t.x_max + 1)) - 1);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
      const uint64_t i0 = ((i << 1) & mask_u) | (i & mask_l);
      const uint64_t i1 = i0 ^ t.x_mask;
      const T a0 = psi[i0], a1 = psi[i1];
      // z = a1 * conj(a0); v0 = Re(phase * z), v1 = Re(phase * conj(z))
      const R zr = a1.x * a0.x + a1.y * a0.y;
      const R zi = a1.y * a0.x - a1.x * a0.y;
      R v0 = pr * zr - pi * zi;
      R v1 = pr * zr + pi * zi;
      if (t.z_mask && (__popcll(i0 & t.z_mask) & 1)) v0 = -v0;
      if (t.z_mask && (__popcll(i1 & t.z_mask) & 1)) v1 = -v1;
      part += v0 + v1;
      if (++cnt == kChunk) { acc += (double)part; part = 0; cnt = 0; }
    }
  }
  acc += (double)part;
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

// The same per state of a stack of 2^sb-amplitude states (one state per
// parameter binding): blockIdx.y = state, blockIdx.x = term * bps + slice,
// so that every term of a state runs back to back while the state is in L2;
// the terms act on qubits below sb (sb <= 31: 32-bit indices).  Per pair the
// kernel sums zr (s0 + s1) and zi (s1 - s0) with s = the Z-parity signs and
// applies the phase once at the end: Re(ph z) s0 + Re(ph conj z) s1 = pr zr
// (s0 + s1) + pi zi (s1 - s0).  complex64 keeps each thread's two sums in
// float with compensated (Kahan) addition and converts once, so that no FP64
// operation runs per amplitude (with a double add per 8 amplitudes the FP64
// pipe was 86 % busy and bounded the kernel); complex128 forms the products
// and the thread's sums as float pairs (compensated dot products,
// gbqv_fpair.cuh), then adds in double.
template <typename R>
struct SegSum {
  R s = 0, c = 0;
  __device__ __forceinline__ void add(R v) {
    if constexpr (sizeof(R) == 4) {
      const R y = v - c, t = s + y;
      c = (t - s) - y;
      s = t;
    } else {
      s += v;
    }
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

template <typename T>
__global__ void __launch_bounds__(256) k_expval_seg(const T *__restrict__ psi, int sb, int bps, uint64_t nseg,
                                                    uint64_t seg0, const TermDev *__restrict__ terms,
                                                    double *__restrict__ partials) {
  const uint32_t term = blockIdx.x / bps, slice = blockIdx.x % bps;
  const uint64_t seg = seg0 + blockIdx.y;
  const TermDev t = terms[term];
  using R = decltype(T::x);
  const T *ps = psi + (seg << sb);
  const uint32_t z = (uint32_t)t.z_mask, stride = (uint32_t)bps * blockDim.x;
  SegSum<R> A, B;
  double acc;
  if constexpr (sizeof(T) == 16) {
    // complex128: products and sums as float pairs (~48 bits, FP32 pipe;
    // conversions on the integer pipe), the thread's sums into double once
    fpair fa(0.0f), fb(0.0f);
    auto dbl2 = [](fpair v) { return fpair(2.0f * v.hi, 2.0f * v.lo); };
    if (!t.x_mask) {
      const uint32_t count = 1u << sb;
      for (uint32_t i = slice * blockDim.x + threadIdx.x; i < count; i += stride) {
        const fcx a = to_reg_pair(ps[i]);
        fp_dot d = fp_dot_first(a.x, a.x);
        fp_dot_add(d, a.y, a.y);
        const fpair v = fp_dot_done(d);
        fa = fa + ((__popc(i & z) & 1) ? -v : v);
      }
      acc = t.ph_re * fpair_to_double(fa);
    } else {
      const uint32_t count = 1u << (sb - 1), x = (uint32_t)t.x_mask;
      const uint32_t mask_l = (1u << t.x_max) - 1;
      for (uint32_t i = slice * blockDim.x + threadIdx.x; i < count; i += stride) {
        const uint32_t i0 = ((i & ~mask_l) << 1) | (i & mask_l), i1 = i0 ^ x;
        const fcx a0 = to_reg_pair(ps[i0]), a1 = to_reg_pair(ps[i1]);
        const bool n0 = __popc(i0 & z) & 1, n1 = __popc(i1 & z) & 1;
        if (n0 == n1) {  // 2 Re(a1 conj a0)
          fp_dot d = fp_dot_first(a1.x, a0.x);
          fp_dot_add(d, a1.y, a0.y);
          const fpair zr = dbl2(fp_dot_done(d));
          fa = fa + (n0 ? -zr : zr);
        } else {  // 2 Im(a1 conj a0)
          fp_dot d = fp_dot_first(a1.y, a0.x);
          fp_dot_add(d, -a1.x, a0.y);
          const fpair zi = dbl2(fp_dot_done(d));
          fb = fb + (n0 ? zi : -zi);
        }
      }
      acc = t.ph_re * fpair_to_double(fa) + t.ph_im * fpair_to_double(fb);
    }
  } else if (!t.x_mask) {
    const uint32_t count = 1u << sb;
    for (uint32_t i = slice * blockDim.x + threadIdx.x; i < count; i += stride) {
      const T a = ps[i];
      const R v = a.x * a.x + a.y * a.y;
      A.add((__popc(i & z) & 1) ? -v : v);
    }
    acc = t.ph_re * A.value();
  } else {
    const uint32_t count = 1u << (sb - 1), x = (uint32_t)t.x_mask;
    const uint32_t mask_l = (1u << t.x_max) - 1;
    for (uint32_t i = slice * blockDim.x + threadIdx.x; i < count; i += stride) {
      const uint32_t i0 = ((i & ~mask_l) << 1) | (i & mask_l), i1 = i0 ^ x;
      const T a0 = ps[i0], a1 = ps[i1];
      // z = a1 * conj(a0)
      const R zr = a1.x * a0.x + a1.y * a0.y;
      const R zi = a1.y * a0.x - a1.x * a0.y;
      const bool n0 = __popc(i0 & z) & 1, n1 = __popc(i1 & z) & 1;
      if (n0 == n1) {
        A.add(n0 ? -2 * zr : 2 * zr);
      } else {
        B.add(n0 ? 2 * zi : -2 * zi);
      }
    }
    acc = t.ph_re * A.value() + t.ph_im * B.value();
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[((size_t)term * nseg + seg) * bps + slice] = acc;
}

// UnitaryMatrix::initialize (unitarymatrix.hpp:236-247): entry (i, j) at
// i + 2^nq j is 1 on the diagonal.
template <typename T>
__global__ void k_set_identity(T *__restrict__ psi, int nq, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t low = (1ULL << nq) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    T z;
    z.x = (i & low) == (i >> nq) ? 1 : 0;
    z.y = 0;
    psi[i] = z;
  }
}

template <typename T>
__global__ void k_set_basis_seg(T *__restrict__ psi, int sb, uint64_t nvalid, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t low = (1ULL << sb) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    T z;
    z.x = ((i & low) == 0 && (i >> sb) < nvalid) ? 1 : 0;
    z.y = 0;
    psi[i] = z;
  }
}

// DensityMatrix::expval_pauli (densitymatrix.hpp:445-496): rho is 2^nq x 2^nq.
template <typename T>
__global__ void __launch_bounds__(256) k_dm_expval(const T *__restrict__ rho, int nq, const TermDev *__restrict__ terms,
                                                   double *__restrict__ partials) {
  const TermDev t = terms[blockIdx.y];
  using R = decltype(T::x);
  const uint64_t nrows = 1ULL << nq;
  double acc = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (!t.x_mask) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrows; i += stride) {
      R v = rho[i * (nrows + 1)].x;
      if (t.z_mask && (__popcll(i & t.z_mask) & 1)) v = -v;
      acc += (double)v;
    }
  } else {
    const R pr = (R)t.ph_re, pi = (R)t.ph_im;
    const uint64_t mask_l = (1ULL << t.x_max) - 1;
    const uint64_t mask_u = ~((1ULL << (t.x_max + 1)) - 1);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (nrows >> 1); i += stride) {
      const uint64_t iv = ((i << 1) & mask_u) | (i & mask_l);
      const T a = rho[(iv ^ t.x_mask) + nrows * iv];
      R v = 2 * (pr * a.x - pi * a.y);
      if (t.z_mask && (__popcll(iv & t.z_mask) & 1)) v = -v;
      acc += (double)v;
    }
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

template <typename T>
__global__ void __launch_bounds__(256) k_inner(const T *__restrict__ psi, const T *__restrict__ ck, uint64_t count,
                                               double *__restrict__ partials) {
  double re = 0.0, im = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const T a = psi[i], b = ck[i];
    // a * conj(b)
    re += (double)(a.x * b.x + a.y * b.y);
    im += (double)(a.y * b.x - a.x * b.y);
  }
  re = block_sum(re);
  if (threadIdx.x == 0) partials[blockIdx.x] = re;
  im = block_sum(im);
  if (threadIdx.x == 0) partials[gridDim.x + blockIdx.x] = im;
}

template <typename T>
__global__ void k_dm_trace(const T *__restrict__ rho, uint64_t nrows, double *__restrict__ partials) {
  double re = 0.0, im = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrows; i += stride) {
    const T a = rho[i * (nrows + 1)];
    re += (double)a.x;
    im += (double)a.y;
  }
  re = block_sum(re);
  if (threadIdx.x == 0) partials[blockIdx.x] = re;
  im = block_sum(im);
  if (threadIdx.x == 0) partials[gridDim.x + blockIdx.x] = im;
}

// Marginal probabilities over k <= 10 qubits (QubitVector::probabilities,
// qubitvector.hpp:2096-2143).  Bins [32*blockIdx.y, +32) per launch row;
// each thread accumulates its 32 bins in registers.
struct ProbParams {
  uint64_t offs[1 << 10];
  uint64_t lowmask[10];
  int k;
  uint64_t ngroups;
  uint64_t diag_stride;  // 0: statevector |a|^2; else density-matrix diagonal stride (nrows+1)
};

template <typename T>
__global__ void __launch_bounds__(256) k_probs(const T *__restrict__ psi, const ProbParams *__restrict__ p,
                                               double *__restrict__ partials) {
  const int D = 1 << p->k;
  const int bin0 = blockIdx.y * 32;
  const int nb = min(32, D - bin0);
  double acc[32];
#pragma unroll
  for (int b = 0; b < 32; ++b) acc[b] = 0.0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p->ngroups; g += stride) {
    const uint64_t base = insert_zeros(g, p->lowmask, p->k);
#pragma unroll
    for (int b = 0; b < 32; ++b) {
      if (b < nb) {
        const uint64_t idx = base + p->offs[bin0 + b];
        if (p->diag_stride) {
          acc[b] += (double)psi[idx * p->diag_stride].x;
        } else {
          const T a = psi[idx];
          acc[b] += (double)(a.x * a.x + a.y * a.y);
        }
      }
    }
  }
  for (int b = 0; b < nb; ++b) {
    const double s = block_sum(acc[b]);
    if (threadIdx.x == 0) partials[(size_t)(bin0 + b) * gridDim.x + blockIdx.x] = s;
  }
}

// Marginals over more than 10 qubits (probabilities(qubits),
// qubitvector.hpp:2106-2143, any k): one thread per outcome v and slice of
// the groups; outcome bit j sits at amplitude bit q[j], the group index
// fills the other bits in ascending order.  Slice s of outcome v sums groups
// s, s + bps, ... and writes partials[v * bps + s]; a second kernel adds the
// slices in order (deterministic).
struct ProbWide {
  uint8_t q[kMaxQubits];     // outcome bit j -> amplitude bit q[j]
  uint8_t free[kMaxQubits];  // group bit i -> amplitude bit free[i]
  int k, nfree;
  uint64_t diag_stride;
};

template <typename T>
__global__ void __launch_bounds__(256) k_probs_wide(const T *__restrict__ psi, const __grid_constant__ ProbWide w,
                                                    int bps, double *__restrict__ partials) {
  const uint64_t D = 1ULL << w.k;
  const uint64_t v = (uint64_t)(blockIdx.x / bps) * blockDim.x + threadIdx.x;
  const uint32_t slice = blockIdx.x % bps;
  if (v >= D) return;
  uint64_t off = 0;
  for (int j = 0; j < w.k; ++j) off |= ((v >> j) & 1ULL) << w.q[j];
  const uint64_t ngroups = 1ULL << w.nfree;
  double acc = 0.0;
  for (uint64_t g = slice; g < ngroups; g += bps) {
    uint64_t idx = off;
    for (int i = 0; i < w.nfree; ++i) idx |= ((g >> i) & 1ULL) << w.free[i];
    if (w.diag_stride) {
      acc += (double)psi[idx * w.diag_stride].x;
    } else {
      const T a = psi[idx];
      acc += (double)(a.x * a.x + a.y * a.y);
    }
  }
  partials[v * bps + slice] = acc;
}

__global__ void k_probs_wide_sum(const double *__restrict__ partials, int bps, uint64_t nvalues,
                                 double *__restrict__ out) {
  const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvalues) return;
  double s = 0.0;
  for (int b = 0; b < bps; ++b) s += partials[v * bps + b];
  out[v] = s;
}

template <typename T>
__global__ void k_probs_all(const T *__restrict__ psi, uint64_t count, uint64_t diag_stride, double *__restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    if (diag_stride) {
      out[i] = (double)psi[i * diag_stride].x;
    } else {
      const T a = psi[i];
      out[i] = (double)(a.x * a.x + a.y * a.y);
    }
  }
}

template <typename T>
T *st(Device &dev) { return reinterpret_cast<T *>(dev.state); }

void ensure_partials(Device &dev, size_t values) {
  grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * kReduceBlocks * values);
  grow(reinterpret_cast<void *&>(dev.results), dev.results_cap, sizeof(double) * values);
}

void finish(Device &dev, int nvalues, int nblocks = kReduceBlocks) {
  k_finish<<<std::min(nvalues, 1024), 256, 0, dev.stream>>>(dev.partials, nblocks, nvalues, dev.results);
  check_launch("reduction finish");
}

uint64_t diag_stride(const Device &dev) { return dev.density ? (1ULL << dev.nq) + 1 : 0; }
int sample_bits(const Device &dev) { return dev.density ? dev.nq : dev.n; }

}  // namespace

uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ============================== launchers ==============================

#define DISPATCH(dev, F, ...) ((dev).dbl ? F<double2>(__VA_ARGS__) : F<float2>(__VA_ARGS__))

void launch_dense(Device &dev, const reg_t &qubits, const cd *mat) { DISPATCH(dev, dense_any, dev, qubits, mat, false); }

void launch_diagonal(Device &dev, const reg_t &qubits, const cd *diag) { DISPATCH(dev, diag_any, dev, qubits, diag); }

void launch_mc(Device &dev, const reg_t &qubits, int kind, const cd *mat) { DISPATCH(dev, mc_any, dev, qubits, kind, mat); }

void launch_swaps(Device &dev, const reg_t &qubits, const std::vector<std::pair<uint32_t, uint32_t>> &pairs) {
  DISPATCH(dev, swaps_any, dev, qubits, pairs);
}

void launch_pauli(Device &dev, uint64_t x_mask, uint64_t z_mask, uint64_t x_max, cd phase) {
  const uint64_t count = x_mask ? dev.amps() >> 1 : dev.amps();
  const int grid = grid_for(count, 256);
  if (dev.dbl)
    k_pauli<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), x_mask, z_mask, x_max, to_dev<double2>(phase), count);
  else
    k_pauli<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), x_mask, z_mask, x_max, to_dev<float2>(phase), count);
  check_launch("pauli kernel");
}

void launch_dm_y(Device &dev, uint64_t q) {
  const uint64_t qa = q, qb = q + dev.nq;
  const uint64_t m0 = (1ULL << qa) - 1, m1 = (1ULL << qb) - 1;
  const uint64_t ngroups = dev.amps() >> 2;
  const int grid = grid_for(ngroups, 256);
  if (dev.dbl)
    k_dm_y<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), m0, m1, 1ULL << qa, 1ULL << qb, ngroups);
  else
    k_dm_y<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), m0, m1, 1ULL << qa, 1ULL << qb, ngroups);
  check_launch("density-matrix Y kernel");
}

void launch_scale(Device &dev, cd s) {
  const int grid = grid_for(dev.amps(), 256);
  if (dev.dbl)
    k_scale<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), to_dev<double2>(s), dev.amps());
  else
    k_scale<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), to_dev<float2>(s), dev.amps());
  check_launch("scale kernel");
}

void launch_set_basis(Device &dev, uint64_t index, cd value) {
  const int grid = grid_for(dev.amps(), 256);
  if (dev.dbl)
    k_set_basis<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), index, to_dev<double2>(value), dev.amps());
  else
    k_set_basis<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), index, to_dev<float2>(value), dev.amps());
  check_launch("initialize kernel");
}

void launch_narrow(Device &dev, const void *src, uint64_t offset, uint64_t count) {
  k_narrow<<<grid_for(count, 256), 256, 0, dev.stream>>>(static_cast<const double2 *>(src),
                                                          st<float2>(dev) + offset, count);
  check_launch("state narrowing kernel");
}

void launch_copy_in(Device &dev, const void *src, uint64_t offset, uint64_t count) {
  k_copy_c128<<<grid_for(count, 256), 256, 0, dev.stream>>>(static_cast<const double2 *>(src),
                                                             st<double2>(dev) + offset, count);
  check_launch("state copy kernel");
}

void launch_widen(Device &dev, uint64_t offset, uint64_t count, void *dst) {
  k_widen<<<grid_for(count, 256), 256, 0, dev.stream>>>(st<float2>(dev) + offset, static_cast<double2 *>(dst),
                                                         count);
  check_launch("state widening kernel");
}

void reduce_norm(Device &dev) {
  ensure_partials(dev, 1);
  if (dev.dbl)
    k_norm<double2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(st<double2>(dev), dev.amps(), dev.partials);
  else
    k_norm<float2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(st<float2>(dev), dev.amps(), dev.partials);
  check_launch("norm kernel");
  finish(dev, 1);
}

void reduce_norm_matrix(Device &dev, const reg_t &qubits, const cd *mat) {
  ensure_partials(dev, 1);
  DISPATCH(dev, dense_any, dev, qubits, mat, true);
  finish(dev, 1);
}

static void upload_terms(Device &dev, const std::vector<PauliTerm> &terms, TermDev **d_terms) {
  const size_t bytes = sizeof(TermDev) * terms.size();
  grow(dev.aux2, dev.aux2_cap, bytes);
  std::vector<TermDev> h(terms.size());
  for (size_t i = 0; i < terms.size(); ++i)
    h[i] = TermDev{terms[i].x_mask, terms[i].z_mask, terms[i].x_max, terms[i].ph_re, terms[i].ph_im, terms[i].diag_only};
  cuda_check(cudaMemcpyAsync(dev.aux2, h.data(), bytes, cudaMemcpyHostToDevice, dev.stream), "term upload");
  *d_terms = reinterpret_cast<TermDev *>(dev.aux2);
}

void reduce_expval(Device &dev, const std::vector<PauliTerm> &terms) {
  if (terms.empty()) return;
  if (terms.size() > (size_t)kMaxTerms) throw Error(1, "too many Pauli terms in one call");
  ensure_partials(dev, terms.size());
  TermDev *d_terms;
  upload_terms(dev, terms, &d_terms);
  dim3 grid(kReduceBlocks / 4, (unsigned)terms.size());
  if (dev.dbl)
    k_expval<double2><<<grid, kReduceThreads, 0, dev.stream>>>(st<double2>(dev), dev.n, d_terms, dev.partials);
  else
    k_expval<float2><<<grid, kReduceThreads, 0, dev.stream>>>(st<float2>(dev), dev.n, d_terms, dev.partials);
  check_launch("expval kernel");
  finish(dev, (int)terms.size(), kReduceBlocks / 4);
}

void reduce_expval_segments(Device &dev, const std::vector<PauliTerm> &terms, int state_bits, uint64_t nseg) {
  if (terms.empty() || nseg == 0) return;
  if (terms.size() > (size_t)kMaxTerms) throw Error(1, "too many Pauli terms in one call");
  if (state_bits > 31) throw Error(1, "stacked expectation values take states of at most 31 qubits");
  // blocks per state: about 8 blocks of 256 threads per SM over the whole launch
  const uint64_t want = std::max<uint64_t>(1, (uint64_t)kReduceBlocks / 4 / std::max<uint64_t>(nseg, 1));
  const uint64_t cap = std::max<uint64_t>(1, (1ULL << state_bits) / (2 * 256));
  const int bps = (int)std::min<uint64_t>(std::min<uint64_t>(want, cap), 1024);
  const size_t values = terms.size() * nseg;
  grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * values * bps);
  grow(reinterpret_cast<void *&>(dev.results), dev.results_cap, sizeof(double) * values);
  TermDev *d_terms;
  upload_terms(dev, terms, &d_terms);
  for (uint64_t s0 = 0; s0 < nseg; s0 += 65535) {  // grid y limit
    dim3 grid((unsigned)(terms.size() * bps), (unsigned)std::min<uint64_t>(65535, nseg - s0));
    if (dev.dbl)
      k_expval_seg<double2><<<grid, kReduceThreads, 0, dev.stream>>>(st<double2>(dev), state_bits, bps, nseg, s0,
                                                                     d_terms, dev.partials);
    else
      k_expval_seg<float2><<<grid, kReduceThreads, 0, dev.stream>>>(st<float2>(dev), state_bits, bps, nseg, s0,
                                                                    d_terms, dev.partials);
    check_launch("segmented expval kernel");
  }
  finish(dev, (int)values, bps);
}

void launch_set_identity(Device &dev) {
  const int grid = grid_for(dev.amps(), 256);
  if (dev.dbl)
    k_set_identity<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), dev.nq, dev.amps());
  else
    k_set_identity<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), dev.nq, dev.amps());
  check_launch("initialize kernel");
}

void launch_set_basis_segments(Device &dev, int state_bits, uint64_t count) {
  const int grid = grid_for(dev.amps(), 256);
  if (dev.dbl)
    k_set_basis_seg<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), state_bits, count, dev.amps());
  else
    k_set_basis_seg<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), state_bits, count, dev.amps());
  check_launch("initialize kernel");
}

void reduce_dm_expval(Device &dev, const std::vector<PauliTerm> &terms) {
  if (terms.empty()) return;
  if (terms.size() > (size_t)kMaxTerms) throw Error(1, "too many Pauli terms in one call");
  ensure_partials(dev, terms.size());
  TermDev *d_terms;
  upload_terms(dev, terms, &d_terms);
  dim3 grid(kReduceBlocks / 4, (unsigned)terms.size());
  if (dev.dbl)
    k_dm_expval<double2><<<grid, kReduceThreads, 0, dev.stream>>>(st<double2>(dev), dev.nq, d_terms, dev.partials);
  else
    k_dm_expval<float2><<<grid, kReduceThreads, 0, dev.stream>>>(st<float2>(dev), dev.nq, d_terms, dev.partials);
  check_launch("density-matrix expval kernel");
  finish(dev, (int)terms.size(), kReduceBlocks / 4);
}

void reduce_inner_product(Device &dev) {
  ensure_partials(dev, 2);
  if (dev.dbl)
    k_inner<double2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(
        st<double2>(dev), reinterpret_cast<const double2 *>(dev.ckpt), dev.amps(), dev.partials);
  else
    k_inner<float2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(
        st<float2>(dev), reinterpret_cast<const float2 *>(dev.ckpt), dev.amps(), dev.partials);
  check_launch("inner product kernel");
  finish(dev, 2);
}

void reduce_dm_trace(Device &dev) {
  ensure_partials(dev, 2);
  const uint64_t nrows = 1ULL << dev.nq;
  if (dev.dbl)
    k_dm_trace<double2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(st<double2>(dev), nrows, dev.partials);
  else
    k_dm_trace<float2><<<kReduceBlocks, kReduceThreads, 0, dev.stream>>>(st<float2>(dev), nrows, dev.partials);
  check_launch("trace kernel");
  finish(dev, 2);
}

// Marginals over k > 10 qubits into dev.results (2^k doubles).
void reduce_probabilities_wide(Device &dev, const reg_t &qubits) {
  const int k = (int)qubits.size();
  const int nbits = sample_bits(dev);
  ProbWide w{};
  w.k = k;
  uint64_t used = 0;
  for (int j = 0; j < k; ++j) {
    w.q[j] = (uint8_t)qubits[j];
    used |= 1ULL << qubits[j];
  }
  w.nfree = 0;
  for (int b = 0; b < nbits; ++b)
    if (!(used >> b & 1)) w.free[w.nfree++] = (uint8_t)b;
  w.diag_stride = diag_stride(dev);
  const uint64_t D = 1ULL << k, chunks = (D + 255) / 256;
  // slices: split the groups while the launch has fewer than ~8 CTAs per SM
  const uint64_t want = std::max<uint64_t>(1, (uint64_t)sm_count() * 8 / chunks);
  const int bps = (int)std::min<uint64_t>(std::min<uint64_t>(want, 1ULL << w.nfree), 64);
  if (chunks * bps > 0x7fffffffULL) throw Error(1, "marginal probabilities: too many outcomes");
  grow(reinterpret_cast<void *&>(dev.results), dev.results_cap, sizeof(double) * D);
  double *dst = dev.results;
  if (bps > 1) {
    grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * D * bps);
    dst = dev.partials;
  }
  if (dev.dbl)
    k_probs_wide<double2><<<(unsigned)(chunks * bps), 256, 0, dev.stream>>>(st<double2>(dev), w, bps, dst);
  else
    k_probs_wide<float2><<<(unsigned)(chunks * bps), 256, 0, dev.stream>>>(st<float2>(dev), w, bps, dst);
  check_launch("probabilities kernel");
  if (bps > 1) {
    k_probs_wide_sum<<<(unsigned)chunks, 256, 0, dev.stream>>>(dev.partials, bps, D, dev.results);
    check_launch("probabilities sum");
  }
}

void reduce_probabilities(Device &dev, const reg_t &qubits) {
  const int k = (int)qubits.size();
  if (k > 10) return reduce_probabilities_wide(dev, qubits);
  if (k < 1) throw Error(1, "marginal probabilities over no qubits: use the full distribution");
  const int D = 1 << k;
  ensure_partials(dev, D);
  auto p = std::make_unique<ProbParams>();
  local_offsets(qubits, p->offs);
  sorted_masks(qubits, p->lowmask);
  p->k = k;
  const int nbits = sample_bits(dev);
  p->ngroups = (1ULL << nbits) >> k;
  p->diag_stride = diag_stride(dev);
  grow(dev.aux2, dev.aux2_cap, sizeof(ProbParams));
  cuda_check(cudaMemcpyAsync(dev.aux2, p.get(), sizeof(ProbParams), cudaMemcpyHostToDevice, dev.stream),
             "probabilities upload");
  dim3 grid(kReduceBlocks / 4, (D + 31) / 32);
  if (dev.dbl)
    k_probs<double2><<<grid, kReduceThreads, 0, dev.stream>>>(st<double2>(dev),
                                                              reinterpret_cast<const ProbParams *>(dev.aux2), dev.partials);
  else
    k_probs<float2><<<grid, kReduceThreads, 0, dev.stream>>>(st<float2>(dev),
                                                             reinterpret_cast<const ProbParams *>(dev.aux2), dev.partials);
  check_launch("probabilities kernel");
  finish(dev, D, kReduceBlocks / 4);
}

void probabilities_all(Device &dev, double *d_out) {
  const uint64_t count = 1ULL << sample_bits(dev);
  const int grid = grid_for(count, 256);
  if (dev.dbl)
    k_probs_all<double2><<<grid, 256, 0, dev.stream>>>(st<double2>(dev), count, diag_stride(dev), d_out);
  else
    k_probs_all<float2><<<grid, 256, 0, dev.stream>>>(st<float2>(dev), count, diag_stride(dev), d_out);
  check_launch("probabilities kernel");
}


// ============================ complex128 on tensor cores ============================
// Dense k-qubit gates (k = 4, 5) on a complex128 state with FP64 emulated by
// exact digit slices (gbqv_ozaki.h): each group's 2^(k+1) real parts are
// split into six bf16 digit planes against the group's exponent, the real
// form of the matrix [[Re U, -Im U], [Im U, Re U]] into six planes against
// each row's exponent (host), the 21 plane products with s + t <= 5 run as
// bf16 MMAs with exact FP32 accumulation per level, and the six level sums
// are recombined exactly in int64 and rounded once to double.  GB300 runs
// DFMA at 1.2 TFLOP/s; this path uses the tensor pipe and integer units.
namespace {

template <int KQ>
struct OzCfg {
  static constexpr int D = 1 << KQ;          // amplitudes per group
  static constexpr int R = 2 * D;            // reals per group (matrix dim)
  static constexpr int MT = R / 16;          // m-tiles of the real matrix
  static constexpr int KS = R / 16;          // k-steps
  static constexpr int MC = 2;               // m-tiles whose level sums are live at once
  static constexpr int G = 64;               // groups per CTA iteration: 8 warps x 8 (one n-tile)
  static constexpr int TPG = 256 / G;        // threads per group in load / store (4)
  static constexpr int APT = D / TPG;        // amplitudes per thread
  static constexpr int PSTRIDE = R + 8;      // bf16 per digit-plane row (bank-conflict pad)
  static constexpr size_t plane_bytes = sizeof(uint16_t) * 6 * G * PSTRIDE;
  static constexpr size_t frag_bytes = sizeof(uint4) * 6 * MT * KS * 32;
  static constexpr size_t stage_bytes = sizeof(double2) * G * (D + 1);
  static constexpr size_t smem = (plane_bytes > stage_bytes ? plane_bytes : stage_bytes) + frag_bytes +
                                 sizeof(int) * (G + R);
};

template <int KQ>
struct OzParams {
  uint64_t offs[1 << KQ];
  uint64_t lowmask[KQ];
  uint64_t ngroups;
  int rowkey[2 << KQ];
};

// bf16 bits of a small integer (|v| <= 256, exact): float via the 2^23 magic
// add (FP32 pipe), then the top half of the float word.
__device__ __forceinline__ uint32_t int_to_bf16(int v) {
  const float f = __int_as_float(0x4B000000 + v + 512) - 8389120.0f;  // 2^23 + 512
  return (uint32_t)__float_as_uint(f) >> 16;
}

__device__ __forceinline__ void mma_bf16(float *c, const uint4 &a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

// Each warp owns 8 groups (one 8-column n-tile).  For a pair of m-tiles the
// six level sums stay live in registers (48 floats) while the k-steps run:
// a matrix fragment of plane t feeds the MMAs with every state plane s <=
// 5 - t, each into a different level accumulator, so consecutive MMAs are
// independent.
template <int KQ>
__global__ void __launch_bounds__(256, 2) k_dense_oz(double2 *__restrict__ psi, const __grid_constant__ OzParams<KQ> p,
                                                     const uint4 *__restrict__ gfrag) {
  using Cfg = OzCfg<KQ>;
  constexpr int D = Cfg::D, R = Cfg::R, MT = Cfg::MT, KS = Cfg::KS, MC = Cfg::MC, G = Cfg::G;
  constexpr int TPG = Cfg::TPG, APT = Cfg::APT, PS = Cfg::PSTRIDE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t *planes = reinterpret_cast<uint16_t *>(smem_raw);
  double2 *stage = reinterpret_cast<double2 *>(smem_raw);
  constexpr size_t big = Cfg::plane_bytes > Cfg::stage_bytes ? Cfg::plane_bytes : Cfg::stage_bytes;
  uint4 *frag = reinterpret_cast<uint4 *>(smem_raw + big);
  int *colkey = reinterpret_cast<int *>(smem_raw + big + Cfg::frag_bytes);
  int *rowkey = colkey + G;
  for (int i = threadIdx.x; i < 6 * MT * KS * 32; i += blockDim.x) frag[i] = gfrag[i];
  for (int i = threadIdx.x; i < R; i += blockDim.x) rowkey[i] = p.rowkey[i];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, gid = lane >> 2, tig = lane & 3;
  const uint64_t ntiles = (p.ngroups + G - 1) / G;
  // thread -> (group g, amplitude pairs): the thread owns amplitudes
  // 2*(tid % TPG) + 2*TPG*i + {0, 1}, i < APT/2 (adjacent pairs pack into one
  // 32-bit word of a digit plane)
  const int g = tid / TPG, pr0 = 2 * (tid % TPG);
  auto amp_of = [&](int i) { return pr0 + 2 * TPG * (i >> 1) + (i & 1); };
  double2 v[APT];
  uint64_t tile = blockIdx.x;
  uint64_t base = 0;
  bool valid = false;
  auto load_tile = [&](uint64_t t, double2 *dst, uint64_t &b, bool &ok) {
    const uint64_t grp = t * G + g;
    ok = t < ntiles && grp < p.ngroups;
    b = ok ? insert_zeros_k<KQ>(grp, p.lowmask) : 0;
#pragma unroll
    for (int i = 0; i < APT; ++i) dst[i] = ok ? psi[b + p.offs[amp_of(i)]] : make_double2(0.0, 0.0);
  };
  // 4-qubit gates prefetch the next tile into registers (APT = 4 keeps it
  // spill-free); 5-qubit gates (APT = 8) load at the top of each iteration
  constexpr bool kPrefetch = KQ == 4;
  if (kPrefetch) load_tile(tile, v, base, valid);
  for (; tile < ntiles; tile += gridDim.x) {
    if (!kPrefetch) load_tile(tile, v, base, valid);
    // ---- split the tile loaded (or prefetched) for this iteration ----
    int key = 0;
#pragma unroll
    for (int i = 0; i < APT; ++i) key = max(key, max(oz::exp_key(v[i].x), oz::exp_key(v[i].y)));
#pragma unroll
    for (int o = 1; o < TPG; o <<= 1) key = max(key, __shfl_xor_sync(0xffffffffu, key, o));
    __syncthreads();  // previous tile's staging reads are done
    if (tid % TPG == 0) colkey[g] = key;
#pragma unroll
    for (int i = 0; i < APT; i += 2) {
      int32_t dr0[6], dr1[6], di0[6], di1[6];
      oz::split6(v[i].x, key, dr0);
      oz::split6(v[i + 1].x, key, dr1);
      oz::split6(v[i].y, key, di0);
      oz::split6(v[i + 1].y, key, di1);
      const int a = amp_of(i);
#pragma unroll
      for (int sl = 0; sl < 6; ++sl) {
        uint32_t *row = reinterpret_cast<uint32_t *>(planes + ((size_t)sl * G + g) * PS);
        row[a >> 1] = int_to_bf16(dr0[sl]) | (int_to_bf16(dr1[sl]) << 16);
        row[(D + a) >> 1] = int_to_bf16(di0[sl]) | (int_to_bf16(di1[sl]) << 16);
      }
    }
    const uint64_t cur_base = base;
    const bool cur_valid = valid;
    // ---- prefetch the next tile: its loads fly during the MMAs below ----
    if (kPrefetch) load_tile(tile + gridDim.x, v, base, valid);
    __syncthreads();
    // ---- tensor-core level sums, then exact recombination ----
    const int gw = warp * 8 + gid;  // this lane's B column (group)
    int64_t out64[MT][4];
#pragma unroll
    for (int mc = 0; mc < MT; mc += MC) {
      float acc[6][MC][4];
#pragma unroll
      for (int l = 0; l < 6; ++l)
#pragma unroll
        for (int j = 0; j < MC; ++j)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[l][j][c] = 0.f;
#pragma unroll
      for (int ks = 0; ks < KS; ++ks) {
        uint32_t b0[6], b1[6];
#pragma unroll
        for (int sl = 0; sl < 6; ++sl) {
          const uint32_t *row = reinterpret_cast<const uint32_t *>(planes + ((size_t)sl * G + gw) * PS);
          b0[sl] = row[ks * 8 + tig];
          b1[sl] = row[ks * 8 + 4 + tig];
        }
#pragma unroll
        for (int t = 0; t < 6; ++t)
#pragma unroll
          for (int j = 0; j < MC; ++j) {
            const uint4 af = frag[((t * MT + mc + j) * KS + ks) * 32 + lane];
#pragma unroll
            for (int sl = 0; sl + t < 6; ++sl) mma_bf16(acc[t + sl][j], af, b0[sl], b1[sl]);
          }
      }
#pragma unroll
      for (int j = 0; j < MC; ++j)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          // level sums are exact integers below 2^22 in magnitude, so a pair
          // (l, l+1) combines exactly in int32: T_l * 256 + T_{l+1} < 2^31
          const int32_t p01 = __float2int_rn(acc[0][j][c]) * 256 + __float2int_rn(acc[1][j][c]);
          const int32_t p23 = __float2int_rn(acc[2][j][c]) * 256 + __float2int_rn(acc[3][j][c]);
          const int32_t p45 = __float2int_rn(acc[4][j][c]) * 256 + __float2int_rn(acc[5][j][c]);
          out64[mc + j][c] = (int64_t)p01 * 4294967296LL + (int64_t)p23 * 65536LL + (int64_t)p45;
        }
    }
    __syncthreads();  // planes are dead; reuse the space as output staging
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int r = mt * 16 + gid + 8 * (c >> 1);
        const int gg = warp * 8 + 2 * tig + (c & 1);
        const int ck = colkey[gg];
        const double y = (ck == 0) ? 0.0 : oz::i64_to_double(out64[mt][c], oz::out_scale(rowkey[r], ck));
        double *slot = reinterpret_cast<double *>(&stage[gg * (D + 1) + (r % D)]);
        slot[r < D ? 0 : 1] = y;
      }
    __syncthreads();
    if (cur_valid) {
#pragma unroll
      for (int i = 0; i < APT; ++i) psi[cur_base + p.offs[amp_of(i)]] = stage[g * (D + 1) + amp_of(i)];
    }
  }
}

// Host: digit planes of the real matrix, in mma.sync A-fragment order.
template <int KQ>
void oz_matrix(const cd *mat, std::vector<uint4> &frag, int *rowkey) {
  using Cfg = OzCfg<KQ>;
  constexpr int D = Cfg::D, R = Cfg::R, MT = Cfg::MT, KS = Cfg::KS;
  std::vector<double> A((size_t)R * R);
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) {
      const cd z = mat[r + (size_t)D * c];
      A[(size_t)r * R + c] = z.real();
      A[(size_t)r * R + c + D] = -z.imag();
      A[(size_t)(r + D) * R + c] = z.imag();
      A[(size_t)(r + D) * R + c + D] = z.real();
    }
  std::vector<int32_t> dig((size_t)6 * R * R);
  for (int r = 0; r < R; ++r) {
    int key = 0;
    for (int c = 0; c < R; ++c) key = std::max(key, oz::exp_key(A[(size_t)r * R + c]));
    rowkey[r] = key;
    for (int c = 0; c < R; ++c) {
      int32_t d[6];
      oz::split6(A[(size_t)r * R + c], key, d);
      for (int sl = 0; sl < 6; ++sl) dig[((size_t)sl * R + r) * R + c] = d[sl];
    }
  }
  auto bf = [](int32_t v) -> uint32_t {
    float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u >> 16;
  };
  auto pk = [&](int sl, int r, int c) -> uint32_t {
    return bf(dig[((size_t)sl * R + r) * R + c]) | (bf(dig[((size_t)sl * R + r) * R + c + 1]) << 16);
  };
  frag.resize((size_t)6 * MT * KS * 32);
  for (int sl = 0; sl < 6; ++sl)
    for (int mt = 0; mt < MT; ++mt)
      for (int ks = 0; ks < KS; ++ks)
        for (int lane = 0; lane < 32; ++lane) {
          const int gid = lane >> 2, tig = lane & 3;
          const int r0 = mt * 16 + gid, c0 = ks * 16 + 2 * tig;
          uint4 f;
          f.x = pk(sl, r0, c0);
          f.y = pk(sl, r0 + 8, c0);
          f.z = pk(sl, r0, c0 + 8);
          f.w = pk(sl, r0 + 8, c0 + 8);
          frag[((sl * MT + mt) * KS + ks) * 32 + lane] = f;
        }
}

template <int KQ>
void dense_oz(Device &dev, const reg_t &qubits, const cd *mat) {
  using Cfg = OzCfg<KQ>;
  OzParams<KQ> p;
  local_offsets(qubits, p.offs);
  sorted_masks(qubits, p.lowmask);
  p.ngroups = dev.amps() >> KQ;
  std::vector<uint4> frag;
  oz_matrix<KQ>(mat, frag, p.rowkey);
  const size_t fb = frag.size() * sizeof(uint4);
  grow(dev.mat, dev.mat_cap, fb);
  cuda_check(cudaMemcpyAsync(dev.mat, frag.data(), fb, cudaMemcpyHostToDevice, dev.stream), "matrix upload");
  static bool attr[2] = {false, false};
  if (!attr[KQ - 4]) {
    cuda_check(cudaFuncSetAttribute(k_dense_oz<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::smem),
               "tensor-core kernel attribute");
    attr[KQ - 4] = true;
  }
  int per_sm = 1;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_oz<KQ>, 256, Cfg::smem), "occupancy");
  const uint64_t ntiles = (p.ngroups + Cfg::G - 1) / Cfg::G;
  const uint64_t grid = std::min<uint64_t>(ntiles, 152ULL * std::max(per_sm, 1));
  k_dense_oz<KQ><<<(unsigned)grid, 256, Cfg::smem, dev.stream>>>(reinterpret_cast<double2 *>(dev.state), p,
                                                                 reinterpret_cast<const uint4 *>(dev.mat));
  check_launch("tensor-core complex128 dense kernel");
}

}  // namespace

// 2- and 3-qubit complex128 gates ride the 4-qubit tcgen05 kernel as U (x) I
// on idle qubits: one HBM pass at the tensor path's speed instead of an
// FP64-bound pass (8 2^k flops per amplitude at 1.2 TFLOP/s).
bool tensor_dense_available(const Device &dev, int k) {
  return dev.dbl && dev.tensor_c128 && (k == 4 || k == 5 || ((k == 2 || k == 3) && tc_dense_available(dev, 4)));
}

void launch_dense_tensor(Device &dev, const reg_t &qubits, const cd *mat) {
  const int k = (int)qubits.size();
  if (k < 4) {
    // extra targets: the highest qubits not acted on (index bits k..3)
    reg_t q = qubits;
    for (int b = dev.n - 1; (int)q.size() < 4; --b)
      if (std::find(qubits.begin(), qubits.end(), (uint64_t)b) == qubits.end()) q.push_back((uint64_t)b);
    const int d = 1 << k;
    std::vector<cd> u(256, cd(0.0, 0.0));
    for (int i = 0; i < 16; ++i)
      for (int j = 0; j < 16; ++j)
        if ((i >> k) == (j >> k)) u[i + 16 * j] = mat[(i & (d - 1)) + (size_t)d * (j & (d - 1))];
    launch_dense_tc(dev, q, u.data());
    return;
  }
  if (tc_dense_available(dev, k))
    launch_dense_tc(dev, qubits, mat);
  else if (qubits.size() == 4)
    dense_oz<4>(dev, qubits, mat);
  else if (tc5_usable(dev, qubits))
    launch_dense_tc5(dev, qubits, mat);
  else
    dense_oz<5>(dev, qubits, mat);
}

// ============================ adjoint-gradient kernels ============================
// (Pψ)[i] = phase * (-1)^{popcount(i & z)} * ψ[i ^ x] for a Pauli string with
// masks (x, z) and phase (-i)^{num_y} (QubitVector::apply_pauli,
// qubitvector.hpp:2392-2433, written as a gather).
namespace {

struct HamTermDev {
  uint64_t x_mask, z_mask;
  double re, im;  // coeff * (-i)^{num_y}
};
constexpr int kHamCache = 512;  // terms staged in shared memory

// out = sum_t c_t P_t psi  (one pass writing out, gathers from psi per term)
template <typename T>
__global__ void __launch_bounds__(256) k_ham_apply(const T *__restrict__ psi, T *__restrict__ out, uint64_t count,
                                                   const HamTermDev *__restrict__ terms, int nterms) {
  using R = decltype(T::x);
  // complex64: the products in float and the sums compensated (Kahan) in
  // float, so that no FP64 operation runs per term (with a double add per 8
  // terms the FP64 pipe bounded the kernel); complex128: everything in double
  // the terms with their coefficients in the data precision, once per CTA
  // (a double -> float conversion per amplitude and term ran on the FP64
  // pipe and bounded the kernel at complex64)
  __shared__ uint64_t s_x[kHamCache], s_z[kHamCache];
  __shared__ R s_re[kHamCache], s_im[kHamCache];
  const bool staged = nterms <= kHamCache;
  if (staged)
    for (int t = threadIdx.x; t < nterms; t += blockDim.x) {
      const HamTermDev h = terms[t];
      s_x[t] = h.x_mask;
      s_z[t] = h.z_mask;
      s_re[t] = (R)h.re;
      s_im[t] = (R)h.im;
    }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    SegSum<R> ar, ai;
#pragma unroll 4
    for (int t = 0; t < nterms; ++t) {
      uint64_t xm, zm;
      R cr, ci;
      if (staged) {
        xm = s_x[t];
        zm = s_z[t];
        cr = s_re[t];
        ci = s_im[t];
      } else {
        const HamTermDev h = terms[t];
        xm = h.x_mask;
        zm = h.z_mask;
        cr = (R)h.re;
        ci = (R)h.im;
      }
      const T a = psi[i ^ xm];
      if (__popcll(i & zm) & 1) { cr = -cr; ci = -ci; }
      ar.add(cr * a.x - ci * a.y);
      ai.add(cr * a.y + ci * a.x);
    }
    T o;
    o.x = (R)ar.value();
    o.y = (R)ai.value();
    out[i] = o;
  }
}

// sum_i conj(lam[i]) (P psi)[i] for one Pauli string, FP64 partials [re | im]
template <typename T>
__global__ void __launch_bounds__(256) k_pauli_inner(const T *__restrict__ lam, const T *__restrict__ psi, uint64_t count,
                                                     uint64_t x_mask, uint64_t z_mask, double ph_re, double ph_im,
                                                     double *__restrict__ partials) {
  using R = decltype(T::x);
  // complex64: products and short sums (8 amplitudes) in float, then into
  // the double sums; complex128: everything in double
  constexpr int kChunk = sizeof(R) == 4 ? 8 : 1;
  double re = 0.0, im = 0.0;
  R sr = 0, si = 0;
  int cnt = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const T l = lam[i], a = psi[i ^ x_mask];
    // conj(l) * a
    R zr = l.x * a.x + l.y * a.y;
    R zi = l.x * a.y - l.y * a.x;
    if (__popcll(i & z_mask) & 1) { zr = -zr; zi = -zi; }
    sr += zr;
    si += zi;
    if (++cnt == kChunk) {
      re += (double)sr;
      im += (double)si;
      sr = 0;
      si = 0;
      cnt = 0;
    }
  }
  re += (double)sr;
  im += (double)si;
  // times the phase
  const double pr = re * ph_re - im * ph_im, pi = re * ph_im + im * ph_re;
  const double r = block_sum(pr);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
  const double q = block_sum(pi);
  if (threadIdx.x == 0) partials[gridDim.x + blockIdx.x] = q;
}

// Adjoint sweep steps for 1-qubit gates: the generator's Im <lam|P|psi>
// contribution (P = phase X^x Z^z with x, z within the gate's bit, the sign
// taken on lam's index as in k_pauli_inner) from the amplitudes as they are,
// then psi <- M psi and lam <- M lam with M = the gate's inverse,
// column-major: one read and one write of each state instead of the inner
// product's read of both and two gate passes.  form: 0 general 2x2, 1 real
// 2x2 (RY, H), 2 diagonal (RZ, phases).
struct AdjMat {
  double re[4], im[4];
};

// The adjoint sweep of a complex128 state with psi and lam held as float
// pairs (fcx, 16 bytes like a double2) for the whole sweep: converted once,
// then every step runs on the FP32 pipe without touching FP64; the sweep's
// final states are not needed, only the inner products.
__global__ void __launch_bounds__(256) k_to_pairs(double2 *__restrict__ a, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    reinterpret_cast<fcx *>(a)[i] = to_reg_pair(a[i]);
}

// lam = H psi on float pairs: psi and lam as fcx, the coefficients c_t =
// coeff_t (-i)^{num_y} as pairs (split on the host); the sign (-1)^{popc(i &
// z)} and the gather psi[i ^ x] as in k_ham_apply.
struct HamTermPair {
  uint64_t x_mask, z_mask;
  float re_hi, re_lo, im_hi, im_lo;
};

__global__ void __launch_bounds__(256) k_ham_apply_pairs(const fcx *__restrict__ psi, fcx *__restrict__ out,
                                                         uint64_t count, const HamTermPair *__restrict__ terms,
                                                         int nterms) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    fpair sr(0.0f), si(0.0f);
    for (int t = 0; t < nterms; ++t) {
      const HamTermPair h = terms[t];
      const fcx a = psi[i ^ h.x_mask];
      fpair cr(h.re_hi, h.re_lo), ci(h.im_hi, h.im_lo);
      if (__popcll(i & h.z_mask) & 1) {
        cr = -cr;
        ci = -ci;
      }
      sr = sr + (cr * a.x - ci * a.y);
      si = si + (cr * a.y + ci * a.x);
    }
    fcx o;
    o.x = sr;
    o.y = si;
    out[i] = o;
  }
}

__global__ void __launch_bounds__(256) k_from_pairs(double2 *__restrict__ a, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    a[i] = from_reg(reinterpret_cast<const fcx *>(a)[i], double2());
}

__device__ __forceinline__ void adj_apply_pairs(fcx &x0, fcx &x1, const fcx (&m)[4], int form) {
  const fcx a = x0, b = x1;
  if (form == 2) {
    x0.x = a.x * m[0].x - a.y * m[0].y;
    x0.y = a.x * m[0].y + a.y * m[0].x;
    x1.x = b.x * m[3].x - b.y * m[3].y;
    x1.y = b.x * m[3].y + b.y * m[3].x;
  } else if (form == 1) {
    x0.x = rfma(m[2].x, b.x, m[0].x * a.x);
    x0.y = rfma(m[2].x, b.y, m[0].x * a.y);
    x1.x = rfma(m[3].x, b.x, m[1].x * a.x);
    x1.y = rfma(m[3].x, b.y, m[1].x * a.y);
  } else {
    x0.x = m[0].x * a.x - m[0].y * a.y + m[2].x * b.x - m[2].y * b.y;
    x0.y = m[0].x * a.y + m[0].y * a.x + m[2].x * b.y + m[2].y * b.x;
    x1.x = m[1].x * a.x - m[1].y * a.y + m[3].x * b.x - m[3].y * b.y;
    x1.y = m[1].x * a.y + m[1].y * a.x + m[3].x * b.y + m[3].y * b.x;
  }
}

__global__ void __launch_bounds__(256) k_adj_step_pairs(fcx *__restrict__ psi, fcx *__restrict__ lam, uint64_t npairs,
                                                        int q, const AdjMat M, int form, int gx, int gz, int inner,
                                                        int apply, double ph_re, double ph_im,
                                                        double *__restrict__ partials) {
  fcx m[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    m[j].x = fpair_from_double(M.re[j]);
    m[j].y = fpair_from_double(M.im[j]);
  }
  fpair sr(0.0f), si(0.0f);
  const uint64_t bit = 1ULL << q, lowm = bit - 1;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += stride) {
    const uint64_t i0 = ((i & ~lowm) << 1) | (i & lowm), i1 = i0 | bit;
    fcx a0 = psi[i0], a1 = psi[i1], l0 = lam[i0], l1 = lam[i1];
    if (inner) {
      const fcx p0 = gx ? a1 : a0, p1 = gx ? a0 : a1;
      const fpair zr = l0.x * p0.x + l0.y * p0.y, zi = l0.x * p0.y - l0.y * p0.x;
      const fpair wr = l1.x * p1.x + l1.y * p1.y, wi = l1.x * p1.y - l1.y * p1.x;
      sr = sr + (gz ? zr - wr : zr + wr);
      si = si + (gz ? zi - wi : zi + wi);
    }
    if (apply) {
      adj_apply_pairs(a0, a1, m, form);
      adj_apply_pairs(l0, l1, m, form);
      psi[i0] = a0;
      psi[i1] = a1;
      lam[i0] = l0;
      lam[i1] = l1;
    }
  }
  if (!inner) return;
  const double re = fpair_to_double(sr), im = fpair_to_double(si);
  const double pr = re * ph_re - im * ph_im, pi = re * ph_im + im * ph_re;
  const double r = block_sum(pr);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
  const double s = block_sum(pi);
  if (threadIdx.x == 0) partials[gridDim.x + blockIdx.x] = s;
}

// K consecutive 1-qubit steps of the adjoint sweep on K distinct qubits in
// one pass: each thread holds a group of 2^K amplitudes of psi and lam
// (local bit j <-> the qubit of step j) and runs the steps in sweep order,
// each step's inner product from the values its predecessors left.  HBM
// traffic per step falls by K.  E: float2 / double2 (plain arithmetic) or
// fcx (complex128 as float pairs).
struct AdjStepDev {
  int q, form, gx, gz, inner;
  double re[4], im[4];
  double ph_re, ph_im;
};
template <int K>
struct AdjSteps {
  AdjStepDev s[K];
  uint64_t lowmask[K];  // (1 << q) - 1 of the step qubits, ascending
};

template <typename E>
struct AdjReal {
  using type = decltype(E::x);
};
template <>
struct AdjReal<fcx> {
  using type = fpair;
};

template <typename E>
__device__ __forceinline__ E adj_mat(double re, double im) {
  E z;
  if constexpr (std::is_same<E, fcx>::value) {
    z.x = fpair_from_double(re);
    z.y = fpair_from_double(im);
  } else {
    z.x = (decltype(E::x))re;
    z.y = (decltype(E::x))im;
  }
  return z;
}

template <typename E>
__device__ __forceinline__ void adj_apply_g(E &x0, E &x1, const E (&m)[4], int form) {
  const E a = x0, b = x1;
  if (form == 2) {
    x0.x = a.x * m[0].x - a.y * m[0].y;
    x0.y = a.x * m[0].y + a.y * m[0].x;
    x1.x = b.x * m[3].x - b.y * m[3].y;
    x1.y = b.x * m[3].y + b.y * m[3].x;
  } else if (form == 1) {
    x0.x = rfma(m[2].x, b.x, m[0].x * a.x);
    x0.y = rfma(m[2].x, b.y, m[0].x * a.y);
    x1.x = rfma(m[3].x, b.x, m[1].x * a.x);
    x1.y = rfma(m[3].x, b.y, m[1].x * a.y);
  } else {
    x0.x = m[0].x * a.x - m[0].y * a.y + m[2].x * b.x - m[2].y * b.y;
    x0.y = m[0].x * a.y + m[0].y * a.x + m[2].x * b.y + m[2].y * b.x;
    x1.x = m[1].x * a.x - m[1].y * a.y + m[3].x * b.x - m[3].y * b.y;
    x1.y = m[1].x * a.y + m[1].y * a.x + m[3].x * b.y + m[3].y * b.x;
  }
}

template <typename E>
__device__ __forceinline__ double adj_to_double(E) { return 0.0; }

template <typename E, int K>
__global__ void __launch_bounds__(256) k_adj_steps(E *__restrict__ psi, E *__restrict__ lam, uint64_t ngroups,
                                                   const AdjSteps<K> S, double *__restrict__ partials) {
  using R = typename AdjReal<E>::type;
  constexpr int G = 1 << K;
  E m[K][4];
#pragma unroll
  for (int j = 0; j < K; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) m[j][e] = adj_mat<E>(S.s[j].re[e], S.s[j].im[e]);
  double accr[K], acci[K];
#pragma unroll
  for (int j = 0; j < K; ++j) accr[j] = acci[j] = 0.0;
  R fr[K], fi[K];  // per-group sums (fcx: carried across groups in pairs)
#pragma unroll
  for (int j = 0; j < K; ++j) fr[j] = fi[j] = R(0.0f);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
    uint64_t base = g;
#pragma unroll
    for (int j = 0; j < K; ++j) base = ((base & ~S.lowmask[j]) << 1) | (base & S.lowmask[j]);
    E a[G], l[G];
#pragma unroll
    for (int t = 0; t < G; ++t) {
      uint64_t idx = base;
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (t >> j & 1) idx |= 1ULL << S.s[j].q;
      a[t] = psi[idx];
      l[t] = lam[idx];
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const AdjStepDev &st = S.s[j];
#pragma unroll
      for (int t = 0; t < G; ++t) {
        if (t >> j & 1) continue;
        const int t1 = t | (1 << j);
        if (st.inner) {
          const E p0 = st.gx ? a[t1] : a[t], p1 = st.gx ? a[t] : a[t1];
          const R zr = l[t].x * p0.x + l[t].y * p0.y, zi = l[t].x * p0.y - l[t].y * p0.x;
          const R wr = l[t1].x * p1.x + l[t1].y * p1.y, wi = l[t1].x * p1.y - l[t1].y * p1.x;
          fr[j] = fr[j] + (st.gz ? zr - wr : zr + wr);
          fi[j] = fi[j] + (st.gz ? zi - wi : zi + wi);
        }
        adj_apply_g(a[t], a[t1], m[j], st.form);
        adj_apply_g(l[t], l[t1], m[j], st.form);
      }
    }
    if constexpr (std::is_same<R, float>::value) {
      // complex64: the group's float sums into the double accumulators
#pragma unroll
      for (int j = 0; j < K; ++j) {
        accr[j] += (double)fr[j];
        acci[j] += (double)fi[j];
        fr[j] = fi[j] = 0.0f;
      }
    }
#pragma unroll
    for (int t = 0; t < G; ++t) {
      uint64_t idx = base;
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (t >> j & 1) idx |= 1ULL << S.s[j].q;
      psi[idx] = a[t];
      lam[idx] = l[t];
    }
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (!S.s[j].inner) continue;  // the same value in every thread
    double re, im;
    if constexpr (std::is_same<R, fpair>::value) {
      re = fpair_to_double(fr[j]);
      im = fpair_to_double(fi[j]);
    } else if constexpr (std::is_same<R, double>::value) {
      re = fr[j];
      im = fi[j];
    } else {
      re = accr[j];
      im = acci[j];
    }
    const double pr = re * S.s[j].ph_re - im * S.s[j].ph_im, pi = re * S.s[j].ph_im + im * S.s[j].ph_re;
    const double r = block_sum(pr);
    if (threadIdx.x == 0) partials[(2 * j) * gridDim.x + blockIdx.x] = r;
    const double q = block_sum(pi);
    if (threadIdx.x == 0) partials[(2 * j + 1) * gridDim.x + blockIdx.x] = q;
  }
}

}  // namespace

void ham_apply(Device &dev, const void *src, void *dst, const std::vector<HamTerm> &terms) {
  const size_t bytes = sizeof(HamTermDev) * terms.size();
  grow(dev.aux2, dev.aux2_cap, bytes);
  std::vector<HamTermDev> h(terms.size());
  for (size_t i = 0; i < terms.size(); ++i) h[i] = HamTermDev{terms[i].x_mask, terms[i].z_mask, terms[i].re, terms[i].im};
  cuda_check(cudaMemcpyAsync(dev.aux2, h.data(), bytes, cudaMemcpyHostToDevice, dev.stream), "hamiltonian upload");
  const int grid = grid_for(dev.amps(), 256);
  if (dev.dbl)
    k_ham_apply<double2><<<grid, 256, 0, dev.stream>>>(reinterpret_cast<const double2 *>(src), reinterpret_cast<double2 *>(dst),
                                                       dev.amps(), reinterpret_cast<const HamTermDev *>(dev.aux2), (int)terms.size());
  else
    k_ham_apply<float2><<<grid, 256, 0, dev.stream>>>(reinterpret_cast<const float2 *>(src), reinterpret_cast<float2 *>(dst),
                                                      dev.amps(), reinterpret_cast<const HamTermDev *>(dev.aux2), (int)terms.size());
  check_launch("hamiltonian kernel");
}

void reduce_pauli_inner(Device &dev, const void *lam, const void *psi, uint64_t x_mask, uint64_t z_mask, cd phase,
                        int slot) {
  // slot: write the (re, im) pair at results[2*slot], [2*slot+1]
  const int blocks = kReduceBlocks;
  grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * blocks * 2);
  if (dev.dbl)
    k_pauli_inner<double2><<<blocks, kReduceThreads, 0, dev.stream>>>(
        reinterpret_cast<const double2 *>(lam), reinterpret_cast<const double2 *>(psi), dev.amps(), x_mask, z_mask,
        phase.real(), phase.imag(), dev.partials);
  else
    k_pauli_inner<float2><<<blocks, kReduceThreads, 0, dev.stream>>>(
        reinterpret_cast<const float2 *>(lam), reinterpret_cast<const float2 *>(psi), dev.amps(), x_mask, z_mask,
        phase.real(), phase.imag(), dev.partials);
  check_launch("pauli inner product kernel");
  k_finish<<<2, 256, 0, dev.stream>>>(dev.partials, blocks, 2, dev.results + 2 * slot);
  check_launch("reduction finish");
}

void adjoint_to_pairs(Device &dev, void *a) {
  k_to_pairs<<<grid_for(dev.amps(), 256), 256, 0, dev.stream>>>(reinterpret_cast<double2 *>(a), dev.amps());
  check_launch("float-pair conversion kernel");
}

void ham_apply_pairs(Device &dev, const void *src, void *dst, const std::vector<HamTerm> &terms) {
  const size_t bytes = sizeof(HamTermPair) * terms.size();
  grow(dev.aux2, dev.aux2_cap, bytes);
  std::vector<HamTermPair> h(terms.size());
  auto split = [](double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
  };
  for (size_t i = 0; i < terms.size(); ++i) {
    h[i].x_mask = terms[i].x_mask;
    h[i].z_mask = terms[i].z_mask;
    split(terms[i].re, h[i].re_hi, h[i].re_lo);
    split(terms[i].im, h[i].im_hi, h[i].im_lo);
  }
  cuda_check(cudaMemcpyAsync(dev.aux2, h.data(), bytes, cudaMemcpyHostToDevice, dev.stream), "hamiltonian upload");
  k_ham_apply_pairs<<<grid_for(dev.amps(), 256), 256, 0, dev.stream>>>(
      reinterpret_cast<const fcx *>(src), reinterpret_cast<fcx *>(dst), dev.amps(),
      reinterpret_cast<const HamTermPair *>(dev.aux2), (int)terms.size());
  check_launch("hamiltonian float-pair kernel");
}

void adjoint_from_pairs(Device &dev, void *a) {
  k_from_pairs<<<grid_for(dev.amps(), 256), 256, 0, dev.stream>>>(reinterpret_cast<double2 *>(a), dev.amps());
  check_launch("float-pair conversion kernel");
}

void adjoint_step_pairs(Device &dev, void *psi, void *lam, int q, const cd *m, int form, bool gx, bool gz, cd phase,
                        int slot, bool apply) {
  AdjMat M;
  for (int j = 0; j < 4; ++j) {
    M.re[j] = m[j].real();
    M.im[j] = m[j].imag();
  }
  const int blocks = kReduceBlocks;
  if (slot >= 0) grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * blocks * 2);
  k_adj_step_pairs<<<blocks, kReduceThreads, 0, dev.stream>>>(reinterpret_cast<fcx *>(psi), reinterpret_cast<fcx *>(lam),
                                                              dev.amps() >> 1, q, M, form, gx, gz, slot >= 0, apply,
                                                              phase.real(), phase.imag(), dev.partials);
  check_launch("adjoint float-pair step kernel");
  if (slot >= 0) {
    k_finish<<<2, 256, 0, dev.stream>>>(dev.partials, blocks, 2, dev.results + 2 * slot);
    check_launch("reduction finish");
  }
}

template <typename E, int K>
void launch_adj_steps(Device &dev, void *psi, void *lam, const std::vector<AdjStepHost> &steps) {
  AdjSteps<K> S;
  std::vector<uint64_t> qs;
  for (int j = 0; j < K; ++j) {
    const AdjStepHost &h = steps[j];
    AdjStepDev &d = S.s[j];
    d.q = h.q;
    d.form = h.form;
    d.gx = h.gx;
    d.gz = h.gz;
    d.inner = h.slot >= 0;
    for (int e = 0; e < 4; ++e) {
      d.re[e] = h.m[e].real();
      d.im[e] = h.m[e].imag();
    }
    d.ph_re = h.phase.real();
    d.ph_im = h.phase.imag();
    qs.push_back((uint64_t)h.q);
  }
  std::sort(qs.begin(), qs.end());
  for (int j = 0; j < K; ++j) S.lowmask[j] = (1ULL << qs[j]) - 1;
  const int blocks = kReduceBlocks;
  grow(reinterpret_cast<void *&>(dev.partials), dev.partials_cap, sizeof(double) * blocks * 2 * K);
  k_adj_steps<E, K><<<blocks, kReduceThreads, 0, dev.stream>>>(reinterpret_cast<E *>(psi), reinterpret_cast<E *>(lam),
                                                               dev.amps() >> K, S, dev.partials);
  check_launch("adjoint steps kernel");
  for (int j = 0; j < K; ++j)
    if (steps[j].slot >= 0) {
      k_finish<<<2, 256, 0, dev.stream>>>(dev.partials + (size_t)2 * j * blocks, blocks, 2,
                                          dev.results + 2 * steps[j].slot);
      check_launch("reduction finish");
    }
}

namespace {
// out[y] = in[src(y)] for a linear (GF(2)) map of the index bits plus a
// constant: the source index from the map's columns, one pass that reads
// and writes each element once (a run of CX / X / SWAP gates is otherwise
// one pass per gate)
struct LinearGather {
  int nq;
  int q[64];
  uint64_t d[64];
  uint64_t c;
};
// The source index through per-byte tables in shared memory: tab[b][v] = the
// xor of d[k] over the map's qubits in byte b of the index whose bit is set
// in v, so that src = y ^ c ^ tab[0][y & 255] ^ tab[1][(y >> 8) & 255] ^ ...
constexpr int kGatherBytes = 5;  // indices below 2^40
template <typename E>
__global__ void __launch_bounds__(256) k_gather_linear(const E *__restrict__ in, E *__restrict__ out, uint64_t count,
                                                       const __grid_constant__ LinearGather G) {
  __shared__ uint64_t tab[kGatherBytes][256];
  for (int e = threadIdx.x; e < kGatherBytes * 256; e += blockDim.x) {
    const int b = e >> 8, v = e & 255;
    uint64_t x = 0;
    for (int k = 0; k < G.nq; ++k)
      if ((G.q[k] >> 3) == b && ((v >> (G.q[k] & 7)) & 1)) x ^= G.d[k];
    tab[b][v] = x;
  }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; y < count; y += stride) {
    uint64_t src = y ^ G.c;
#pragma unroll
    for (int b = 0; b < kGatherBytes; ++b) src ^= tab[b][(y >> (8 * b)) & 255];
    out[y] = in[src];
  }
}
}  // namespace

void gather_linear(Device &dev, const void *in, void *out, const LinearGatherHost &g) {
  LinearGather G;
  std::memset(&G, 0, sizeof(G));
  if (g.q.size() > 64 || g.q.size() != g.d.size()) throw Error(1, "linear gather: bad map");
  for (int q : g.q)
    if (q < 0 || q >= 8 * kGatherBytes) throw Error(1, "linear gather: qubit beyond the tables");
  G.nq = (int)g.q.size();
  for (int k = 0; k < G.nq; ++k) {
    G.q[k] = g.q[k];
    G.d[k] = g.d[k];
  }
  G.c = g.c;
  const uint64_t count = dev.amps();
  const unsigned grid = (unsigned)std::min<uint64_t>((count + 255) / 256, (uint64_t)sm_count() * 16);
  if (dev.amp_bytes() == 16)
    k_gather_linear<uint4><<<grid, 256, 0, dev.stream>>>(static_cast<const uint4 *>(in), static_cast<uint4 *>(out),
                                                         count, G);
  else
    k_gather_linear<uint2><<<grid, 256, 0, dev.stream>>>(static_cast<const uint2 *>(in), static_cast<uint2 *>(out),
                                                         count, G);
  check_launch("linear gather");
}

void adjoint_steps(Device &dev, void *psi, void *lam, const std::vector<AdjStepHost> &steps, bool pairs) {
  const int K = (int)steps.size();
  if (K < 1 || K > 3) throw Error(1, "adjoint steps: 1 to 3 per pass");
  auto run = [&](auto tag) {
    using E = decltype(tag);
    if (K == 1) launch_adj_steps<E, 1>(dev, psi, lam, steps);
    else if (K == 2) launch_adj_steps<E, 2>(dev, psi, lam, steps);
    else launch_adj_steps<E, 3>(dev, psi, lam, steps);
  };
  if (pairs)
    run(fcx{});
  else if (dev.dbl)
    run(double2{});
  else
    run(float2{});
}

// ============================ cache-blocked runs ============================
// A run is a sequence of dense (k <= 5) / diagonal ops whose qubits all lie in
// one tile of kRunTileBits vector qubits.  A persistent CTA loads a tile
// (the kRunLowBits lowest qubits are always part of it, so a tile is
// 2^(m - c) contiguous segments of 2^c amplitudes: coalesced 16-byte loads),
// applies every op of the run in shared memory, and writes the tile back:
// one HBM read + write for the whole run instead of one per op.
namespace {

constexpr int kRunMaxOps = 24;

struct RunOpDev {
  int kind;                 // 0 dense, 1 diagonal, 2 multi-controlled X
  int k;
  int bound;                // 1: the matrix is in the per-binding block of the tile's state
  int mat_off;              // offset into the matrix pool / per-binding block (complex entries)
  uint32_t lowmask[5];      // sorted local positions as masks, for zero insertion
  uint32_t offs[32];        // local offset of matrix index a
  uint32_t qbit[5];         // local bit of op qubit j (diagonal index)
};

struct RunParams {
  int m, c, nops, pool_elems;
  int bound_elems;          // complex entries per binding in the per-binding pool (0: none)
  int state_bits;           // bound runs: log2 of the amplitudes per state of the stack
  uint64_t nbind;           // bound runs: states of the stack that hold a binding
  uint64_t ntiles;
  uint64_t tile_lowmask[kMaxQubits];  // sorted tile qubits (zero insertion of the tile id)
  int nt;                             // number of tile qubits = m
  int T[24];                          // T[j]: global qubit of local bit j
  RunOpDev ops[kRunMaxOps];
};

__device__ __forceinline__ uint32_t ins32(uint32_t i, const uint32_t *lowmask, int k) {
  for (int j = 0; j < k; ++j) {
    const uint32_t msk = lowmask[j];
    i = ((i & ~msk) << 1) | (i & msk);
  }
  return i;
}

template <typename T, int K>
__device__ __forceinline__ void run_dense(T *tile, const T *mat, const RunOpDev &op, int m) {
  constexpr int D = 1 << K;
  const uint32_t G = 1u << (m - K);
  for (uint32_t g = threadIdx.x; g < G; g += blockDim.x) {
    const uint32_t base = ins32(g, op.lowmask, K);
    T v[D];
#pragma unroll
    for (int a = 0; a < D; ++a) v[a] = tile[base + op.offs[a]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      T acc;
      acc.x = 0;
      acc.y = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) cfma(acc, mat[r + D * c], v[c]);
      tile[base + op.offs[r]] = acc;
    }
  }
}

template <typename T>
__device__ __forceinline__ void run_diag(T *tile, const T *diag, const RunOpDev &op, int m) {
  const uint32_t L = 1u << m;
  for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) {
    uint32_t iv = 0;
    for (int j = 0; j < op.k; ++j) iv |= ((l & op.qbit[j]) != 0) << j;
    const T d = diag[iv];
    if (!is_one(d)) tile[l] = cmul(tile[l], d);
  }
}

// Multi-controlled X inside a tile: swap the pairs that differ in the target
// bit and have every control bit set (QubitVector::apply_mcx,
// qubitvector.hpp:1446-1486); no arithmetic.
template <typename T>
__device__ __forceinline__ void run_mcx(T *tile, const RunOpDev &op, int m) {
  const uint32_t tb = op.qbit[op.k - 1], low = tb - 1;
  uint32_t cm = 0;
  for (int j = 0; j + 1 < op.k; ++j) cm |= op.qbit[j];
  const uint32_t half = 1u << (m - 1);
  for (uint32_t p = threadIdx.x; p < half; p += blockDim.x) {
    const uint32_t i0 = ((p & ~low) << 1) | (p & low);
    if ((i0 & cm) == cm) {
      const T a = tile[i0];
      tile[i0] = tile[i0 | tb];
      tile[i0 | tb] = a;
    }
  }
}

// bpool (bound runs only): bound_elems complex entries per binding, binding
// j of the stack at bpool + j * bound_elems.
template <typename T>
__global__ void __launch_bounds__(256, 2) k_run(T *__restrict__ psi, const RunParams *__restrict__ P,
                                             const T *__restrict__ pool, const T *__restrict__ bpool) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = P->m, c = P->c;
  T *tile = reinterpret_cast<T *>(smem_raw);
  T *mats = tile + (1u << m);
  T *bmats = mats + P->pool_elems;
  uint64_t *hi = reinterpret_cast<uint64_t *>(bmats + P->bound_elems);
  for (int i = threadIdx.x; i < P->pool_elems; i += blockDim.x) mats[i] = pool[i];
  const uint32_t nhi = 1u << (m - c);
  for (uint32_t h = threadIdx.x; h < nhi; h += blockDim.x) {
    uint64_t a = 0;
    for (int j = c; j < m; ++j)
      if ((h >> (j - c)) & 1) a |= 1ULL << P->T[j];
    hi[h] = a;
  }
  __syncthreads();
  const uint32_t L = 1u << m, cmask = (1u << c) - 1;
  for (uint64_t t = blockIdx.x; t < P->ntiles; t += gridDim.x) {
    const uint64_t gbase = insert_zeros(t, P->tile_lowmask, P->nt);
    if (P->bound_elems) {
      // the tile lies inside one state of the stack (no tile qubit reaches
      // state_bits): its binding's matrices, or nothing for a padding state
      const uint64_t st = gbase >> P->state_bits;
      if (st >= P->nbind) continue;  // same value in every thread of the CTA
      const T *src = bpool + st * (uint64_t)P->bound_elems;
      for (int i = threadIdx.x; i < P->bound_elems; i += blockDim.x) bmats[i] = src[i];
    }
    for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) tile[l] = psi[gbase | hi[l >> c] | (l & cmask)];
    __syncthreads();
    for (int o = 0; o < P->nops; ++o) {
      const RunOpDev &op = P->ops[o];
      const T *mat = (op.bound ? bmats : mats) + op.mat_off;
      if (op.kind == 1) {
        run_diag(tile, mat, op, m);
      } else if (op.kind == 2) {
        run_mcx(tile, op, m);
      } else {
        switch (op.k) {
          case 1: run_dense<T, 1>(tile, mat, op, m); break;
          case 2: run_dense<T, 2>(tile, mat, op, m); break;
          case 3: run_dense<T, 3>(tile, mat, op, m); break;
          case 4: run_dense<T, 4>(tile, mat, op, m); break;
          case 5: run_dense<T, 5>(tile, mat, op, m); break;
        }
      }
      __syncthreads();
    }
    for (uint32_t l = threadIdx.x; l < L; l += blockDim.x) psi[gbase | hi[l >> c] | (l & cmask)] = tile[l];
    __syncthreads();
  }
}

int run_tile_bits(const Device &dev) { return dev.run_tile_bits ? dev.run_tile_bits : dev.dbl ? 12 : 13; }
constexpr int kRunLowBits = 4;
constexpr int kRunPoolBytes = 32 * 1024;

constexpr int kRunBoundBytes = 16 * 1024;

template <typename T>
void launch_run_t(Device &dev, const std::vector<const RunOp *> &ops, const RunBound *bound) {
  const int n = dev.n;
  // a bound run's tiles stay inside one state of the stack
  const int m = std::min(run_tile_bits(dev), bound ? bound->state_bits : n);
  // tile qubits: the low c qubits, the ops' qubits, then padding from the bottom
  std::vector<bool> in(n, false);
  const int c = std::min(kRunLowBits, m);
  for (int q = 0; q < c; ++q) in[q] = true;
  for (auto *op : ops)
    for (auto q : op->qubits) in[q] = true;
  int cnt = 0;
  for (int q = 0; q < n; ++q) cnt += in[q];
  if (cnt > m) throw Error(1, "run does not fit in a tile");
  for (int q = 0; q < n && cnt < m; ++q)
    if (!in[q]) { in[q] = true; ++cnt; }
  auto P = std::make_unique<RunParams>();
  std::memset(P.get(), 0, sizeof(RunParams));
  std::vector<int> tq, local(n, -1);
  for (int q = 0; q < n; ++q)
    if (in[q]) { local[q] = (int)tq.size(); tq.push_back(q); }
  // cc = length of the contiguous low prefix of the tile qubits
  int cc = 0;
  while (cc < m && tq[cc] == cc) ++cc;
  if (dev.blocking != 2 && launch_run_reg(dev, ops, tq, cc, bound)) return;
  P->m = m;
  P->c = cc;
  P->nt = m;
  for (int j = 0; j < m; ++j) { P->T[j] = tq[j]; P->tile_lowmask[j] = (1ULL << tq[j]) - 1; }
  P->ntiles = 1ULL << (n - m);
  if ((int)ops.size() > kRunMaxOps) throw Error(1, "run too long");
  std::vector<T> pool;
  int bound_elems = 0;
  for (size_t o = 0; o < ops.size(); ++o) {
    const RunOp &op = *ops[o];
    RunOpDev &d = P->ops[o];
    d.kind = op.kind;
    d.k = (int)op.qubits.size();
    d.bound = !op.bmat.empty();
    if (d.bound && !bound) throw Error(1, "bound run op outside a bound run");
    d.mat_off = d.bound ? bound_elems : (int)pool.size();
    reg_t lq;
    for (auto q : op.qubits) lq.push_back(local[q]);
    reg_t sq = lq;
    std::sort(sq.begin(), sq.end());
    for (int j = 0; j < d.k; ++j) { d.lowmask[j] = (1u << sq[j]) - 1; d.qbit[j] = 1u << lq[j]; }
    d.offs[0] = 0;
    for (int j = 0; j < d.k; ++j) {
      const uint32_t nn = 1u << j, bit = 1u << lq[j];
      for (uint32_t a = 0; a < nn; ++a) d.offs[nn + a] = d.offs[a] | bit;
    }
    if (d.bound)
      bound_elems += (int)op.mat.size();
    else
      for (const cd &z : op.mat) pool.push_back(to_dev<T>(z));
  }
  P->nops = (int)ops.size();
  P->pool_elems = (int)pool.size();
  P->bound_elems = bound_elems;
  if (pool.size() * sizeof(T) > (size_t)kRunPoolBytes) throw Error(1, "run matrices exceed the pool");
  if ((size_t)bound_elems * sizeof(T) > (size_t)kRunBoundBytes) throw Error(1, "run matrices exceed the bound pool");
  // per-binding matrices of the stack's states, binding-major
  std::vector<T> bpool;
  if (bound_elems) {
    P->state_bits = bound->state_bits;
    P->nbind = bound->count;
    bpool.reserve((size_t)bound_elems * bound->count);
    for (uint64_t j = 0; j < bound->count; ++j)
      for (const RunOp *op : ops) {
        if (op->bmat.empty()) continue;
        const size_t msz = op->mat.size();
        if (op->bmat.size() < (bound->first + j + 1) * msz) throw Error(1, "bound run op has too few bindings");
        const cd *src = op->bmat.data() + (bound->first + j) * msz;
        for (size_t e = 0; e < msz; ++e) bpool.push_back(to_dev<T>(src[e]));
      }
  }
  const size_t pbytes = sizeof(RunParams), poolb = pool.size() * sizeof(T), bpoolb = bpool.size() * sizeof(T);
  const size_t pool_off = (pbytes + 255) & ~size_t(255);
  const size_t bpool_off = (pool_off + poolb + 255) & ~size_t(255);
  grow(dev.mat, dev.mat_cap, bpool_off + bpoolb + 256);
  char *base = reinterpret_cast<char *>(dev.mat);
  cuda_check(cudaMemcpyAsync(base, P.get(), pbytes, cudaMemcpyHostToDevice, dev.stream), "run upload");
  if (poolb)
    cuda_check(cudaMemcpyAsync(base + pool_off, pool.data(), poolb, cudaMemcpyHostToDevice, dev.stream), "run upload");
  if (bpoolb)
    cuda_check(cudaMemcpyAsync(base + bpool_off, bpool.data(), bpoolb, cudaMemcpyHostToDevice, dev.stream),
               "run upload");
  const size_t smem =
      sizeof(T) * ((1u << m) + pool.size() + (size_t)bound_elems) + sizeof(uint64_t) * (1u << (m - cc));
  static bool attr_set[2] = {false, false};
  if (!attr_set[dev.dbl]) {
    cuda_check(cudaFuncSetAttribute(k_run<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
               "run kernel attribute");
    attr_set[dev.dbl] = true;
  }
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run<T>, 256, smem), "occupancy");
  per_sm = std::max(per_sm, 1);
  const uint64_t grid = std::min<uint64_t>(P->ntiles, 152ULL * per_sm);
  k_run<T><<<(unsigned)grid, 256, smem, dev.stream>>>(reinterpret_cast<T *>(dev.state),
                                                     reinterpret_cast<const RunParams *>(base),
                                                     reinterpret_cast<const T *>(base + pool_off),
                                                     reinterpret_cast<const T *>(base + bpool_off));
  check_launch("run kernel");
}

}  // namespace

int run_tile_qubits(const Device &dev) { return std::min(run_tile_bits(dev), dev.n); }
int run_low_qubits(const Device &dev) { return std::min(kRunLowBits, dev.n); }
size_t run_pool_bytes(const Device &dev) { return kRunPoolBytes / dev.amp_bytes() * 16; }
int run_max_ops() { return kRunMaxOps; }

size_t run_bound_pool_bytes(const Device &dev) { return kRunBoundBytes / dev.amp_bytes() * 16; }

void launch_run(Device &dev, const std::vector<const RunOp *> &ops, const RunBound *bound) {
  if (dev.dbl)
    launch_run_t<double2>(dev, ops, bound);
  else
    launch_run_t<float2>(dev, ops, bound);
}

}  // namespace gbqv
