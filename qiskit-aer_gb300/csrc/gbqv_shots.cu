// Batched shots for circuits that cannot be measure-sampled: a group of
// shots is a stack of 2^b states of sb qubits (state s at amplitudes
// [s 2^sb, (s + 1) 2^sb)), each starting from |0...0> and carrying its own
// classical memory and RNG stream on the host.  The reference runs such shots
// one state per chunk with a per-outcome loop of probability sums and
// conditional register writes on the device
// (QubitVectorThrust::apply_batched_measure / apply_batched_reset,
// qubitvector_thrust.hpp:2251-2448; conditional gates through
// set_batched_system_conditional, :2568).  Here one pass gives every state's
// marginal probabilities of the measured qubits (all outcomes at once), the
// host draws each shot's outcome from its own stream, and one pass collapses
// every state; a classically conditioned gate is applied to the states whose
// condition holds by a kernel that reads a per-state mask.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "gbqv_internal.h"

namespace gbqv {
namespace {

constexpr int kMaxSegK = 5;      // measured qubits summed in registers (more: one thread per outcome)
constexpr int kMaxSegMatK = 4;   // qubits of a conditioned matrix

// Positions of the k op qubits inside a state: offs[v] = the amplitude
// offset of outcome v (bit j of v on qubits[j]); lowmask = masks below the
// sorted qubits, for inserting zero bits into a group index.
struct SegQ {
  uint64_t offs[1 << kMaxSegK];
  uint64_t lowmask[kMaxSegK];
};

template <int K>
__device__ __forceinline__ uint64_t spread_zeros(uint64_t i, const uint64_t *lowmask) {
#pragma unroll
  for (int j = 0; j < K; ++j) i = ((i & ~lowmask[j]) << 1) | (i & lowmask[j]);
  return i;
}

__device__ __forceinline__ double seg_block_sum(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // red[] may still be read by the previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  v = 0.0;
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// Marginal probabilities of K qubits per state (QubitVector::probabilities
// (qubits), qubitvector.hpp:2089-2143, once per state): grid (bps, states),
// slice blockIdx.x of state seg0 + blockIdx.y; partials[(state D + v) bps + slice].
template <typename T, int K>
__global__ void __launch_bounds__(256) k_probs_seg(const T *__restrict__ psi, int sb, int bps, uint64_t seg0, SegQ q,
                                                   double *__restrict__ partials) {
  constexpr int D = 1 << K;
  const uint64_t seg = seg0 + blockIdx.y;
  const T *ps = psi + (seg << sb);
  const uint64_t ngroups = 1ULL << (sb - K);
  double acc[D];
#pragma unroll
  for (int v = 0; v < D; ++v) acc[v] = 0.0;
  const uint64_t stride = (uint64_t)bps * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
    const uint64_t base = spread_zeros<K>(g, q.lowmask);
#pragma unroll
    for (int v = 0; v < D; ++v) {
      const T a = ps[base + q.offs[v]];
      acc[v] += (double)(a.x * a.x + a.y * a.y);
    }
  }
#pragma unroll
  for (int v = 0; v < D; ++v) {
    const double s = seg_block_sum(acc[v]);
    if (threadIdx.x == 0) partials[(seg * D + v) * bps + blockIdx.x] = s;
  }
}

__global__ void k_sum_slices(const double *__restrict__ partials, int bps, uint64_t nvalues, double *__restrict__ out) {
  const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvalues) return;
  double s = 0.0;
  for (int b = 0; b < bps; ++b) s += partials[v * bps + b];
  out[v] = s;
}

// Any number of op qubits (up to a whole state): qubit j of the op at bit
// q[j] of the amplitude index, lowmask for the sorted positions.
struct SegQW {
  uint32_t q[32];
  uint64_t lowmask[32];
  uint64_t qmask;  // OR of the op qubits' bits
  int k;
};

__device__ __forceinline__ uint64_t deposit(uint64_t v, const SegQW &w) {
  uint64_t r = 0;
  for (int j = 0; j < w.k; ++j) r |= ((v >> j) & 1ULL) << w.q[j];
  return r;
}

__device__ __forceinline__ uint64_t gather(uint64_t i, const SegQW &w) {
  uint64_t v = 0;
  for (int j = 0; j < w.k; ++j) v |= ((i >> w.q[j]) & 1ULL) << j;
  return v;
}

// Marginal probabilities of k > 5 qubits per state: one thread per outcome
// (grid.x = outcome chunks of 256 x bps slices), each summing its outcome's
// groups in order; partials laid out as in k_probs_seg.
template <typename T>
__global__ void __launch_bounds__(256) k_probs_seg_wide(const T *__restrict__ psi, int sb, int bps, uint64_t seg0,
                                                        SegQW w, double *__restrict__ partials) {
  const uint64_t D = 1ULL << w.k;
  const uint64_t v = (uint64_t)(blockIdx.x / bps) * blockDim.x + threadIdx.x;
  const uint32_t slice = blockIdx.x % bps;
  const uint64_t seg = seg0 + blockIdx.y;
  if (v >= D) return;
  const T *ps = psi + (seg << sb);
  const uint64_t off = deposit(v, w), ngroups = 1ULL << (sb - w.k);
  double acc = 0.0;
  for (uint64_t g = slice; g < ngroups; g += bps) {
    uint64_t base = g;
    for (int j = 0; j < w.k; ++j) base = ((base & ~w.lowmask[j]) << 1) | (base & w.lowmask[j]);
    const T a = ps[base | off];
    acc += (double)(a.x * a.x + a.y * a.y);
  }
  partials[(seg * D + v) * bps + slice] = acc;
}

// State::measure_reset_update (statevector_state.hpp:936-1011) per state:
// the amplitude of outcome meas[s], times scale[s] (1/sqrt(p)), moves to
// outcome fin[s] (meas for a measurement, 0 for a reset); every other
// outcome becomes 0.  One thread per amplitude; the thread of outcome fin
// also clears the source amplitude, so each amplitude has one writer (the
// pairing of the reference's reset_func, qubitvector_thrust.hpp:2333-2383).
// meas[s] = ~0u leaves state s as it is (a padding state, or a shot whose
// condition does not hold).
template <typename T>
__global__ void __launch_bounds__(256) k_collapse_seg(T *__restrict__ psi, int sb, uint64_t total, SegQW w,
                                                      const uint32_t *__restrict__ meas,
                                                      const uint32_t *__restrict__ fin,
                                                      const double *__restrict__ scale) {
  using R = decltype(T::x);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t low = (1ULL << sb) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const uint64_t seg = i >> sb;
    const uint32_t m = meas[seg];
    if (m == 0xffffffffu) continue;
    const uint32_t f = fin[seg];
    const uint64_t v = gather(i & low, w);
    if (v == f) {
      const uint64_t src = (i & ~w.qmask) | deposit(m, w);
      const R s = (R)scale[seg];
      T a = psi[src];
      a.x *= s;
      a.y *= s;
      psi[i] = a;
      if (m != f) {
        T z;
        z.x = 0;
        z.y = 0;
        psi[src] = z;
      }
    } else if (v != m) {
      T z;
      z.x = 0;
      z.y = 0;
      psi[i] = z;
    }
  }
}

// RngEngine::rand_int(probs) (rng.hpp:94-96, std::discrete_distribution)
// on the device for wide registers: per state (one CTA of 1024 threads),
// total = sum of the 2^k outcome probabilities, then the normalised
// cumulative sum chunk by chunk (block scans of 1024 outcomes), the last
// entry set to 1, and the first outcome whose cumulative value reaches the
// uniform.  Parallel sums round differently from the sequential ones, so an
// outcome can differ only when the uniform lies within a few ulps of a
// cumulative boundary.  u[s] < 0: no draw (out[s] = ~0u).  D >= 1024, a
// multiple of 1024.
__global__ void __launch_bounds__(1024) k_draw_seg(const double *__restrict__ probs, uint64_t D,
                                                   const double *__restrict__ u, uint32_t *__restrict__ out,
                                                   double *__restrict__ pout) {
  __shared__ double wsum[32];
  __shared__ int first;
  const uint64_t seg = blockIdx.x;
  const double r = u[seg];
  if (r < 0.0) {
    if (threadIdx.x == 0) {
      out[seg] = 0xffffffffu;
      pout[seg] = 0.0;
    }
    return;
  }
  const double *p = probs + seg * D;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double t = 0.0;
  for (uint64_t i = threadIdx.x; i < D; i += blockDim.x) t += p[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) wsum[warp] = t;
  __syncthreads();
  double total = 0.0;
  for (int w = 0; w < 32; ++w) total += wsum[w];
  __syncthreads();
  double running = 0.0;
  for (uint64_t c0 = 0; c0 < D; c0 += 1024) {
    const uint64_t i = c0 + threadIdx.x;
    double x = p[i] / total;
    // inclusive scan: within the warp, then over the warp totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    if (threadIdx.x == 0) first = 0x7fffffff;
    __syncthreads();
    double before = 0.0, chunk = 0.0;
    for (int w = 0; w < 32; ++w) {
      if (w < warp) before += wsum[w];
      chunk += wsum[w];
    }
    double cp = running + before + x;
    if (i == D - 1) cp = 1.0;
    if (cp >= r) atomicMin(&first, (int)threadIdx.x);
    __syncthreads();
    const int f = first;
    if (f != 0x7fffffff) {
      if ((int)threadIdx.x == f) {
        out[seg] = (uint32_t)i;
        pout[seg] = p[i];
      }
      return;
    }
    running += chunk;
    __syncthreads();  // wsum and first are rewritten by the next chunk
  }
}

// A K-qubit matrix (column-major, as QubitVector::apply_matrix) applied to
// the states whose mask byte is set.
template <typename T, int K>
__global__ void __launch_bounds__(256) k_matrix_seg(T *__restrict__ psi, int sb, uint64_t total, SegQ q,
                                                    const double2 *__restrict__ mat,
                                                    const uint8_t *__restrict__ mask) {
  using R = decltype(T::x);
  constexpr int D = 1 << K;
  __shared__ T m[D * D];
  for (int i = threadIdx.x; i < D * D; i += blockDim.x) {
    T z;
    z.x = (R)mat[i].x;
    z.y = (R)mat[i].y;
    m[i] = z;
  }
  __syncthreads();
  const int gb = sb - K;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t G = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; G < total; G += stride) {
    const uint64_t seg = G >> gb;
    if (!mask[seg]) continue;
    T *ps = psi + (seg << sb);
    const uint64_t base = spread_zeros<K>(G & ((1ULL << gb) - 1), q.lowmask);
    T x[D];
#pragma unroll
    for (int c = 0; c < D; ++c) x[c] = ps[base + q.offs[c]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      T y;
      y.x = 0;
      y.y = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const T w = m[r + D * c];
        y.x = fma(w.x, x[c].x, y.x);
        y.x = fma(-w.y, x[c].y, y.x);
        y.y = fma(w.x, x[c].y, y.y);
        y.y = fma(w.y, x[c].x, y.y);
      }
      ps[base + q.offs[r]] = y;
    }
  }
}

// Reduced density matrix of K qubits per state, rho[a][b] = sum over the
// other qubits of x_a conj(x_b): every Kraus operator's probability
// ||K psi||^2 = tr(K^dag K rho) then follows on the host from one pass over
// the stack, where State::apply_kraus (statevector_state.hpp:1112-1156)
// takes one QubitVector::norm(qubits, mat) pass (qubitvector.hpp:1878-2082)
// per operator.  Value e of a state: e = a D + a holds rho[a][a]; for a < b,
// e = a D + b the real and e = b D + a the imaginary part of rho[a][b].
// Grid and partials as k_probs_seg, D^2 values per state.
template <typename T, int K>
__global__ void __launch_bounds__(256) k_rdm_seg(const T *__restrict__ psi, int sb, int bps, uint64_t seg0, SegQ q,
                                                 double *__restrict__ partials) {
  constexpr int D = 1 << K, E = D * D;
  const uint64_t seg = seg0 + blockIdx.y;
  const T *ps = psi + (seg << sb);
  const uint64_t ngroups = 1ULL << (sb - K);
  double acc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) acc[e] = 0.0;
  const uint64_t stride = (uint64_t)bps * blockDim.x;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
    const uint64_t base = spread_zeros<K>(g, q.lowmask);
    double xr[D], xi[D];
#pragma unroll
    for (int v = 0; v < D; ++v) {
      const T a = ps[base + q.offs[v]];
      xr[v] = (double)a.x;
      xi[v] = (double)a.y;
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      acc[a * D + a] += xr[a] * xr[a] + xi[a] * xi[a];
#pragma unroll
      for (int b = a + 1; b < D; ++b) {
        acc[a * D + b] += xr[a] * xr[b] + xi[a] * xi[b];
        acc[b * D + a] += xi[a] * xr[b] - xr[a] * xi[b];
      }
    }
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const double s = seg_block_sum(acc[e]);
    if (threadIdx.x == 0) partials[(seg * E + e) * bps + blockIdx.x] = s;
  }
}

// The Kraus operator State::apply_kraus chose for each selected state,
// normalised: state sel[i] gets the column-major matrix smats[i] (the chosen
// operator with every entry already times 1/sqrt(p), as the reference
// scales it before applying it), in the state's precision.  Only the
// selected states are visited.
template <typename T, int K>
__global__ void __launch_bounds__(256) k_kraus_seg(T *__restrict__ psi, int sb, uint64_t total, SegQ q,
                                                   const T *__restrict__ smats,
                                                   const uint32_t *__restrict__ sel) {
  constexpr int D = 1 << K;
  const int gb = sb - K;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t G = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; G < total; G += stride) {
    const uint64_t i = G >> gb;
    const T *m = smats + i * (D * D);
    T *ps = psi + ((uint64_t)sel[i] << sb);
    const uint64_t base = spread_zeros<K>(G & ((1ULL << gb) - 1), q.lowmask);
    T x[D];
#pragma unroll
    for (int c = 0; c < D; ++c) x[c] = ps[base + q.offs[c]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      T y;
      y.x = 0;
      y.y = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const T w = m[r + D * c];
        const auto wx = w.x, wy = w.y;
        y.x = fma(wx, x[c].x, y.x);
        y.x = fma(-wy, x[c].y, y.x);
        y.y = fma(wx, x[c].y, y.y);
        y.y = fma(wy, x[c].x, y.y);
      }
      ps[base + q.offs[r]] = y;
    }
  }
}

SegQ make_segq(const reg_t &qubits) {
  SegQ q{};
  local_offsets(qubits, q.offs);
  sorted_masks(qubits, q.lowmask);
  return q;
}

SegQW make_segqw(const reg_t &qubits) {
  SegQW w{};
  w.k = (int)qubits.size();
  for (int j = 0; j < w.k; ++j) {
    w.q[j] = (uint32_t)qubits[j];
    w.qmask |= 1ULL << qubits[j];
  }
  sorted_masks(qubits, w.lowmask);
  return w;
}

template <typename T> T *st(Device &d) { return reinterpret_cast<T *>(d.state); }

int grid_of(uint64_t work) {
  const uint64_t cap = (uint64_t)sm_count() * 8;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(cap, (work + 255) / 256));
}

template <typename T, int K>
void probs_k(Device &d, int sb, uint64_t nseg, const SegQ &q, int bps) {
  for (uint64_t s0 = 0; s0 < nseg; s0 += 65535) {
    dim3 grid((unsigned)bps, (unsigned)std::min<uint64_t>(65535, nseg - s0));
    k_probs_seg<T, K><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, bps, s0, q, d.partials);
  }
}

template <typename T>
void probs_any(Device &d, int sb, uint64_t nseg, const SegQ &q, int k, int bps) {
  switch (k) {
    case 1: probs_k<T, 1>(d, sb, nseg, q, bps); break;
    case 2: probs_k<T, 2>(d, sb, nseg, q, bps); break;
    case 3: probs_k<T, 3>(d, sb, nseg, q, bps); break;
    case 4: probs_k<T, 4>(d, sb, nseg, q, bps); break;
    default: probs_k<T, 5>(d, sb, nseg, q, bps); break;
  }
}

template <typename T>
void matrix_any(Device &d, int sb, uint64_t nseg, const SegQ &q, int k, const double2 *mat, const uint8_t *mask) {
  const uint64_t total = nseg << (sb - k);
  const int grid = grid_of(total);
  switch (k) {
    case 1: k_matrix_seg<T, 1><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, mat, mask); break;
    case 2: k_matrix_seg<T, 2><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, mat, mask); break;
    case 3: k_matrix_seg<T, 3><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, mat, mask); break;
    default: k_matrix_seg<T, 4><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, mat, mask); break;
  }
}

template <typename T, int K>
void rdm_k(Device &d, int sb, uint64_t nseg, const SegQ &q, int bps) {
  for (uint64_t s0 = 0; s0 < nseg; s0 += 65535) {
    dim3 grid((unsigned)bps, (unsigned)std::min<uint64_t>(65535, nseg - s0));
    k_rdm_seg<T, K><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, bps, s0, q, d.partials);
  }
}

template <typename T>
void rdm_any(Device &d, int sb, uint64_t nseg, const SegQ &q, int k, int bps) {
  switch (k) {
    case 1: rdm_k<T, 1>(d, sb, nseg, q, bps); break;
    case 2: rdm_k<T, 2>(d, sb, nseg, q, bps); break;
    default: rdm_k<T, 3>(d, sb, nseg, q, bps); break;
  }
}

template <typename T>
void kraus_any(Device &d, int sb, uint64_t nsel, const SegQ &q, int k, const T *smats, const uint32_t *sel) {
  const uint64_t total = nsel << (sb - k);
  const int grid = grid_of(total);
  switch (k) {
    case 1: k_kraus_seg<T, 1><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, smats, sel); break;
    case 2: k_kraus_seg<T, 2><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, smats, sel); break;
    default: k_kraus_seg<T, 3><<<grid, 256, 0, d.stream>>>(st<T>(d), sb, total, q, smats, sel); break;
  }
}

}  // namespace

int seg_max_measure_qubits() { return 30; }
int seg_max_matrix_qubits() { return kMaxSegMatK; }
int seg_max_kraus_qubits() { return 3; }

void reduce_rdm_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg) {
  const int k = (int)qubits.size();
  if (k < 1 || k > seg_max_kraus_qubits() || k > sb) throw Error(1, "segment density matrices: 1..3 qubits");
  const uint64_t nvalues = nseg << (2 * k);
  const SegQ q = make_segq(qubits);
  // slices per state as for the probabilities: ~8 CTAs per SM, >= 2 groups per thread
  const uint64_t want = std::max<uint64_t>(1, (uint64_t)sm_count() * 8 / nseg);
  const uint64_t cap = std::max<uint64_t>(1, (1ULL << (sb - k)) / 512);
  const int bps = (int)std::min<uint64_t>(std::min(want, cap), 256);
  grow(reinterpret_cast<void *&>(d.partials), d.partials_cap, sizeof(double) * nvalues * bps);
  grow(reinterpret_cast<void *&>(d.results), d.results_cap, sizeof(double) * nvalues);
  if (d.dbl)
    rdm_any<double2>(d, sb, nseg, q, k, bps);
  else
    rdm_any<float2>(d, sb, nseg, q, k, bps);
  check_launch("segment density matrix kernel");
  k_sum_slices<<<(unsigned)((nvalues + 255) / 256), 256, 0, d.stream>>>(d.partials, bps, nvalues, d.results);
  check_launch("segment density matrix sum");
}

void launch_kraus_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg, const cd *mats, int m,
                           const uint8_t *branch, const double *scale) {
  const int k = (int)qubits.size();
  if (k < 1 || k > seg_max_kraus_qubits() || k > sb) throw Error(1, "segment Kraus operators: 1..3 qubits");
  (void)m;
  // the states that take an operator, each with its scaled matrix
  // (std::complex times double, entry by entry, as the reference scales it)
  const size_t D2 = (size_t)1 << (2 * k);
  std::vector<uint32_t> sel;
  std::vector<cd> smats;
  for (uint64_t s = 0; s < nseg; ++s) {
    if (branch[s] == 0xff) continue;
    sel.push_back((uint32_t)s);
    const cd *src = mats + (size_t)branch[s] * D2;
    for (size_t e = 0; e < D2; ++e) smats.push_back(src[e] * scale[s]);
  }
  if (sel.empty()) return;
  // the matrices in the state's precision (a complex64 entry rounded once)
  const size_t esize = d.dbl ? sizeof(double2) : sizeof(float2);
  const size_t mbytes = smats.size() * esize;
  grow(d.aux2, d.aux2_cap, mbytes + sel.size() * 4);
  char *base = reinterpret_cast<char *>(d.aux2);
  if (d.dbl) {
    cuda_check(cudaMemcpyAsync(base, smats.data(), mbytes, cudaMemcpyHostToDevice, d.stream), "Kraus upload");
  } else {
    std::vector<float2> f(smats.size());
    for (size_t e = 0; e < f.size(); ++e) f[e] = make_float2((float)smats[e].real(), (float)smats[e].imag());
    cuda_check(cudaMemcpyAsync(base, f.data(), mbytes, cudaMemcpyHostToDevice, d.stream), "Kraus upload");
  }
  cuda_check(cudaMemcpyAsync(base + mbytes, sel.data(), sel.size() * 4, cudaMemcpyHostToDevice, d.stream),
             "Kraus upload");
  const SegQ q = make_segq(qubits);
  const uint32_t *ds = reinterpret_cast<const uint32_t *>(base + mbytes);
  if (d.dbl)
    kraus_any<double2>(d, sb, sel.size(), q, k, reinterpret_cast<const double2 *>(base), ds);
  else
    kraus_any<float2>(d, sb, sel.size(), q, k, reinterpret_cast<const float2 *>(base), ds);
  check_launch("segment Kraus kernel");
}

void reduce_probabilities_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg) {
  const int k = (int)qubits.size();
  if (k < 1 || k > sb || k > 30) throw Error(1, "segment probabilities: 1..min(state qubits, 30) qubits");
  const uint64_t nvalues = nseg << k;
  if (k <= kMaxSegK) {
    const SegQ q = make_segq(qubits);
    // slices per state: about 8 CTAs per SM over the launch, at least 2 groups per thread
    const uint64_t want = std::max<uint64_t>(1, (uint64_t)sm_count() * 8 / nseg);
    const uint64_t cap = std::max<uint64_t>(1, (1ULL << (sb - k)) / 512);
    const int bps = (int)std::min<uint64_t>(std::min(want, cap), 256);
    grow(reinterpret_cast<void *&>(d.partials), d.partials_cap, sizeof(double) * nvalues * bps);
    grow(reinterpret_cast<void *&>(d.results), d.results_cap, sizeof(double) * nvalues);
    if (d.dbl)
      probs_any<double2>(d, sb, nseg, q, k, bps);
    else
      probs_any<float2>(d, sb, nseg, q, k, bps);
    check_launch("segment probabilities kernel");
    k_sum_slices<<<(unsigned)((nvalues + 255) / 256), 256, 0, d.stream>>>(d.partials, bps, nvalues, d.results);
    check_launch("segment probabilities sum");
    return;
  }
  const SegQW w = make_segqw(qubits);
  const uint64_t chunks = ((1ULL << k) + 255) / 256;
  // slices: split a state's groups while the launch has fewer than ~8 CTAs per SM
  const uint64_t want = std::max<uint64_t>(1, (uint64_t)sm_count() * 8 / (nseg * chunks));
  const int bps = (int)std::min<uint64_t>(std::min<uint64_t>(want, 1ULL << (sb - k)), 64);
  if (chunks * bps > 0x7fffffffULL) throw Error(1, "segment probabilities: too many outcomes");
  grow(reinterpret_cast<void *&>(d.partials), d.partials_cap, sizeof(double) * nvalues * bps);
  grow(reinterpret_cast<void *&>(d.results), d.results_cap, sizeof(double) * nvalues);
  for (uint64_t s0 = 0; s0 < nseg; s0 += 65535) {
    dim3 grid((unsigned)(chunks * bps), (unsigned)std::min<uint64_t>(65535, nseg - s0));
    if (d.dbl)
      k_probs_seg_wide<double2><<<grid, 256, 0, d.stream>>>(st<double2>(d), sb, bps, s0, w, d.partials);
    else
      k_probs_seg_wide<float2><<<grid, 256, 0, d.stream>>>(st<float2>(d), sb, bps, s0, w, d.partials);
  }
  check_launch("segment probabilities kernel");
  k_sum_slices<<<(unsigned)((nvalues + 255) / 256), 256, 0, d.stream>>>(d.partials, bps, nvalues, d.results);
  check_launch("segment probabilities sum");
}

void launch_collapse_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg, const uint32_t *meas,
                              const uint32_t *fin, const double *scale) {
  const int k = (int)qubits.size();
  if (k < 1 || k > sb || k > 30) throw Error(1, "segment collapse: 1..min(state qubits, 30) qubits");
  // per-state arrays: scale (8 B), meas and fin (4 B each), 8-byte aligned
  const size_t bytes = nseg * 16;
  grow(d.aux2, d.aux2_cap, bytes);
  char *base = reinterpret_cast<char *>(d.aux2);
  cuda_check(cudaMemcpyAsync(base, scale, nseg * 8, cudaMemcpyHostToDevice, d.stream), "collapse upload");
  cuda_check(cudaMemcpyAsync(base + nseg * 8, meas, nseg * 4, cudaMemcpyHostToDevice, d.stream), "collapse upload");
  cuda_check(cudaMemcpyAsync(base + nseg * 12, fin, nseg * 4, cudaMemcpyHostToDevice, d.stream), "collapse upload");
  const SegQW w = make_segqw(qubits);
  const double *ds = reinterpret_cast<const double *>(base);
  const uint32_t *dm = reinterpret_cast<const uint32_t *>(base + nseg * 8);
  const uint32_t *df = reinterpret_cast<const uint32_t *>(base + nseg * 12);
  const uint64_t total = nseg << sb;
  const int grid = grid_of(total);
  if (d.dbl)
    k_collapse_seg<double2><<<grid, 256, 0, d.stream>>>(st<double2>(d), sb, total, w, dm, df, ds);
  else
    k_collapse_seg<float2><<<grid, 256, 0, d.stream>>>(st<float2>(d), sb, total, w, dm, df, ds);
  check_launch("segment collapse kernel");
}

void draw_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg, const double *u, uint32_t *outcome,
                   double *prob) {
  const int k = (int)qubits.size();
  if (k < 10) throw Error(1, "device draws are for registers of 10 or more qubits");
  reduce_probabilities_segments(d, qubits, sb, nseg);
  // uniforms in, outcomes and probabilities out, through the io slice of aux2
  grow(d.aux2, d.aux2_cap, nseg * 24);
  char *base = reinterpret_cast<char *>(d.aux2);
  cuda_check(cudaMemcpyAsync(base, u, nseg * 8, cudaMemcpyHostToDevice, d.stream), "uniform upload");
  double *dp = reinterpret_cast<double *>(base + nseg * 8);
  uint32_t *dout = reinterpret_cast<uint32_t *>(base + nseg * 16);
  k_draw_seg<<<(unsigned)nseg, 1024, 0, d.stream>>>(d.results, 1ULL << k, reinterpret_cast<const double *>(base),
                                                    dout, dp);
  check_launch("segment draw kernel");
  cuda_check(cudaMemcpyAsync(prob, dp, nseg * 8, cudaMemcpyDeviceToHost, d.stream), "draw copy");
  cuda_check(cudaMemcpyAsync(outcome, dout, nseg * 4, cudaMemcpyDeviceToHost, d.stream), "draw copy");
  cuda_check(cudaStreamSynchronize(d.stream), "stream synchronize");
}

void launch_matrix_segments(Device &d, const reg_t &qubits, int sb, uint64_t nseg, const cd *mat,
                            const uint8_t *mask) {
  const int k = (int)qubits.size();
  if (k < 1 || k > kMaxSegMatK || k > sb) throw Error(1, "masked segment matrices support 1..4 qubits");
  const size_t D = 1ULL << k, mbytes = D * D * 16;
  grow(d.aux2, d.aux2_cap, mbytes + nseg);
  char *base = reinterpret_cast<char *>(d.aux2);
  cuda_check(cudaMemcpyAsync(base, mat, mbytes, cudaMemcpyHostToDevice, d.stream), "matrix upload");
  cuda_check(cudaMemcpyAsync(base + mbytes, mask, nseg, cudaMemcpyHostToDevice, d.stream), "mask upload");
  const SegQ q = make_segq(qubits);
  const double2 *dmat = reinterpret_cast<const double2 *>(base);
  const uint8_t *dmask = reinterpret_cast<const uint8_t *>(base + mbytes);
  if (d.dbl)
    matrix_any<double2>(d, sb, nseg, q, k, dmat, dmask);
  else
    matrix_any<float2>(d, sb, nseg, q, k, dmat, dmask);
  check_launch("masked segment matrix kernel");
}

}  // namespace gbqv
