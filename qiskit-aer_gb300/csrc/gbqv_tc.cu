// gbqv_tc.cu — complex128 dense 4-qubit gates on the 5th-generation tensor
// cores (tcgen05.mma, TMEM accumulators), the hot op of the 30-qubit
// complex128 quantum-volume workload after Aer's fusion
// (QubitVector::apply_matrix, src/simulators/statevector/qubitvector.hpp:1419
// -> apply_lambda over 2^4-amplitude groups, qubitvector.hpp:1018-1042).
//
// FP64 runs at 1.2 TFLOP/s on GB300, so the gate is computed exactly in
// integer digit slices instead (gbqv_ozaki.h): each group's 32 reals are
// split into six signed 8-bit digits against the group's exponent, the real
// form of the matrix into six digits against each row's exponent (host), and
// the 21 digit-plane products with s + t <= 5 accumulate per level l = s + t
// in fp32 TMEM, exactly.  Levels are recombined in int64 and rounded once.
//
// One persistent CTA per SM, 17 warps, warp-specialised:
//   warps 0-7       producers: load a tile of 128 groups (two threads per
//                    group), split it into 6 fp16 digit planes in shared
//                    memory stage (tile parity);
//   warp 16 lane 0   issues 12 tcgen05.mma per tile (per state plane s, two
//                    K = 16 steps, N = 32 * (6 - s) matrix rows of planes
//                    t = 0..5-s), accumulating level s + t at TMEM column
//                    32 (s + t);
//   warps 8-11, 12-15 epilogues E0, E1: read the six level sums of their
//                    group from TMEM, recombine, store 16 amplitudes.
// Tiles alternate between two lanes of the pipeline (even tiles: smem stage
// 0, TMEM columns 0-191, E0; odd tiles: stage 1, columns 256-447, E1), so
// the split of one tile overlaps the MMAs and epilogue of the previous one.
//
// Shared-memory operands use the K-major no-swizzle layout: 8 rows x 16
// bytes core matrices, 128 bytes apart along K, 512 bytes apart per 8 rows.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "gbqv_internal.h"
#include "gbqv_ozaki.h"
#include "gbqv_tc.cuh"

namespace gbqv {
namespace {

constexpr int kTcGroups = 128;                 // groups per tile (MMA M)
constexpr int kTcReals = 32;                   // reals per group (MMA K, matrix rows)
constexpr int kPlaneBytes = kTcGroups * kTcReals * 2;   // 8 KB: one fp16 digit plane of a tile
constexpr int kStageBytes = 6 * kPlaneBytes;            // 48 KB
constexpr int kMatBytes = 6 * kTcReals * kTcReals * 2;  // 12 KB: six matrix planes
constexpr int kOffStage = kMatBytes;
constexpr int kOffKey = kOffStage + 2 * kStageBytes;
constexpr int kOffBar = kOffKey + 2 * kTcGroups * 4;
constexpr int kOffMisc = kOffBar + 16 * 8;
// + alignment slack; at least 116 KB so that a second CTA never fits on an SM
// (each CTA allocates all 512 TMEM columns)
constexpr int kTcSmemUsed = kOffMisc + 64 + 128;
constexpr int kTcSmem = kTcSmemUsed > 116 * 1024 ? kTcSmemUsed : 116 * 1024;
constexpr int kTcThreads = 17 * 32;
constexpr uint32_t kTmemCols = 512;

struct TcParams {
  uint64_t offs[16];
  uint64_t lowmask[4];
  uint64_t ngroups;
  uint64_t ntiles;
  int rowkey[kTcReals];
};

// amplitude index of group g: a zero bit inserted at each (sorted) target
__device__ __forceinline__ uint64_t insert_zeros_k4(uint64_t g, const uint64_t *lowmask) {
#pragma unroll
  for (int j = 0; j < 4; ++j) g = ((g & ~lowmask[j]) << 1) | (g & lowmask[j]);
  return g;
}

// byte offset of element (row, k) in a K-major no-swizzle operand
__host__ __device__ constexpr uint32_t core_off(uint32_t row, uint32_t k) {
  return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ double combine(const uint32_t (&T)[6][8], int i, int scale) {
  const int64_t v = oz::levels_to_i64(__uint_as_float(T[0][i]), __uint_as_float(T[1][i]), __uint_as_float(T[2][i]),
                                      __uint_as_float(T[3][i]), __uint_as_float(T[4][i]), __uint_as_float(T[5][i]));
  return oz::i64_to_double_fast(v, scale);
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_dense_tc4(double2 *psi, const __grid_constant__ TcParams p, const uint4 *__restrict__ gmat, int *status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128 - (tc::smem_u32(smem_raw) & 127)) & 127);
  int *colkey = reinterpret_cast<int *>(smem + kOffKey);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kOffBar);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kOffMisc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kOffMisc + 4);
  // barriers: full[2] (256 producer arrivals), sempty[2] (128 epilogue
  // arrivals: stage and colkey read), accf[2] (MMA commit), acce[2] (128
  // epilogue arrivals: TMEM read), done (final commit)
  const uint32_t bar0 = tc::smem_u32(bars);
  auto full = [&](int b) { return bar0 + 8u * b; };
  auto sempty = [&](int b) { return bar0 + 8u * (2 + b); };
  auto accf = [&](int b) { return bar0 + 8u * (4 + b); };
  auto acce = [&](int b) { return bar0 + 8u * (6 + b); };
  const uint32_t done = bar0 + 8u * 8;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(full(b), 2 * kTcGroups);
      tc::mbar_init(sempty(b), kTcGroups);
      tc::mbar_init(accf(b), 1);
      tc::mbar_init(acce(b), kTcGroups);
    }
    tc::mbar_init(done, 1);
    *abort_flag = 0;
    tc::mbar_init_fence();
  }
  if (warp == 16) {
    tc::tmem_alloc(tc::smem_u32(tmem_slot), kTmemCols);
    tc::tmem_relinquish();
  }
  {
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = tid; i < kMatBytes / 16; i += kTcThreads) dst[i] = gmat[i];
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint64_t ntiles = p.ntiles;
  const uint64_t stride2 = 2ULL * gridDim.x;

  if (warp < 8) {
    // ---------------- producers ----------------
    // two threads per group, in the two half-warps (h = lane / 16): half h
    // owns amplitudes 8h..8h+7, i.e. K chunks 2h, 2h+1 of the group's row
    const int m = 16 * warp + (lane & 15), h = lane >> 4;
    double2 v[8];
    auto load = [&](uint64_t t) {
      const uint64_t grp = t * kTcGroups + m;
      const bool ok = t < ntiles && grp < p.ngroups;
      const uint64_t base = ok ? insert_zeros_k4(grp, p.lowmask) : 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = ok ? psi[base + p.offs[8 * h + j]] : make_double2(0.0, 0.0);
    };
    uint64_t tile = blockIdx.x;
    load(tile);
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      int key = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) key = max(key, max(oz::exp_key(v[j].x), oz::exp_key(v[j].y)));
      key = max(key, __shfl_xor_sync(0xffffffffu, key, 16));
      const bool ok = c == 0 || tc::mbar_wait(sempty(b), (c - 1) & 1, abort_flag);
      if (!__all_sync(0xffffffffu, ok)) break;
      unsigned char *stage = smem + kOffStage + b * kStageBytes;
      const uint32_t K64 = 0x64646464u;
#pragma unroll
      for (int q2 = 0; q2 < 2; ++q2) {
        // the chunk's 8 reals (amplitudes 4q..4q+3, re/im) as signed digit words
        uint32_t lo[8], hi[8];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int64_t rb = oz::split_bsum(v[4 * q2 + jj].x, key);
          const int64_t ib = oz::split_bsum(v[4 * q2 + jj].y, key);
          lo[2 * jj] = (uint32_t)rb;
          hi[2 * jj] = (uint32_t)((uint64_t)rb >> 32);
          lo[2 * jj + 1] = (uint32_t)ib;
          hi[2 * jj + 1] = (uint32_t)((uint64_t)ib >> 32);
        }
        unsigned char *row = stage + core_off(m, 8 * (2 * h + q2));
        // digits 1..5 are byte (5 - s) of bsum plus 128: fp16 0x64xx = 1152 + d
        // after a byte permute; subtract 1152 in packed halves
        uint32_t w[4];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t g = tc::prmt(lo[2 * jj], lo[2 * jj + 1], 0x5140);
          w[jj] = tc::hadd2(tc::prmt(g, K64, 0x4140), 0xE480E480u);
        }
        *reinterpret_cast<uint4 *>(row + 5 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t g = tc::prmt(lo[2 * jj], lo[2 * jj + 1], 0x5140);
          w[jj] = tc::hadd2(tc::prmt(g, K64, 0x4342), 0xE480E480u);
        }
        *reinterpret_cast<uint4 *>(row + 4 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t g = tc::prmt(lo[2 * jj], lo[2 * jj + 1], 0x7362);
          w[jj] = tc::hadd2(tc::prmt(g, K64, 0x4140), 0xE480E480u);
        }
        *reinterpret_cast<uint4 *>(row + 3 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t g = tc::prmt(lo[2 * jj], lo[2 * jj + 1], 0x7362);
          w[jj] = tc::hadd2(tc::prmt(g, K64, 0x4342), 0xE480E480u);
        }
        *reinterpret_cast<uint4 *>(row + 2 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t g = tc::prmt(hi[2 * jj], hi[2 * jj + 1], 0x0040);
          w[jj] = tc::hadd2(tc::prmt(g, K64, 0x4140), 0xE480E480u);
        }
        *reinterpret_cast<uint4 *>(row + 1 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
        // digit 0 in [-256, 256]: fp16 bits 0x6600 + d are 1536 + d
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const uint32_t r0 = (uint32_t)(((int32_t)hi[2 * jj] >> 8) + 0x6600);
          const uint32_t i0 = (uint32_t)(((int32_t)hi[2 * jj + 1] >> 8) + 0x6600);
          w[jj] = tc::hadd2(tc::prmt(r0, i0, 0x5410), 0xE600E600u);
        }
        *reinterpret_cast<uint4 *>(row) = make_uint4(w[0], w[1], w[2], w[3]);
      }
      if (h == 0) colkey[b * kTcGroups + m] = key;
      tc::fence_async_smem();
      tc::mbar_arrive(full(b));
      load(tile + gridDim.x);
    }
  } else if (warp < 16) {
    // ---------------- epilogues ----------------
    const int b = (warp - 8) >> 2, quarter = warp & 3, m = 32 * quarter + lane;
    const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)b * 256u;
    uint64_t tile = blockIdx.x + (uint64_t)b * gridDim.x;
    for (uint32_t c = 0; tile < ntiles; tile += stride2, ++c) {
      bool ok = tc::mbar_wait(accf(b), c & 1, abort_flag);
      ok = ok && tc::mbar_wait(full(b), c & 1, abort_flag);  // producer's colkey write
      if (!__all_sync(0xffffffffu, ok)) break;
      tc::fence_after_sync();
      const int ck = colkey[b * kTcGroups + m];
      tc::mbar_arrive(sempty(b));
      const uint64_t grp = tile * kTcGroups + m;
      const bool live = grp < p.ngroups && ck != 0;
      const uint64_t base = live ? insert_zeros_k4(grp, p.lowmask) : 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t T[6][8];
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::tmem_ld8(tbase + 32u * l + 8u * q, T[l]);
        tc::tmem_wait_ld();
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::pin(T[l]);
        if (live) {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const double re = combine(T, 2 * jj, p.rowkey[8 * q + 2 * jj] + ck - 2102);
            const double im = combine(T, 2 * jj + 1, p.rowkey[8 * q + 2 * jj + 1] + ck - 2102);
            psi[base + p.offs[4 * q + jj]] = make_double2(re, im);
          }
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(acce(b));
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t mat = tc::smem_u32(smem);
    uint64_t tile = blockIdx.x;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      if (!tc::mbar_wait(full(b), c & 1, abort_flag)) break;
      if (c >= 1 && !tc::mbar_wait(acce(b), (c - 1) & 1, abort_flag)) break;
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(smem + kOffStage + b * kStageBytes);
      const uint32_t d0 = tmem + (uint32_t)b * 256u;
#pragma unroll
      for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int kk = 0; kk < 2; ++kk)
          tc::mma_f16(d0 + 32u * s, tc::smem_desc(a0 + s * kPlaneBytes + kk * 256, 128, 512),
                      tc::smem_desc(mat + kk * 256, 128, 512), tc::idesc_f16_f32(128, 32 * (6 - s)),
                      (s | kk) != 0);
      tc::mma_commit(accf(b));
    }
    // every MMA issued above has completed once `done` flips (bounded wait,
    // independent of the abort flag so TMEM is never freed under a live MMA)
    tc::mma_commit(done);
    int never = 0;
    tc::mbar_wait(done, 0, &never);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 16) tc::tmem_dealloc(tmem, kTmemCols);
  if (tid == 0 && *abort_flag) atomicExch(status, 1);
}

// Fp16 bits of a small integer (|d| <= 256).
uint16_t half_bits(int32_t d) {
  if (d == 0) return 0;
  const uint16_t sg = d < 0 ? 0x8000 : 0;
  const uint32_t a = (uint32_t)(d < 0 ? -d : d);
  int e = 31 - __builtin_clz(a);
  const uint32_t mant = (a << (10 - e)) & 0x3FF;
  return (uint16_t)(sg | ((e + 15) << 10) | mant);
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "device query");
    cuda_check(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), "device query");
  }
  return n;
}

}  // namespace

// Host: six fp16 digit planes of the real form of a 16x16 column-major
// complex matrix, rows ordered (amplitude j, re/im) -> 2j + c and columns
// likewise, in the core-matrix layout of the B operand (row = 32 t + r).
void tc_matrix4(const cd *mat, uint16_t *planes, int *rowkey) {
  constexpr int D = 16, R = 32;
  std::vector<double> A((size_t)R * R);
  for (int j = 0; j < D; ++j)
    for (int jp = 0; jp < D; ++jp) {
      const cd z = mat[j + (size_t)D * jp];
      A[(size_t)(2 * j) * R + 2 * jp] = z.real();
      A[(size_t)(2 * j) * R + 2 * jp + 1] = -z.imag();
      A[(size_t)(2 * j + 1) * R + 2 * jp] = z.imag();
      A[(size_t)(2 * j + 1) * R + 2 * jp + 1] = z.real();
    }
  std::memset(planes, 0, kMatBytes);
  for (int r = 0; r < R; ++r) {
    int key = 0;
    for (int k = 0; k < R; ++k) key = std::max(key, oz::exp_key(A[(size_t)r * R + k]));
    rowkey[r] = key;
    for (int k = 0; k < R; ++k) {
      int32_t d[6];
      oz::bsum_digits(oz::split_bsum(A[(size_t)r * R + k], key), d);
      for (int t = 0; t < 6; ++t) planes[core_off(32 * t + r, k) / 2] = half_bits(d[t]);
    }
  }
}

bool tc_dense_available(const Device &dev, int k) {
  return dev.dbl && dev.tensor_c128 == 1 && k == 4 && dev.n >= 11;
}

void launch_dense_tc(Device &dev, const reg_t &qubits, const cd *mat) {
  TcParams p;
  local_offsets(qubits, p.offs);
  sorted_masks(qubits, p.lowmask);
  p.ngroups = dev.amps() >> 4;
  p.ntiles = (p.ngroups + kTcGroups - 1) / kTcGroups;
  std::vector<uint16_t> planes(kMatBytes / 2);
  tc_matrix4(mat, planes.data(), p.rowkey);
  grow(dev.mat, dev.mat_cap, kMatBytes);
  cuda_check(cudaMemcpyAsync(dev.mat, planes.data(), kMatBytes, cudaMemcpyHostToDevice, dev.stream), "matrix upload");
  int *status = tc_status_word(dev);
  static bool attr = false;
  if (!attr) {
    cuda_check(cudaFuncSetAttribute(k_dense_tc4, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem),
               "tcgen05 kernel attribute");
    attr = true;
  }
  const uint64_t grid = std::min<uint64_t>(p.ntiles, (uint64_t)sm_count());
  k_dense_tc4<<<(unsigned)grid, kTcThreads, kTcSmem, dev.stream>>>(reinterpret_cast<double2 *>(dev.state), p,
                                                                   reinterpret_cast<const uint4 *>(dev.mat), status);
  check_launch("tcgen05 complex128 dense kernel");
}

}  // namespace gbqv
