// gbqv_tc64.cu — complex64 dense 4- and 5-qubit gates on the 5th-generation
// tensor cores in split precision (3xTF32): QubitVector<float>::apply_matrix
// (src/simulators/statevector/qubitvector.hpp:1298-1303, apply_lambda over
// 2^k-amplitude groups) for the fused ops of the complex64 workloads (Aer's
// Fusion emits dense ops of up to 5 qubits).
//
// Every real x of a group and every entry a of the real form of the matrix
// [[Re U, -Im U], [Im U, Re U]] is split as x = x_hi + x_lo with x_hi = x
// rounded to TF32 (10-bit mantissa) and x_lo = x - x_hi exact in fp32; the
// tensor core computes a_hi x_hi and a_lo x_hi + a_hi x_lo (the a_lo x_lo
// term is below fp32 resolution) with fp32 accumulation in TMEM: the hi x hi
// products of the R / 8 K steps in 4 (k = 4) or 3 (k = 5) accumulators and
// the cross terms in one more, added in fp32 in the epilogue.  The tensor
// core's accumulation truncates; with one accumulator the 3 R / 8 - 1
// accumulating MMAs biased every output towards zero and the norm drifted
// (2e-5 after 24 5-qubit gates, 8e-6 with the cross terms apart).  The split costs two SIMT ops per
// real and the result is read straight from TMEM, so, unlike the complex128
// kernel, the SIMT side is light.
//
// One persistent CTA per SM, 18 warps, the same pipeline as the complex128
// kernel (gbqv_tc.cu); R = 2^(k+1) reals per group (32 or 64):
//   warps 0-7       producers: two threads per group split each tile of 128
//                    groups from the raw ring into two tf32 planes (hi, lo)
//                    in the smem stage of the tile's parity;
//   warps 8-15      epilogues: one warpgroup per pipeline lane reads the R
//                    fp32 outputs of its group from TMEM and stores them;
//   warp 16 lane 0  issues 3 R / 8 tcgen05.mma.kind::tf32 per tile (R / 8
//                    K = 8 steps x {hi*lo, lo*hi -> cross accumulator,
//                    hi*hi -> main accumulator kk mod kMain}, M = 128,
//                    N = R) into the lane's TMEM columns, commits to accf
//                    (epilogue) and sfree (producers);
//   warp 17 lane 0  loader: tiled TMA loads (rows of 16 amplitudes, 128-byte
//                    swizzle) of each tile's <= 2^k contiguous runs into the
//                    raw ring (4 stages of 16 KB for k = 4, 2 of 32 KB for
//                    k = 5), 1 to 4 requests per tile (a descriptor with up
//                    to three high targets as extra dimensions; runs of 1 KB
//                    fetched one by one ran at 0.45 of HBM).
// Shared-memory operands: K-major, no swizzle, 8-row x 16-byte core matrices
// (4 tf32), 128 bytes apart along K, 4 R bytes apart per 8 rows.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "gbqv_internal.h"
#include "gbqv_tc.cuh"

namespace gbqv {
namespace {

constexpr int kG = 128;  // groups per tile (MMA M)

// Sizes of the k-qubit kernel (k = 4, 5).
template <int KQ>
struct Tc64Shape {
  static constexpr int kAmps = 1 << KQ;                 // amplitudes per group
  static constexpr int kR = 2 * kAmps;                  // reals per group (MMA K, matrix rows, N)
  static constexpr int kHalf = kAmps / 2;               // amplitudes per producer thread
  static constexpr int kPlane = kG * kR * 4;            // one tf32 plane of a tile (16 / 32 KB)
  static constexpr int kStage = 2 * kPlane;             // hi, lo
  static constexpr int kMatBytes = 2 * kR * kR * 4;     // matrix hi, lo (8 / 32 KB)
  static constexpr int kRawStage = kG * kAmps * 8;      // a tile's raw amplitudes (16 / 32 KB)
  static constexpr int kRawStages = KQ == 4 ? 4 : 2;    // 64 KB in flight either way
  static constexpr int kSbo = kR * 32;                  // bytes between 8-row groups of an operand
  static constexpr int kOffStage = kMatBytes;
  static constexpr int kOffRaw = kOffStage + 2 * kStage;
  static constexpr int kOffBar = kOffRaw + kRawStages * kRawStage;
  static constexpr int kOffMisc = kOffBar + 24 * 8;
  static constexpr int kSmem = kOffMisc + 64 + 1024;   // + 1024-byte alignment slack
  // per pipeline lane b (columns 256 b ..): kMain accumulators of the hi * hi
  // products (K step kk into accumulator kk mod kMain) at 256 b + j R, then
  // the cross terms at 256 b + kMain R
  static constexpr int kMain = KQ == 4 ? 4 : 3;
  static constexpr uint32_t kTmemCols = 512;
  static_assert((kMain + 1) * kR <= 256, "accumulators of a pipeline lane");
  static_assert(kSmem <= 232448, "shared memory per CTA");
};
constexpr int kThreads = 18 * 32;
constexpr int kMmaWarp = 16, kLoadWarp = 17;

template <int KQ>
struct Tc64Params {
  CUtensorMap tmap;   // 128-byte aligned type; the state as rows of 16 amplitudes
  // loads of a tile's runs into the 128-byte swizzle layout: 2 = 1..4
  // requests per tile of a descriptor whose extra dimensions are the high
  // targets (rank, row_off: see tc_runs_map); 1 = one 2D request per run;
  // 0 = 1D bulk copies, plain layout (35 qubits)
  uint32_t swz, rank, nreq;
  uint32_t row_off[4];
  // targets are sorted ascending (the matrix permuted to match); pair0 = 1
  // when qubit 0 is a target: amplitudes j, j + 1 (j even) are then adjacent
  // in memory and move as one 16-byte access
  uint32_t pair0;
  uint64_t offs[1 << KQ];
  uint64_t lowmask[KQ];
  uint64_t hoff[1 << KQ];
  uint64_t ngroups;
  uint64_t ntiles;
  uint32_t roff[1 << KQ];
  uint32_t nruns, runbytes;
  uint16_t zl[kG];
};

template <int KQ>
__device__ __forceinline__ uint64_t insert_zeros_k(uint64_t g, const uint64_t *lowmask) {
#pragma unroll
  for (int j = 0; j < KQ; ++j) g = ((g & ~lowmask[j]) << 1) | (g & lowmask[j]);
  return g;
}

// byte offset of tf32 element (row, k) in a K-major no-swizzle operand whose
// rows hold R reals
template <int R>
__host__ __device__ constexpr uint32_t off_r(uint32_t row, uint32_t k) {
  return (row >> 3) * (R * 32) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// TF32 rounding (nearest, ties away from zero) of an fp32 bit pattern.
__host__ __device__ __forceinline__ uint32_t tf32_bits(uint32_t f) { return (f + 0x1000u) & 0xFFFFE000u; }

// Instruction descriptor of kind::tf32: D f32, A and B tf32 (format 2), K-major.
__host__ __device__ __forceinline__ uint32_t idesc_tf32_f32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

template <int KQ>
__global__ void __launch_bounds__(kThreads, 1)
    k_dense_tc_c64(float2 *psi, const __grid_constant__ Tc64Params<KQ> p, const uint4 *__restrict__ gmat, int *status) {
  using S = Tc64Shape<KQ>;
  constexpr int kR = S::kR, kHalf = S::kHalf, kPlane = S::kPlane, kStage = S::kStage, kMatBytes = S::kMatBytes;
  constexpr int kRawStage = S::kRawStage, kRawStages = S::kRawStages, kOffStage = S::kOffStage;
  constexpr int kOffRaw = S::kOffRaw, kOffBar = S::kOffBar, kOffMisc = S::kOffMisc;
  constexpr uint32_t kTmemCols = S::kTmemCols;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 1024-byte alignment: the swizzle pattern is taken from address bits 4-9
  unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kOffBar);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kOffMisc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kOffMisc + 4);
  // barriers, each with one ordered waiter sequence: full[2] (256 producer
  // arrivals; the MMA thread waits), sfree[2] (MMA commit: the stage has been
  // read; producers wait), accf[2] (MMA commit: accumulator ready; the lane's
  // epilogue waits), acce[2] (128 epilogue arrivals: TMEM read; the MMA
  // thread waits), done (final commit), raw_full[4] (loader arrival + bytes;
  // producers wait), raw_empty[4] (256 producer arrivals; the loader waits)
  const uint32_t bar0 = tc::smem_u32(bars);
  auto full = [&](int b) { return bar0 + 8u * b; };
  auto sfree = [&](int b) { return bar0 + 8u * (2 + b); };
  auto accf = [&](int b) { return bar0 + 8u * (4 + b); };
  auto acce = [&](int b) { return bar0 + 8u * (6 + b); };
  const uint32_t done = bar0 + 8u * 8;
  auto raw_full = [&](int r) { return bar0 + 8u * (9 + r); };
  auto raw_empty = [&](int r) { return bar0 + 8u * (13 + r); };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(full(b), 2 * kG);
      tc::mbar_init(sfree(b), 1);
      tc::mbar_init(accf(b), 1);
      tc::mbar_init(acce(b), kG);
    }
    tc::mbar_init(done, 1);
    for (int r = 0; r < kRawStages; ++r) {
      tc::mbar_init(raw_full(r), 1);
      tc::mbar_init(raw_empty(r), 2 * kG);
    }
    *abort_flag = 0;
    tc::mbar_init_fence();
  }
  if (warp == kMmaWarp) {
    tc::tmem_alloc(tc::smem_u32(tmem_slot), kTmemCols);
    tc::tmem_relinquish();
  }
  {
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = tid; i < kMatBytes / 16; i += kThreads) dst[i] = gmat[i];
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint64_t ntiles = p.ntiles;

  if (warp < 8) {
    // ---------------- producers ----------------
    // two threads per group, in the two half-warps: half h owns amplitudes
    // kHalf h .. kHalf (h + 1) - 1, i.e. K chunks of 4 reals from kHalf h / 2
    const int m = 16 * warp + (lane & 15), h = lane >> 4;
    uint32_t ro[kHalf];
#pragma unroll
    for (int j = 0; j < kHalf; ++j) {
      const uint32_t off = p.roff[kHalf * h + j] + 8u * p.zl[m];
      ro[j] = p.swz != 0 ? off ^ (((off >> 7) & 7u) << 4) : off;
    }
    uint64_t tile = blockIdx.x;
    int slot = 0;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i, slot = slot == kRawStages - 1 ? 0 : slot + 1) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      const bool landed = tc::mbar_wait(raw_full(slot), (i / kRawStages) & 1, abort_flag);
      if (!__all_sync(0xffffffffu, landed)) break;
      const unsigned char *raw = smem + kOffRaw + slot * kRawStage;
      float2 v[kHalf];
      if (p.pair0) {
#pragma unroll
        for (int j = 0; j < kHalf; j += 2) {
          const float4 w = *reinterpret_cast<const float4 *>(raw + ro[j]);
          v[j] = make_float2(w.x, w.y);
          v[j + 1] = make_float2(w.z, w.w);
        }
      } else {
#pragma unroll
        for (int j = 0; j < kHalf; ++j) v[j] = *reinterpret_cast<const float2 *>(raw + ro[j]);
      }
      // in registers: the raw slot goes back to the loader (the proxy fence
      // orders these reads before its next async-proxy write)
      tc::fence_async_smem();
      tc::mbar_arrive(raw_empty(slot));
      const bool ok = c == 0 || tc::mbar_wait(sfree(b), (c - 1) & 1, abort_flag);
      if (!__all_sync(0xffffffffu, ok)) break;
      unsigned char *stage = smem + kOffStage + b * kStage;
#pragma unroll
      for (int cc = 0; cc < kHalf / 2; ++cc) {
        const float x[4] = {v[2 * cc].x, v[2 * cc].y, v[2 * cc + 1].x, v[2 * cc + 1].y};
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          hi[e] = tf32_bits(__float_as_uint(x[e]));
          lo[e] = __float_as_uint(x[e] - __uint_as_float(hi[e]));  // exact
        }
        const uint32_t o = off_r<kR>((uint32_t)m, 4u * ((kHalf / 2) * h + cc));
        *reinterpret_cast<uint4 *>(stage + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4 *>(stage + kPlane + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
      tc::fence_async_smem();
      tc::mbar_arrive(full(b));
    }
  } else if (warp < kMmaWarp) {
    // ---------------- epilogues: warpgroup b serves pipeline lane b ----------------
    const int b = (warp - 8) >> 2, quarter = warp & 3, m = 32 * quarter + lane;
    const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)b * 256u;
    uint64_t tile = blockIdx.x + (uint64_t)b * gridDim.x;
    for (uint32_t c = 0; tile < ntiles; tile += 2ULL * gridDim.x, ++c) {
      // one polling warp per warpgroup, the others wait in named barrier 1 + b
      const bool ok = quarter != 0 || tc::mbar_wait(accf(b), c & 1, abort_flag);
      if (!tc::bar_and(1 + b, 128, ok)) break;
      tc::fence_after_sync();
      uint32_t T[kR / 8][8];
#pragma unroll
      for (int q = 0; q < kR / 8; ++q) tc::tmem_ld8(tbase + 8u * q, T[q]);
      tc::tmem_wait_ld();
#pragma unroll
      for (int q = 0; q < kR / 8; ++q) tc::pin(T[q]);
      // output = the kMain hi * hi sums + the cross-term sum, added in fp32
      // (round to nearest): no full-size partial sum passes through the
      // tensor core's truncating accumulation
      constexpr int kC = kR / 8 <= 4 ? kR / 8 : 2;
#pragma unroll
      for (int a = 1; a <= S::kMain; ++a)
#pragma unroll
      for (int q0 = 0; q0 < kR / 8; q0 += kC) {
        uint32_t C[kC][8];
#pragma unroll
        for (int qq = 0; qq < kC; ++qq) tc::tmem_ld8(tbase + (uint32_t)(a * kR) + 8u * (q0 + qq), C[qq]);
        tc::tmem_wait_ld();
#pragma unroll
        for (int qq = 0; qq < kC; ++qq) {
          tc::pin(C[qq]);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            T[q0 + qq][i] = __float_as_uint(__uint_as_float(T[q0 + qq][i]) + __uint_as_float(C[qq][i]));
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(acce(b));
      // n >= 11: every tile is full, so the whole warp takes this branch
      // (the lane-pair exchange below needs all 32 lanes)
      const uint64_t grp = tile * kG + m;
      if (grp < p.ngroups) {
        const uint64_t base = insert_zeros_k<KQ>(grp, p.lowmask);
        // output reals 2j, 2j + 1 (columns) are amplitude j (re, im)
        auto out = [&](int j) {
          return make_float2(__uint_as_float(T[j >> 2][(2 * j) & 7]), __uint_as_float(T[j >> 2][(2 * j + 1) & 7]));
        };
        if (p.pair0) {
#pragma unroll
          for (int j = 0; j < S::kAmps; j += 2) {
            const float2 a = out(j), c = out(j + 1);
            *reinterpret_cast<float4 *>(psi + base + p.offs[j]) = make_float4(a.x, a.y, c.x, c.y);
          }
        } else {
          // qubit 0 is free: groups 2i, 2i + 1 (lanes 2i, 2i + 1) are adjacent
          // for every j; after one exchange the even lane stores amplitude
          // 2jj of both groups, the odd lane amplitude 2jj + 1 of both
          const bool odd = lane & 1;
#pragma unroll
          for (int jj = 0; jj < S::kAmps / 2; ++jj) {
            const float2 e = out(2 * jj), o = out(2 * jj + 1);
            const float2 give = odd ? e : o;
            const float2 got = make_float2(__shfl_xor_sync(0xffffffffu, give.x, 1), __shfl_xor_sync(0xffffffffu, give.y, 1));
            if (odd)
              *reinterpret_cast<float4 *>(psi + (base - 1) + p.offs[2 * jj + 1]) = make_float4(got.x, got.y, o.x, o.y);
            else
              *reinterpret_cast<float4 *>(psi + base + p.offs[2 * jj]) = make_float4(e.x, e.y, got.x, got.y);
          }
        }
      }
    }
  } else if (warp == kMmaWarp && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t mat = tc::smem_u32(smem);
    const uint32_t idesc = idesc_tf32_f32(128, kR);
    uint64_t tile = blockIdx.x;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      if (!tc::mbar_wait(full(b), c & 1, abort_flag, 32)) break;
      if (c >= 1 && !tc::mbar_wait(acce(b), (c - 1) & 1, abort_flag, 32)) break;
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(smem + kOffStage + b * kStage);
      const uint32_t d = tmem + (uint32_t)b * 256u;
#pragma unroll
      for (int kk = 0; kk < kR / 8; ++kk) {
        const uint64_t ahi = tc::smem_desc(a0 + kk * 256, 128, S::kSbo);
        const uint64_t alo = tc::smem_desc(a0 + kPlane + kk * 256, 128, S::kSbo);
        const uint64_t bhi = tc::smem_desc(mat + kk * 256, 128, S::kSbo);
        const uint64_t blo = tc::smem_desc(mat + kR * kR * 4 + kk * 256, 128, S::kSbo);
        // the two cross terms (small) into their own accumulator, hi * hi
        // into main accumulator kk mod kMain
        const uint32_t dc = d + (uint32_t)(S::kMain * kR), dm = d + (uint32_t)((kk % S::kMain) * kR);
        mma_tf32(dc, ahi, blo, idesc, kk != 0);
        mma_tf32(dc, alo, bhi, idesc, 1);
        mma_tf32(dm, ahi, bhi, idesc, kk >= S::kMain);
      }
      tc::mma_commit(accf(b));
      tc::mma_commit(sfree(b));
    }
    // every MMA issued above has completed once `done` flips (bounded wait,
    // independent of the abort flag so TMEM is never freed under a live MMA)
    tc::mma_commit(done);
    int never = 0;
    tc::mbar_wait(done, 0, &never);
  } else if (warp == kLoadWarp && lane == 0) {
    // ---------------- loader: TMA copies of the raw ring ----------------
    uint64_t tile = blockIdx.x;
    uint32_t issued = 0;
    int slot = 0;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i, slot = slot == kRawStages - 1 ? 0 : slot + 1) {
      if (i >= kRawStages && !tc::mbar_wait(raw_empty(slot), (i / kRawStages - 1) & 1, abort_flag, 64)) break;
      const uint64_t first = insert_zeros_k<KQ>(tile * kG, p.lowmask);
      const uint32_t dst = tc::smem_u32(smem + kOffRaw + slot * kRawStage);
      tc::mbar_arrive_expect_tx(raw_full(slot), kRawStage);
      if (p.swz == 2) {
        for (uint32_t q = 0; q < p.nreq; ++q) {
          const uint32_t d = dst + q * 8u * p.runbytes;
          const int y = (int)(first >> 4) + (int)p.row_off[q];
          if (p.rank == 2)
            tc::tma_load_2d(d, &p.tmap, 0, y, raw_full(slot));
          else if (p.rank == 3)
            tc::tma_load_nd<3>(d, &p.tmap, y, raw_full(slot));
          else if (p.rank == 4)
            tc::tma_load_nd<4>(d, &p.tmap, y, raw_full(slot));
          else
            tc::tma_load_nd<5>(d, &p.tmap, y, raw_full(slot));
        }
      } else if (p.swz == 1) {
        for (uint32_t r = 0; r < p.nruns; ++r)
          tc::tma_load_2d(dst + r * p.runbytes, &p.tmap, 0, (int)((first + p.hoff[r]) >> 4), raw_full(slot));
      } else {
        for (uint32_t r = 0; r < p.nruns; ++r)
          tc::bulk_g2s(dst + r * p.runbytes, psi + first + p.hoff[r], p.runbytes, raw_full(slot));
      }
      issued = i + 1;
    }
    // copies still in flight after an abort land before the CTA exits
    int never = 0;
    for (uint32_t i = issued > kRawStages ? issued - kRawStages : 0; i < issued; ++i)
      tc::mbar_wait(raw_full((int)(i % kRawStages)), (i / kRawStages) & 1, &never);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, kTmemCols);
  if (tid == 0 && *abort_flag) atomicExch(status, 1);
}

}  // namespace

// Host: the hi / lo tf32 planes of the real form of a D x D column-major
// complex matrix (D = 2^KQ; rows and columns ordered (amplitude j, re/im) ->
// 2j + c), in the core-matrix layout of the B operand: hi = entry rounded to
// TF32, lo = fp32 of the remainder (the tensor core reads its TF32 part).
template <int KQ>
void tc64_matrix(const cd *mat, uint32_t *planes) {
  constexpr int D = 1 << KQ, R = 2 * D;
  std::memset(planes, 0, Tc64Shape<KQ>::kMatBytes);
  auto put = [&](int r, int k, double x) {
    const float xf = (float)x;
    uint32_t fb;
    std::memcpy(&fb, &xf, 4);
    const uint32_t hb = tf32_bits(fb);
    float hf;
    std::memcpy(&hf, &hb, 4);
    const float lf = (float)(x - (double)hf);
    uint32_t lb;
    std::memcpy(&lb, &lf, 4);
    planes[off_r<R>((uint32_t)r, (uint32_t)k) / 4] = hb;
    planes[(R * R * 4 + off_r<R>((uint32_t)r, (uint32_t)k)) / 4] = lb;
  };
  for (int j = 0; j < D; ++j)
    for (int jp = 0; jp < D; ++jp) {
      const cd z = mat[j + (size_t)D * jp];
      put(2 * j, 2 * jp, z.real());
      put(2 * j, 2 * jp + 1, -z.imag());
      put(2 * j + 1, 2 * jp, z.imag());
      put(2 * j + 1, 2 * jp + 1, z.real());
    }
}

template <int KQ>
void launch_tc64(Device &dev, const reg_t &qubits_in, const cd *mat_in) {
  using S = Tc64Shape<KQ>;
  constexpr int D = 1 << KQ;
  // sort the targets; local index bit b' of the sorted order is bit o[b'] of
  // the caller's order
  reg_t qubits = qubits_in;
  std::sort(qubits.begin(), qubits.end());
  int o[KQ];
  for (int b = 0; b < KQ; ++b)
    o[b] = (int)(std::find(qubits_in.begin(), qubits_in.end(), qubits[b]) - qubits_in.begin());
  auto perm = [&](int x) {
    int y = 0;
    for (int b = 0; b < KQ; ++b) y |= ((x >> b) & 1) << o[b];
    return y;
  };
  std::vector<cd> matv((size_t)D * D);
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) matv[r + D * c] = mat_in[perm(r) + D * perm(c)];
  Tc64Params<KQ> p;
  p.pair0 = qubits[0] == 0 ? 1u : 0u;
  local_offsets(qubits, p.offs);
  sorted_masks(qubits, p.lowmask);
  p.ngroups = dev.amps() >> KQ;
  p.ntiles = (p.ngroups + kG - 1) / kG;
  tc_tile_geometry(qubits, p.hoff, p.roff, p.zl, p.nruns, p.runbytes, 8);
  uint32_t L = 0;
  while ((8u << L) < p.runbytes) ++L;
  p.rank = 2;
  p.nreq = 1;
  for (uint32_t &r : p.row_off) r = 0;
  if (tc_runs_map(dev, qubits, L, &p.tmap, p.rank, p.nreq, p.row_off))
    p.swz = 2;
  else
    p.swz = tc_tensor_map(dev, L, &p.tmap) ? 1u : 0u;
  std::vector<uint32_t> planes(S::kMatBytes / 4);
  tc64_matrix<KQ>(matv.data(), planes.data());
  grow(dev.mat, dev.mat_cap, S::kMatBytes);
  cuda_check(cudaMemcpyAsync(dev.mat, planes.data(), S::kMatBytes, cudaMemcpyHostToDevice, dev.stream),
             "matrix upload");
  int *status = tc_status_word(dev);
  static bool attr = false;
  if (!attr) {
    cuda_check(cudaFuncSetAttribute(k_dense_tc_c64<KQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem),
               "tcgen05 complex64 kernel attribute");
    attr = true;
  }
  const uint64_t grid = std::min<uint64_t>(p.ntiles, (uint64_t)sm_count());
  k_dense_tc_c64<KQ><<<(unsigned)grid, kThreads, S::kSmem, dev.stream>>>(
      reinterpret_cast<float2 *>(dev.state), p, reinterpret_cast<const uint4 *>(dev.mat), status);
  check_launch("tcgen05 complex64 dense kernel");
}

bool tc64_dense_available(const Device &dev, int k) {
  return !dev.dbl && dev.tensor_c128 == 1 && (k == 4 || k == 5) && dev.n >= 7 + k;
}

void launch_dense_tc64(Device &dev, const reg_t &qubits, const cd *mat) {
  if (qubits.size() == 5)
    launch_tc64<5>(dev, qubits, mat);
  else
    launch_tc64<4>(dev, qubits, mat);
}

}  // namespace gbqv
