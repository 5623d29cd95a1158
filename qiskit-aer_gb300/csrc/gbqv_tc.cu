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
// in fp32 TMEM, exactly.  Levels are recombined in int64 and rounded once
// (the int64 -> double conversion runs on the FP64 pipe, which is otherwise
// idle here, so that the integer pipe serves the digit split).
//
// One persistent CTA per SM, 17 warps, warp-specialised:
//   warps 0-7       producers: split each tile of 128 groups (two threads
//                    per group) from the raw ring into 6 fp16 digit planes
//                    in the smem stage of its parity;
//   warp M+1 lane 0  loader: bulk (TMA) copies of each tile's contiguous
//                    amplitude runs into a 3-stage raw ring;
//   warp M lane 0    issues 12 tcgen05.mma per tile (per state plane s, two
//                    K = 16 steps, N = 32 * (6 - s) matrix rows of planes
//                    t = 0..5-s), accumulating level s + t at TMEM column
//                    32 (s + t);
//   warps 8..M-1     epilogues: per pipeline lane, EH warpgroups each read
//                    the six level sums of 4/EH output chunks of their group
//                    from TMEM, recombine, store the amplitudes;
//   (M = 8 + 8 EH).
// Tiles alternate between two lanes of the pipeline (even tiles: smem stage
// 0, TMEM columns 0-191, E0; odd tiles: stage 1, columns 256-447, E1), so
// the split of one tile overlaps the MMAs and epilogue of the previous one.
//
// Shared-memory operands use the K-major no-swizzle layout: 8 rows x 16
// bytes core matrices, 128 bytes apart along K, 512 bytes apart per 8 rows.
#include <cuda.h>
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
constexpr int kRawStage = kTcGroups * 16 * 16;  // 32 KB: a tile's raw amplitudes, in run order
constexpr int kRawStages = 3;                    // bulk loads run up to three tiles ahead
// bf16 operands of the accumulator-initialising MMA: A = 128 x 16 (column 0
// ones), B = 192 x 16 (column 0 = 1.5 * 2^23), K-major, 8-row groups 256 B
// apart: D = 1.5 * 2^23 everywhere, so every level sum lands in TMEM as the
// word 0x4B400000 + T
constexpr int kInitABytes = kTcGroups * 16 * 2, kInitBBytes = 6 * kTcReals * 16 * 2;
constexpr int kOffInit = kMatBytes;
constexpr int kOffStage = kOffInit + kInitABytes + kInitBBytes;
constexpr int kOffRaw = kOffStage + 2 * kStageBytes;
constexpr int kOffKey = kOffRaw + kRawStages * kRawStage;
constexpr int kOffBar = kOffKey + 2 * kTcGroups * 4;
constexpr int kOffMisc = kOffBar + 16 * 8;
// + alignment slack; at least 116 KB so that a second CTA never fits on an SM
// (each CTA allocates all 512 TMEM columns)
constexpr int kTcSmemUsed = kOffMisc + 64 + 1024;
constexpr int kTcSmem = kTcSmemUsed > 116 * 1024 ? kTcSmemUsed : 116 * 1024;
// warps: 8 producers, 8 * EH epilogue warps (EH warpgroups per pipeline
// lane, each taking 4 / EH of the 4 output chunks), 1 MMA issuer, 1 loader
template <int EH>
constexpr int tc_threads() { return (8 + 8 * EH + 2) * 32; }
constexpr uint32_t kTmemCols = 512;

// A tile's 128 groups are the groups whose free index bits outside
// [0, L) agree, where [0, L) holds 7 free bits and the L - 7 targets below
// L.  Its 2048 amplitudes are therefore 2^(11 - L) contiguous runs of 2^L
// amplitudes (one per combination of the targets >= L): at most 16 bulk
// copies of >= 2 KB, whatever the target qubits.
struct TcParams {
  // swz = 1: the loader fetches each run with a 2D tiled TMA (rows of 8
  // amplitudes) into the 128-byte swizzle layout (16-byte chunk index XOR row
  // index mod 8), which spreads the producers' reads over all banks for any
  // targets; swz = 0 (states of >= 34 qubits): 1D bulk copies, plain layout
  CUtensorMap tmap;  // 128-byte aligned type
  uint32_t swz;
  uint64_t offs[16];
  uint64_t lowmask[4];
  uint64_t hoff[16];      // amplitude offset of run r from the tile's first amplitude
  uint64_t ngroups;
  uint64_t ntiles;
  uint32_t roff[16];      // byte offset in the raw stage of local amplitude j of group 0
  uint32_t nruns, runbytes;
  uint32_t stall;         // test hook: no accumulator commit for the CTA's first tile
  uint16_t zl[kTcGroups]; // amplitude index of group m within its run (zeros at targets < L)
  int rowbase[kTcReals];  // row key - 1017 per output real (see combine)
  int rowscale[kTcReals]; // (rowbase - 1085) * 2^20: the exponent-field add of the converting path
  int rowbase_min;        // min over rowbase: rowbase_min + group key >= 32 lets every row take a fast path
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

// A producer thread's share of a group row: the digit words (lo, hi) of its
// 8 amplitudes' 16 magnitudes and the (re, im) sign pairs (bit 15 <- sign of
// re, bit 31 <- sign of im, byte sign replication).  near: every shift of
// the warp below 32 (the two-funnel-shift split).
__device__ __forceinline__ void split_words8(const double2 (&v)[8], const uint32_t (&ex)[16], uint32_t E4, bool near,
                                             uint32_t (&lo)[16], uint32_t (&hi)[16], uint32_t (&sb)[8]) {
  if (near) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t xh = (uint32_t)__double2hiint(v[j].x), yh = (uint32_t)__double2hiint(v[j].y);
      // dithered truncation: real parts truncated (toward zero), imaginary
      // parts truncated plus one unit (away from zero), so that the two
      // biases cancel in the norm; the fast path only ever sees non-zero
      // reals, and the +1 folds into the split's constant
      const uint64_t rw = oz::split_word_abs_near(xh, (uint32_t)__double2loint(v[j].x), E4 - ex[2 * j]);
      const uint64_t iw = oz::split_word_abs_near(yh, (uint32_t)__double2loint(v[j].y), E4 - ex[2 * j + 1]) + 1;
      lo[2 * j] = (uint32_t)rw;
      hi[2 * j] = (uint32_t)(rw >> 32);
      lo[2 * j + 1] = (uint32_t)iw;
      hi[2 * j + 1] = (uint32_t)(iw >> 32);
      sb[j] = tc::prmt(xh, yh, 0xF0B0);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint64_t rw = oz::split_word_abs(v[j].x, ex[2 * j], E4);
      const uint64_t iw = oz::split_word_abs(v[j].y, ex[2 * j + 1], E4);
      lo[2 * j] = (uint32_t)rw;
      hi[2 * j] = (uint32_t)(rw >> 32);
      lo[2 * j + 1] = (uint32_t)iw;
      hi[2 * j + 1] = (uint32_t)(iw >> 32);
      sb[j] = tc::prmt((uint32_t)__double2hiint(v[j].x), (uint32_t)__double2hiint(v[j].y), 0xF0B0);
    }
  }
}

// The six fp16 digit planes of those 16 reals: K chunks 2h, 2h + 1 of group
// row m in the K-major core-matrix layout of a stage (32 reals per row).
__device__ __forceinline__ void store_planes8(unsigned char *stage, int m, int h, const uint32_t (&lo)[16],
                                              const uint32_t (&hi)[16], const uint32_t (&sb)[8]) {
  const uint32_t K64 = 0x64646464u;
#pragma unroll
  for (int q2 = 0; q2 < 2; ++q2) {
    // the chunk's 8 reals (amplitudes 4q..4q+3, re/im): per amplitude the
    // (re, im) sign pair as half2 (+-1, +-1) with the bias constants
    // times it, so that one HFMA2 per plane word both removes the fp16
    // bias and applies the signs
    uint32_t sg[4], c1[4], c0[4];
    const uint32_t *lo8 = lo + 8 * q2, *hi8 = hi + 8 * q2;
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      sg[jj] = (sb[4 * q2 + jj] & 0x80008000u) | 0x3C003C00u;
      c1[jj] = tc::hmul2(sg[jj], 0xE480E480u);  // -1152 * sign
      c0[jj] = tc::hmul2(sg[jj], 0xE600E600u);  // -1536 * sign
    }
    unsigned char *row = stage + core_off(m, 8 * (2 * h + q2));
    // digits 1..5 are byte (5 - s) of the word plus 128: fp16 0x64xx =
    // 1152 + |d| after a byte permute
    uint32_t w[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const uint32_t g = tc::prmt(lo8[2 * jj], lo8[2 * jj + 1], 0x5140);
      w[jj] = tc::hfma2(tc::prmt(g, K64, 0x4140), sg[jj], c1[jj]);
    }
    *reinterpret_cast<uint4 *>(row + 5 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const uint32_t g = tc::prmt(lo8[2 * jj], lo8[2 * jj + 1], 0x5140);
      w[jj] = tc::hfma2(tc::prmt(g, K64, 0x4342), sg[jj], c1[jj]);
    }
    *reinterpret_cast<uint4 *>(row + 4 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const uint32_t g = tc::prmt(lo8[2 * jj], lo8[2 * jj + 1], 0x7362);
      w[jj] = tc::hfma2(tc::prmt(g, K64, 0x4140), sg[jj], c1[jj]);
    }
    *reinterpret_cast<uint4 *>(row + 3 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const uint32_t g = tc::prmt(lo8[2 * jj], lo8[2 * jj + 1], 0x7362);
      w[jj] = tc::hfma2(tc::prmt(g, K64, 0x4342), sg[jj], c1[jj]);
    }
    *reinterpret_cast<uint4 *>(row + 2 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const uint32_t g = tc::prmt(hi8[2 * jj], hi8[2 * jj + 1], 0x0040);
      w[jj] = tc::hfma2(tc::prmt(g, K64, 0x4140), sg[jj], c1[jj]);
    }
    *reinterpret_cast<uint4 *>(row + 1 * kPlaneBytes) = make_uint4(w[0], w[1], w[2], w[3]);
    // digit 0: bytes 5-6 of the word are the fp16 bits of 1536 + |d_0|
#pragma unroll
    for (int jj = 0; jj < 4; ++jj)
      w[jj] = tc::hfma2(tc::prmt(hi8[2 * jj], hi8[2 * jj + 1], 0x6521), sg[jj], c0[jj]);
    *reinterpret_cast<uint4 *>(row) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// The 8 output reals of one chunk (4 amplitudes at psi[base + offs[0..3]],
// re/im) from their six TMEM level words, for rows with row key - 1017 =
// rowbase[i] and rowscale[i] = (rowbase[i] - 1085) * 2^20, group key ck.
// One vote picks the branch-free path for the whole warp (every output at
// least 2^-23 of row max x group max, and every scale in range: the usual
// case): the int64 -> double conversion on the otherwise idle FP64 pipe
// (about 2 per clock per SM) instead of ~11 integer operations per output
// on the integer pipe that the producers' split needs.  Otherwise the
// general integer normalisation.
__device__ __forceinline__ void store_outputs8(double2 *psi, uint64_t base, const uint64_t *offs,
                                               const uint32_t (&T)[6][8], const int *rowbase, const int *rowscale,
                                               int ck, bool scale_ok, bool live) {
  uint32_t vh[8], vl[8];
  bool fast = scale_ok;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    oz::words_to_v(T[0][i], T[1][i], T[2][i], T[3][i], T[4][i], T[5][i], vh[i], vl[i]);
    fast = fast && vh[i] + 1u > 1u;
  }
  const int ck20 = ck << 20;
  if (__all_sync(0xffffffffu, fast || !live)) {
    if (live) {
#pragma unroll
      for (int jj = 0; jj < 4; ++jj)
        psi[base + offs[jj]] = make_double2(oz::v_to_double_cvt(vh[2 * jj], vl[2 * jj], rowscale[2 * jj] + ck20),
                                            oz::v_to_double_cvt(vh[2 * jj + 1], vl[2 * jj + 1], rowscale[2 * jj + 1] + ck20));
    }
  } else if (live) {
    auto out_any = [&](int i) {
      const uint32_t sg = (uint32_t)((int32_t)vh[i] >> 31);
      return oz::mag_to_double(vh[i] ^ sg, vl[i] ^ sg, sg, rowbase[i] + ck);
    };
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) psi[base + offs[jj]] = make_double2(out_any(2 * jj), out_any(2 * jj + 1));
  }
}

template <int EH>
__global__ void __launch_bounds__(tc_threads<EH>(), 1)
    k_dense_tc4(double2 *psi, const __grid_constant__ TcParams p, const uint4 *__restrict__ gmat, int *status) {
  constexpr int kThreads = tc_threads<EH>(), kMmaWarp = 8 + 8 * EH, kChunks = 4 / EH;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 1024-byte alignment: the swizzle pattern is taken from address bits 4-9
  unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  int *colkey = reinterpret_cast<int *>(smem + kOffKey);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kOffBar);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kOffMisc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kOffMisc + 4);
  // barriers: full[2] (256 producer arrivals), sempty[2] (128 * EH
  // epilogue arrivals: stage and colkey read), accf[2] (MMA commit), acce[2]
  // (128 * EH epilogue arrivals: TMEM read), done (final commit)
  const uint32_t bar0 = tc::smem_u32(bars);
  auto full = [&](int b) { return bar0 + 8u * b; };
  auto sempty = [&](int b) { return bar0 + 8u * (2 + b); };
  auto accf = [&](int b) { return bar0 + 8u * (4 + b); };
  auto acce = [&](int b) { return bar0 + 8u * (6 + b); };
  const uint32_t done = bar0 + 8u * 8;
  // raw ring: raw_full[3] (loader arrival + bulk bytes), raw_empty[3] (256
  // producer arrivals once the tile's amplitudes are in registers)
  auto raw_full = [&](int r) { return bar0 + 8u * (9 + r); };
  auto raw_empty = [&](int r) { return bar0 + 8u * (12 + r); };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(full(b), 2 * kTcGroups);
      tc::mbar_init(sempty(b), kTcGroups * EH);
      tc::mbar_init(accf(b), 1);
      tc::mbar_init(acce(b), kTcGroups * EH);
    }
    tc::mbar_init(done, 1);
    for (int r = 0; r < kRawStages; ++r) {
      tc::mbar_init(raw_full(r), 1);
      tc::mbar_init(raw_empty(r), 2 * kTcGroups);
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
    // init operands: element (row, k) at (row / 8) * 256 + (k / 8) * 128 +
    // (row % 8) * 16 + (k % 8) * 2; only k = 0 is non-zero
    uint16_t *ia = reinterpret_cast<uint16_t *>(smem + kOffInit);
    for (int i = tid; i < (kInitABytes + kInitBBytes) / 2; i += kThreads) ia[i] = 0;
    __syncthreads();
    if (tid < kTcGroups) ia[(tid >> 3) * 128 + (tid & 7) * 8] = 0x3F80;  // bf16 1.0
    if (tid < 6 * kTcReals) ia[kInitABytes / 2 + (tid >> 3) * 128 + (tid & 7) * 8] = 0x4B40;  // bf16 1.5 * 2^23
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
    // raw amplitudes arrive by bulk copies from the loader; this thread's 8
    // amplitudes sit at fixed offsets of each raw stage
    uint32_t ro[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t off = p.roff[8 * h + j] + 16u * p.zl[m];
      ro[j] = p.swz ? off ^ (((off >> 7) & 7u) << 4) : off;
    }
    uint64_t tile = blockIdx.x;
    int slot = 0;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i, slot = slot == kRawStages - 1 ? 0 : slot + 1) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      const bool landed = tc::mbar_wait(raw_full(slot), (i / kRawStages) & 1, abort_flag);
      if (!__all_sync(0xffffffffu, landed)) break;
      const unsigned char *raw = smem + kOffRaw + slot * kRawStage;
      auto amp = [&](int j) { return *reinterpret_cast<const double2 *>(raw + ro[j]); };
      // the group key: the largest biased exponent field plus one (0 for an
      // all-zero group, which is never stored); the fields are kept
      double2 v[8];
      uint32_t ex[16];
      uint32_t mx = 0, mn = 0x7ff;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        v[j] = amp(j);
        ex[2 * j] = ((uint32_t)__double2hiint(v[j].x) >> 20) & 0x7ff;
        ex[2 * j + 1] = ((uint32_t)__double2hiint(v[j].y) >> 20) & 0x7ff;
        mx = max(mx, max(ex[2 * j], ex[2 * j + 1]));
        mn = min(mn, min(ex[2 * j], ex[2 * j + 1]));
      }
      // the amplitudes are in registers now: the raw slot goes back to the
      // loader before the split.  The proxy fence orders these generic-proxy
      // reads before the loader's next bulk (async-proxy) write to the slot.
      tc::fence_async_smem();
      tc::mbar_arrive(raw_empty(slot));
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
      const int key = mx ? (int)mx + 1 : 0;
      const uint32_t E4 = (uint32_t)key + 4;
      // every real of the warp non-zero and within 2^-26 of its group's
      // largest: the split takes two 32-bit funnel shifts (the usual case
      // for a dense state); otherwise the general 64-bit shift
      const bool near = __all_sync(0xffffffffu, mn != 0 && mn + 31 >= E4);
      const bool ok = c == 0 || tc::mbar_wait(sempty(b), (c - 1) & 1, abort_flag);
      if (!__all_sync(0xffffffffu, ok)) break;
      // digit words of the 16 magnitudes and the sign pairs, then the planes
      uint32_t lo[16], hi[16], sb[8];
      split_words8(v, ex, E4, near, lo, hi, sb);
      store_planes8(smem + kOffStage + b * kStageBytes, m, h, lo, hi, sb);
      if (h == 0) colkey[b * kTcGroups + m] = key;
      tc::fence_async_smem();
      tc::mbar_arrive(full(b));
    }
  } else if (warp < kMmaWarp) {
    // ---------------- epilogues ----------------
    const int e = warp - 8, b = (e >> 2) & 1, half = e >> 3, quarter = warp & 3, m = 32 * quarter + lane;
    const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)b * 256u;
    uint64_t tile = blockIdx.x + (uint64_t)b * gridDim.x;
    for (uint32_t c = 0; tile < ntiles; tile += stride2, ++c) {
      // the first warp of the warpgroup polls; the other three sleep in the
      // named barrier (ids 1..2 EH), which keeps the issue slots for the
      // producers while the accumulator is not ready
      bool ok = true;
      if (quarter == 0) {
        ok = tc::mbar_wait(accf(b), c & 1, abort_flag);
        ok = ok && tc::mbar_wait(full(b), c & 1, abort_flag);  // producer's colkey write
      }
      if (!tc::bar_and(1 + (e >> 2), 128, ok)) break;
      tc::fence_after_sync();
      const int ck = colkey[b * kTcGroups + m];
      tc::mbar_arrive(sempty(b));
      const uint64_t grp = tile * kTcGroups + m;
      const bool live = grp < p.ngroups && ck != 0;
      const uint64_t base = live ? insert_zeros_k4(grp, p.lowmask) : 0;
      const bool scale_ok = p.rowbase_min + ck >= 32;
#pragma unroll
      for (int qq = 0; qq < kChunks; ++qq) {
        const int q = half * kChunks + qq;
        uint32_t T[6][8];
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::tmem_ld8(tbase + 32u * l + 8u * q, T[l]);
        tc::tmem_wait_ld();
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::pin(T[l]);
        store_outputs8(psi, base, p.offs + 4 * q, T, p.rowbase + 8 * q, p.rowscale + 8 * q, ck, scale_ok, live);
      }
      tc::fence_before_sync();
      tc::mbar_arrive(acce(b));
    }
  } else if (warp == kMmaWarp + 1 && lane == 0) {
    // ---------------- loader: bulk copies of the raw ring ----------------
    uint64_t tile = blockIdx.x;
    uint32_t issued = 0;
    int slot = 0;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i, slot = slot == kRawStages - 1 ? 0 : slot + 1) {
      if (i >= kRawStages && !tc::mbar_wait(raw_empty(slot), (i / kRawStages - 1) & 1, abort_flag, 64)) break;
      const uint64_t first = insert_zeros_k4(tile * kTcGroups, p.lowmask);
      const uint32_t dst = tc::smem_u32(smem + kOffRaw + slot * kRawStage);
      tc::mbar_arrive_expect_tx(raw_full(slot), kRawStage);
      if (p.swz) {
        for (uint32_t r = 0; r < p.nruns; ++r)
          tc::tma_load_2d(dst + r * p.runbytes, &p.tmap, 0, (int)((first + p.hoff[r]) >> 3), raw_full(slot));
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
  } else if (warp == kMmaWarp && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t mat = tc::smem_u32(smem);
    uint64_t tile = blockIdx.x;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = (int)(i & 1);
      const uint32_t c = i >> 1;
      if (!tc::mbar_wait(full(b), c & 1, abort_flag, 32)) break;
      if (c >= 1 && !tc::mbar_wait(acce(b), (c - 1) & 1, abort_flag, 32)) break;
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(smem + kOffStage + b * kStageBytes);
      const uint32_t d0 = tmem + (uint32_t)b * 256u;
      const uint32_t ini = tc::smem_u32(smem + kOffInit);
      tc::mma_f16(d0, tc::smem_desc(ini, 128, 256), tc::smem_desc(ini + kInitABytes, 128, 256),
                  tc::idesc_bf16_f32(128, 6 * kTcReals), 0);
#pragma unroll
      for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int kk = 0; kk < 2; ++kk)
          tc::mma_f16(d0 + 32u * s, tc::smem_desc(a0 + s * kPlaneBytes + kk * 256, 128, 512),
                      tc::smem_desc(mat + kk * 256, 128, 512), tc::idesc_f16_f32(128, 32 * (6 - s)), 1);
      // the test hook leaves the first tile's accumulator uncommitted: its
      // epilogue's bounded wait runs out and the CTA takes the abort path
      if (!(p.stall && i == 0)) tc::mma_commit(accf(b));
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
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, kTmemCols);
  if (tid == 0 && *abort_flag) atomicExch(status, 1);
}

// ---------------------------------------------------------------------------
// 5-qubit gates (k_dense_tc5): a group is 32 amplitudes (64 reals).  The
// tile's 128 groups are taken in two K-halves, split by the highest target:
// half kh holds local amplitudes 16 kh .. 16 kh + 15 of every group, which is
// a 4-qubit tile (32 KB raw, 32 reals per row) on the four lower targets.
// Both halves of a tile share one group key (the exponent pass reads both
// raw halves first).  The two output halves (output reals 0-31, 32-63) take
// the two TMEM accumulators (columns 0 and 256) the 4-qubit kernel gives its
// pipeline lanes, so epilogue warpgroups 0-1 drain output half 0 and 2-3
// output half 1 of the same tile.  Per tile the MMA thread issues, for each
// output half o and K-half kh, the 12 digit-plane MMAs of the 4-qubit kernel
// with B = the matrix planes of rows 32 o .. 32 o + 31, columns 32 kh ..
// 32 kh + 31: 48 MMAs and two accumulator preloads.  Shared memory: matrix
// planes 48 KB (6 planes x 64 rows x 64 reals, rows of an output half
// contiguous across planes), two K-half plane stages of 48 KB, two raw
// K-half slots of 32 KB.
constexpr int k5MatBytes = 6 * 64 * 64 * 2;  // 48 KB
constexpr int k5OffInit = k5MatBytes;
constexpr int k5OffStage = k5OffInit + kInitABytes + kInitBBytes;
constexpr int k5OffRaw = k5OffStage + 2 * kStageBytes;
constexpr int k5OffKey = k5OffRaw + 2 * kRawStage;
constexpr int k5OffBar = k5OffKey + 2 * kTcGroups * 4;
constexpr int k5OffMisc = k5OffBar + 16 * 8;
constexpr int k5Smem = k5OffMisc + 64 + 1024;
static_assert(k5Smem <= 232448, "shared memory per CTA");
static_assert(k5OffRaw % 1024 == 0, "raw slots on the swizzle period");

struct Tc5Params {
  CUtensorMap tmap;  // 2D, rows of 8 amplitudes, box = a run (swz = 1)
  uint32_t swz;
  uint64_t offs[32];      // amplitude offset of local amplitude j (targets sorted ascending)
  uint64_t lowmask[5];
  uint64_t hoff[32];      // amplitude offset of run r from the tile's first amplitude
  uint64_t ngroups;
  uint64_t ntiles;
  uint32_t roff[16];      // byte offset in a raw K-half slot of local amplitude j (< 16) of group 0
  uint32_t nhalf, runbytes;  // runs per K-half (runs [kh nhalf, (kh + 1) nhalf) form half kh)
  uint16_t zl[kTcGroups];
  int rowbase[64];        // row key - 1017 per output real
  int rowscale[64];       // (rowbase - 1085) * 2^20
  int rowbase_min;
};

// byte offset of element (row, k) in the matrix operand: rows of 64 reals
__host__ __device__ constexpr uint32_t core_off64(uint32_t row, uint32_t k) {
  return (row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint64_t insert_zeros_k5(uint64_t g, const uint64_t *lowmask) {
#pragma unroll
  for (int j = 0; j < 5; ++j) g = ((g & ~lowmask[j]) << 1) | (g & lowmask[j]);
  return g;
}

__global__ void __launch_bounds__(tc_threads<2>(), 1)
    k_dense_tc5(double2 *psi, const __grid_constant__ Tc5Params p, const uint4 *__restrict__ gmat, int *status) {
  constexpr int kThreads = tc_threads<2>(), kMmaWarp = 24;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  int *colkey = reinterpret_cast<int *>(smem + k5OffKey);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + k5OffBar);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + k5OffMisc);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + k5OffMisc + 4);
  // barriers, each with one ordered waiter sequence:
  //   full[kh]  256 producer arrivals: K-half kh's planes written (MMA waits)
  //   sfree[kh] MMA commit: stage kh read (producers wait)
  //   accf[o]   MMA commit: output half o ready (its epilogue waits)
  //   acce[o]   256 epilogue arrivals: output half o read (MMA waits)
  //   keyf[p]   256 producer arrivals: colkey[p] written (epilogues wait)
  //   raw_full[kh] loader + bytes (producers wait), raw_empty[kh] 256
  //   producer arrivals (loader waits), done: final commit
  const uint32_t bar0 = tc::smem_u32(bars);
  auto full = [&](int x) { return bar0 + 8u * x; };
  auto sfree = [&](int x) { return bar0 + 8u * (2 + x); };
  auto accf = [&](int x) { return bar0 + 8u * (4 + x); };
  auto acce = [&](int x) { return bar0 + 8u * (6 + x); };
  auto keyf = [&](int x) { return bar0 + 8u * (8 + x); };
  auto raw_full = [&](int x) { return bar0 + 8u * (10 + x); };
  auto raw_empty = [&](int x) { return bar0 + 8u * (12 + x); };
  const uint32_t done = bar0 + 8u * 14;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int x = 0; x < 2; ++x) {
      tc::mbar_init(full(x), 2 * kTcGroups);
      tc::mbar_init(sfree(x), 1);
      tc::mbar_init(accf(x), 1);
      tc::mbar_init(acce(x), 2 * kTcGroups);
      tc::mbar_init(keyf(x), 2 * kTcGroups);
      tc::mbar_init(raw_full(x), 1);
      tc::mbar_init(raw_empty(x), 2 * kTcGroups);
    }
    tc::mbar_init(done, 1);
    *abort_flag = 0;
    tc::mbar_init_fence();
  }
  if (warp == kMmaWarp) {
    tc::tmem_alloc(tc::smem_u32(tmem_slot), kTmemCols);
    tc::tmem_relinquish();
  }
  {
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = tid; i < k5MatBytes / 16; i += kThreads) dst[i] = gmat[i];
    uint16_t *ia = reinterpret_cast<uint16_t *>(smem + k5OffInit);
    for (int i = tid; i < (kInitABytes + kInitBBytes) / 2; i += kThreads) ia[i] = 0;
    __syncthreads();
    if (tid < kTcGroups) ia[(tid >> 3) * 128 + (tid & 7) * 8] = 0x3F80;  // bf16 1.0
    if (tid < 6 * kTcReals) ia[kInitABytes / 2 + (tid >> 3) * 128 + (tid & 7) * 8] = 0x4B40;  // bf16 1.5 * 2^23
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint64_t ntiles = p.ntiles;

  if (warp < 8) {
    // ---------------- producers: two threads per group, 8 amplitudes of each K-half ----------------
    const int m = 16 * warp + (lane & 15), h = lane >> 4;
    uint32_t ro[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t off = p.roff[8 * h + j] + 16u * p.zl[m];
      ro[j] = p.swz ? off ^ (((off >> 7) & 7u) << 4) : off;
    }
    uint64_t tile = blockIdx.x;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      bool ok = tc::mbar_wait(raw_full(0), i & 1, abort_flag);
      ok = ok && tc::mbar_wait(raw_full(1), i & 1, abort_flag);
      if (!__all_sync(0xffffffffu, ok)) break;
      // the group key over both K-halves (exponent fields of the 32 reals)
      uint32_t mx = 0, mn = 0x7ff;
#pragma unroll
      for (int kh = 0; kh < 2; ++kh) {
        const unsigned char *raw = smem + k5OffRaw + kh * kRawStage;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const uint32_t xh = *reinterpret_cast<const uint32_t *>(raw + ro[j] + 4);
          const uint32_t yh = *reinterpret_cast<const uint32_t *>(raw + ro[j] + 12);
          const uint32_t ea = (xh >> 20) & 0x7ff, eb = (yh >> 20) & 0x7ff;
          mx = max(mx, max(ea, eb));
          mn = min(mn, min(ea, eb));
        }
      }
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
      const int key = mx ? (int)mx + 1 : 0;
      const uint32_t E4 = (uint32_t)key + 4;
      const bool near = __all_sync(0xffffffffu, mn != 0 && mn + 31 >= E4);
      bool stop = false;
#pragma unroll 1
      for (int kh = 0; kh < 2; ++kh) {
        const unsigned char *raw = smem + k5OffRaw + kh * kRawStage;
        double2 v[8];
        uint32_t ex[16];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          v[j] = *reinterpret_cast<const double2 *>(raw + ro[j]);
          ex[2 * j] = ((uint32_t)__double2hiint(v[j].x) >> 20) & 0x7ff;
          ex[2 * j + 1] = ((uint32_t)__double2hiint(v[j].y) >> 20) & 0x7ff;
        }
        tc::fence_async_smem();
        tc::mbar_arrive(raw_empty(kh));
        uint32_t lo[16], hi[16], sb[8];
        split_words8(v, ex, E4, near, lo, hi, sb);
        const bool freed = i == 0 || tc::mbar_wait(sfree(kh), (i - 1) & 1, abort_flag);
        if (!__all_sync(0xffffffffu, freed)) {
          stop = true;
          break;
        }
        store_planes8(smem + k5OffStage + kh * kStageBytes, m, h, lo, hi, sb);
        if (kh == 0) {
          if (h == 0) colkey[(i & 1) * kTcGroups + m] = key;
          tc::mbar_arrive(keyf(i & 1));
        }
        tc::fence_async_smem();
        tc::mbar_arrive(full(kh));
      }
      if (stop) break;
    }
  } else if (warp < kMmaWarp) {
    // ---------------- epilogues: warpgroups 0-1 output half 0, 2-3 output half 1 ----------------
    const int e = warp - 8, o = (e >> 3) & 1, half = (e >> 2) & 1, quarter = warp & 3, m = 32 * quarter + lane;
    const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)o * 256u;
    uint64_t tile = blockIdx.x;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      // one polling warp per warpgroup, the others wait in named barrier
      // 1 + warpgroup
      bool ok = true;
      if (quarter == 0) {
        ok = tc::mbar_wait(accf(o), i & 1, abort_flag);
        ok = ok && tc::mbar_wait(keyf(i & 1), (i >> 1) & 1, abort_flag);
      }
      if (!tc::bar_and(1 + (e >> 2), 128, ok)) break;
      tc::fence_after_sync();
      const int ck = colkey[(i & 1) * kTcGroups + m];
      const uint64_t grp = tile * kTcGroups + m;
      const bool live = grp < p.ngroups && ck != 0;
      const uint64_t base = live ? insert_zeros_k5(grp, p.lowmask) : 0;
      const bool scale_ok = p.rowbase_min + ck >= 32;
#pragma unroll
      for (int qq = 0; qq < 2; ++qq) {
        const int q = half * 2 + qq;  // chunk of 8 output reals within the output half
        uint32_t T[6][8];
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::tmem_ld8(tbase + 32u * l + 8u * q, T[l]);
        tc::tmem_wait_ld();
#pragma unroll
        for (int l = 0; l < 6; ++l) tc::pin(T[l]);
        const int a0 = 16 * o + 4 * q;  // first local amplitude of the chunk
        store_outputs8(psi, base, p.offs + a0, T, p.rowbase + 32 * o + 8 * q, p.rowscale + 32 * o + 8 * q, ck,
                       scale_ok, live);
      }
      tc::fence_before_sync();
      tc::mbar_arrive(acce(o));
    }
  } else if (warp == kMmaWarp + 1 && lane == 0) {
    // ---------------- loader: K-half kh of each tile into raw slot kh ----------------
    uint64_t tile = blockIdx.x;
    uint32_t issued = 0;
    for (uint32_t i = 0; tile < ntiles; tile += gridDim.x, ++i) {
      const uint64_t first = insert_zeros_k5(tile * kTcGroups, p.lowmask);
      bool ok = true;
      for (int kh = 0; kh < 2 && ok; ++kh) {
        if (i >= 1 && !tc::mbar_wait(raw_empty(kh), (i - 1) & 1, abort_flag, 64)) {
          ok = false;
          break;
        }
        const uint32_t dst = tc::smem_u32(smem + k5OffRaw + kh * kRawStage);
        tc::mbar_arrive_expect_tx(raw_full(kh), kRawStage);
        for (uint32_t r = 0; r < p.nhalf; ++r) {
          const uint64_t off = first + p.hoff[kh * p.nhalf + r];
          if (p.swz)
            tc::tma_load_2d(dst + r * p.runbytes, &p.tmap, 0, (int)(off >> 3), raw_full(kh));
          else
            tc::bulk_g2s(dst + r * p.runbytes, psi + off, p.runbytes, raw_full(kh));
        }
        issued = 2 * i + kh + 1;
      }
      if (!ok) break;
      // the CTA's next tile into L2 now: its K-halves are loaded only as the
      // producers free this tile's slots, and then arrive from L2
      const uint64_t next = tile + gridDim.x;
      if (next < ntiles) {
        const uint64_t nfirst = insert_zeros_k5(next * kTcGroups, p.lowmask);
        for (uint32_t r = 0; r < 2 * p.nhalf; ++r) {
          const uint64_t off = nfirst + p.hoff[r];
          if (p.swz)
            tc::tma_prefetch_2d(&p.tmap, 0, (int)(off >> 3));
          else
            tc::bulk_prefetch_l2(psi + off, p.runbytes);
        }
      }
    }
    // copies in flight after an abort land before the CTA exits
    int never = 0;
    for (uint32_t x = issued > 2 ? issued - 2 : 0; x < issued; ++x)
      tc::mbar_wait(raw_full((int)(x & 1)), (x >> 1) & 1, &never);
  } else if (warp == kMmaWarp && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t mat = tc::smem_u32(smem);
    const uint32_t ini = tc::smem_u32(smem + k5OffInit);
    uint64_t tile = blockIdx.x;
    bool ok = true;
    for (uint32_t i = 0; tile < ntiles && ok; tile += gridDim.x, ++i) {
      for (int kh = 0; kh < 2 && ok; ++kh) {
        if (!tc::mbar_wait(full(kh), i & 1, abort_flag, 32)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t a0 = tc::smem_u32(smem + k5OffStage + kh * kStageBytes);
        for (int o = 0; o < 2; ++o) {
          const uint32_t d0 = tmem + (uint32_t)o * 256u;
          if (kh == 0) {
            // output half o of the previous tile has been read: preload its accumulators
            if (i >= 1 && !tc::mbar_wait(acce(o), (i - 1) & 1, abort_flag, 32)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            tc::mma_f16(d0, tc::smem_desc(ini, 128, 256), tc::smem_desc(ini + kInitABytes, 128, 256),
                        tc::idesc_bf16_f32(128, 6 * kTcReals), 0);
          }
#pragma unroll
          for (int s = 0; s < 6; ++s)
#pragma unroll
            for (int kk = 0; kk < 2; ++kk)
              tc::mma_f16(d0 + 32u * s, tc::smem_desc(a0 + s * kPlaneBytes + kk * 256, 128, 512),
                          tc::smem_desc(mat + (uint32_t)o * 24576u + (uint32_t)(4 * kh + 2 * kk) * 128u, 128, 1024),
                          tc::idesc_f16_f32(128, 32 * (6 - s)), 1);
          if (kh == 1) tc::mma_commit(accf(o));
        }
        if (ok) tc::mma_commit(sfree(kh));
      }
    }
    tc::mma_commit(done);
    int never = 0;
    tc::mbar_wait(done, 0, &never);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, kTmemCols);
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

}  // namespace

// Run geometry of a 128-group tile of a k-qubit gate (k = 4, 5) on targets
// `qubits`: run offsets hoff[r] (amplitudes), byte offsets roff[j] of local
// amplitude j of group 0 in the raw stage, zl[m] = amplitude index of group m
// inside its run; amp_bytes = 16 (complex128) or 8 (complex64).
void tc_tile_geometry(const reg_t &qubits, uint64_t *hoff, uint32_t *roff, uint16_t *zl, uint32_t &nruns,
                      uint32_t &runbytes, uint32_t amp_bytes) {
  const int k = (int)qubits.size();
  reg_t sq = qubits;
  std::sort(sq.begin(), sq.end());
  uint32_t L = 7;
  for (uint64_t q : sq)
    if (q < L) ++L;
  std::vector<uint64_t> high;
  for (uint64_t q : sq)
    if (q >= L) high.push_back(q);
  nruns = 1u << high.size();
  runbytes = amp_bytes << L;
  for (uint32_t r = 0; r < nruns; ++r) {
    uint64_t off = 0;
    for (size_t t = 0; t < high.size(); ++t)
      if (r >> t & 1) off |= 1ULL << high[t];
    hoff[r] = off;
  }
  for (uint32_t j = 0; j < (1u << k); ++j) {
    uint64_t lowpart = 0;
    uint32_t r = 0;
    for (int t = 0; t < k; ++t) {
      if (!(j >> t & 1)) continue;
      const uint64_t q = qubits[t];
      if (q < L) {
        lowpart |= 1ULL << q;
      } else {
        const size_t rank = (size_t)(std::find(high.begin(), high.end(), q) - high.begin());
        r |= 1u << rank;
      }
    }
    roff[j] = r * runbytes + (uint32_t)(lowpart * amp_bytes);
  }
  for (uint32_t m = 0; m < 128u; ++m) {
    uint64_t g = m;
    for (uint64_t q : sq)
      if (q < L) g = ((g >> q) << (q + 1)) | (g & ((1ULL << q) - 1));
    zl[m] = (uint16_t)g;
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encode_tiled() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(ptr);
    cudaGetLastError();
  }
  return fn;
}

// The swizzled descriptor for run length L (the state as rows of 128 bytes,
// box height = the run), or false (1D bulk path) when the state is too large
// for int32 row coordinates or encoding fails.
bool tc_tensor_map(Device &dev, uint32_t L, void *out) {
  const uint32_t amp_log2 = dev.dbl ? 4 : 3, row_amps_log2 = 7 - amp_log2;
  if ((uint32_t)dev.n - row_amps_log2 >= 31 || L < 7 || L > 12) return false;
  if (dev.tmap_state != dev.state) {
    dev.tmap_ok = 0;
    dev.tmap_state = dev.state;
  }
  const int i = (int)L - 7;
  if (!(dev.tmap_ok >> i & 1u)) {
    const EncodeTiled fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {16, (cuuint64_t)1 << (dev.n - row_amps_log2)};
    const cuuint64_t strides[1] = {128};
    const cuuint32_t box[2] = {16, 1u << (L - row_amps_log2)};
    const cuuint32_t es[2] = {1, 1};
    if (fn(reinterpret_cast<CUtensorMap *>(dev.tmap[i]), CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, dev.state, dims, strides,
           box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
    dev.tmap_ok |= 1u << i;
  }
  std::memcpy(out, dev.tmap[i], 128);
  return true;
}

// A descriptor that fetches several runs of a tile in one request: the state
// as rows of 128 bytes (dims 0, 1) plus one dimension of size 2 and stride
// 2^q amplitudes for each of the first (up to three) targets q >= L, box
// height = the run.  Up to three high targets take one request per tile; each
// further high target doubles the requests: request q starts row_off[q] rows
// further (bits of q over the fourth and fifth high targets) and 8 runs
// further in shared memory.  Same shared-memory layout as one request per run
// (run r = bits of r over the high targets, ascending).  False: use the
// per-run path.
bool tc_runs_map(Device &dev, const reg_t &qubits, uint32_t L, void *out, uint32_t &rank, uint32_t &nreq,
                 uint32_t *row_off) {
  const uint32_t amp_log2 = dev.dbl ? 4 : 3, row_amps_log2 = 7 - amp_log2;
  if ((uint32_t)dev.n - row_amps_log2 >= 31 || L < 7 || L > 12) return false;
  const EncodeTiled fn = encode_tiled();
  if (!fn) return false;
  reg_t high;
  for (uint64_t q : qubits)
    if (q >= L) high.push_back(q);
  std::sort(high.begin(), high.end());
  if (high.size() > 5) return false;
  const uint32_t nd = (uint32_t)std::min<size_t>(high.size(), 3);
  rank = 2 + nd;
  nreq = high.size() > 3 ? 1u << (high.size() - 3) : 1u;
  for (uint32_t q = 0; q < nreq; ++q) {
    uint64_t rows = 0;
    for (size_t t = 3; t < high.size(); ++t)
      if (q >> (t - 3) & 1) rows += 1ULL << (high[t] - row_amps_log2);
    if (rows > 0x7fffffffULL) return false;
    row_off[q] = (uint32_t)rows;
  }
  cuuint64_t dims[5] = {16, (cuuint64_t)1 << (dev.n - row_amps_log2), 2, 2, 2};
  cuuint64_t strides[4] = {128, 0, 0, 0};
  cuuint32_t box[5] = {16, 1u << (L - row_amps_log2), 2, 2, 2};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  for (uint32_t t = 0; t < nd; ++t) strides[1 + t] = (cuuint64_t)1 << (high[t] + amp_log2);
  return fn(reinterpret_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_UINT64, rank, dev.state, dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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

// Host: six fp16 digit planes of the real form of a 32x32 column-major
// complex matrix (targets sorted), rows = output reals (2j + c), K = input
// reals; matrix row r = 32 o + r' of plane t at operand row (6 o + t) 32 + r'.
void tc_matrix5(const cd *mat, uint16_t *planes, int *rowkey) {
  constexpr int D = 32, R = 64;
  std::vector<double> A((size_t)R * R);
  for (int j = 0; j < D; ++j)
    for (int jp = 0; jp < D; ++jp) {
      const cd z = mat[j + (size_t)D * jp];
      A[(size_t)(2 * j) * R + 2 * jp] = z.real();
      A[(size_t)(2 * j) * R + 2 * jp + 1] = -z.imag();
      A[(size_t)(2 * j + 1) * R + 2 * jp] = z.imag();
      A[(size_t)(2 * j + 1) * R + 2 * jp + 1] = z.real();
    }
  std::memset(planes, 0, k5MatBytes);
  for (int r = 0; r < R; ++r) {
    int key = 0;
    for (int k = 0; k < R; ++k) key = std::max(key, oz::exp_key(A[(size_t)r * R + k]));
    rowkey[r] = key;
    const int o = r / 32, rr = r % 32;
    for (int k = 0; k < R; ++k) {
      int32_t d[6];
      oz::bsum_digits(oz::split_bsum(A[(size_t)r * R + k], key), d);
      for (int t = 0; t < 6; ++t) planes[core_off64((uint32_t)((6 * o + t) * 32 + rr), (uint32_t)k) / 2] = half_bits(d[t]);
    }
  }
}

// The 5-qubit tcgen05 kernel takes a gate whose highest target lies above
// the tile's run bits (so that the two K-halves are two sets of runs) on a
// state of at least 12 qubits; 4 targets below L at most keep a run within
// the 2D descriptor's 256-row box.
bool tc5_usable(const Device &dev, const reg_t &qubits) {
  if (!dev.dbl || dev.tensor_c128 != 1 || qubits.size() != 5 || dev.n < 12) return false;
  reg_t sq = qubits;
  std::sort(sq.begin(), sq.end());
  uint32_t L = 7;
  for (uint64_t q : sq)
    if (q < L) ++L;
  return sq[4] >= L;
}

void launch_dense_tc5(Device &dev, const reg_t &qubits_in, const cd *mat_in) {
  // targets sorted ascending, the matrix permuted to match
  reg_t qubits = qubits_in;
  std::sort(qubits.begin(), qubits.end());
  int ob[5];
  for (int b = 0; b < 5; ++b)
    ob[b] = (int)(std::find(qubits_in.begin(), qubits_in.end(), qubits[b]) - qubits_in.begin());
  auto perm = [&](int x) {
    int y = 0;
    for (int b = 0; b < 5; ++b) y |= ((x >> b) & 1) << ob[b];
    return y;
  };
  std::vector<cd> matv(32 * 32);
  for (int r = 0; r < 32; ++r)
    for (int c = 0; c < 32; ++c) matv[r + 32 * c] = mat_in[perm(r) + 32 * perm(c)];
  Tc5Params p;
  local_offsets(qubits, p.offs);
  sorted_masks(qubits, p.lowmask);
  p.ngroups = dev.amps() >> 5;
  p.ntiles = (p.ngroups + kTcGroups - 1) / kTcGroups;
  uint64_t hoff[32];
  uint32_t roff[32], nruns = 0, runbytes = 0;
  tc_tile_geometry(qubits, hoff, roff, p.zl, nruns, runbytes, 16);
  if (nruns < 2) throw Error(1, "5-qubit tensor kernel: the highest target must lie above the tile's runs");
  for (uint32_t r = 0; r < nruns; ++r) p.hoff[r] = hoff[r];
  for (int j = 0; j < 16; ++j) p.roff[j] = roff[j];
  p.nhalf = nruns / 2;
  p.runbytes = runbytes;
  uint32_t L = 0;
  while ((16u << L) < runbytes) ++L;
  p.swz = tc_tensor_map(dev, L, &p.tmap) ? 1u : 0u;
  std::vector<uint16_t> planes(k5MatBytes / 2);
  int rowkey[64];
  tc_matrix5(matv.data(), planes.data(), rowkey);
  p.rowbase_min = 1 << 30;
  for (int r = 0; r < 64; ++r) {
    p.rowbase[r] = rowkey[r] - 1017;
    p.rowscale[r] = (int)((uint32_t)(p.rowbase[r] - 1085) << 20);
    p.rowbase_min = std::min(p.rowbase_min, p.rowbase[r]);
  }
  grow(dev.mat, dev.mat_cap, k5MatBytes);
  cuda_check(cudaMemcpyAsync(dev.mat, planes.data(), k5MatBytes, cudaMemcpyHostToDevice, dev.stream),
             "matrix upload");
  int *status = tc_status_word(dev);
  static bool attr = false;
  if (!attr) {
    cuda_check(cudaFuncSetAttribute(k_dense_tc5, cudaFuncAttributeMaxDynamicSharedMemorySize, k5Smem),
               "tcgen05 5-qubit kernel attribute");
    attr = true;
  }
  const uint64_t grid = std::min<uint64_t>(p.ntiles, (uint64_t)sm_count());
  k_dense_tc5<<<(unsigned)grid, tc_threads<2>(), k5Smem, dev.stream>>>(reinterpret_cast<double2 *>(dev.state), p,
                                                                      reinterpret_cast<const uint4 *>(dev.mat), status);
  check_launch("tcgen05 complex128 5-qubit dense kernel");
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
  tc_tile_geometry(qubits, p.hoff, p.roff, p.zl, p.nruns, p.runbytes, 16);
  uint32_t L = 0;
  while ((16u << L) < p.runbytes) ++L;
  p.swz = tc_tensor_map(dev, L, &p.tmap) ? 1u : 0u;
  std::vector<uint16_t> planes(kMatBytes / 2);
  int rowkey[kTcReals];
  tc_matrix4(mat, planes.data(), rowkey);
  p.rowbase_min = 1 << 30;
  for (int r = 0; r < kTcReals; ++r) {
    p.rowbase[r] = rowkey[r] - 1017;
    p.rowscale[r] = (int)((uint32_t)(p.rowbase[r] - 1085) << 20);
    p.rowbase_min = std::min(p.rowbase_min, p.rowbase[r]);
  }
  p.stall = dev.tc_test_stall ? 1u : 0u;
  grow(dev.mat, dev.mat_cap, kMatBytes);
  cuda_check(cudaMemcpyAsync(dev.mat, planes.data(), kMatBytes, cudaMemcpyHostToDevice, dev.stream), "matrix upload");
  int *status = tc_status_word(dev);
  const uint64_t grid = std::min<uint64_t>(p.ntiles, (uint64_t)sm_count());
  auto launch = [&](auto kernel, int threads, bool &attr) {
    if (!attr) {
      cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem),
                 "tcgen05 kernel attribute");
      attr = true;
    }
    kernel<<<(unsigned)grid, threads, kTcSmem, dev.stream>>>(reinterpret_cast<double2 *>(dev.state), p,
                                                             reinterpret_cast<const uint4 *>(dev.mat), status);
  };
  // two epilogue warpgroups per pipeline lane measured 11% faster than one
  // (30 qubits: 8.7 vs 9.8 ms per gate)
  static bool attr = false;
  launch(k_dense_tc4<2>, tc_threads<2>(), attr);
  check_launch("tcgen05 complex128 dense kernel");
}

}  // namespace gbqv
