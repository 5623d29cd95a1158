// gbqv_runreg.cu — cache-blocked runs with the tile held in registers.
//
// A run (a sequence of 1-2 qubit dense ops, diagonals and multi-controlled
// X gates whose qubits all lie in one tile of m vector qubits) costs one
// HBM read and one write of the state.  Inside the tile the ops used to
// sweep shared memory one by one with a barrier between them; here each of
// the 256 threads holds 2^(m-8) amplitudes of the tile in registers.  The m
// tile bits are split into register bits (the thread's own amplitudes) and
// 8 thread bits; an op whose dense qubits are register bits is applied in
// registers, a 1-qubit dense op or an X target on one of the 5 lane bits is
// applied with warp shuffles, diagonals and controls may sit on any bit.
// When an op needs a bit that is neither, the tile is re-laid out once
// through shared memory (a "segment" boundary) so that its bits become
// register bits; the host picks each segment's register bits by next use.
// Arithmetic per op is that of the shared-memory run kernel (the same
// products; a lane op sums its two terms in the order own, partner).
#include <cuda.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "gbqv_internal.h"
#include "gbqv_runreg_dev_src.inc"  // kFpairSrc, kRunRegDevSrc: texts of gbqv_fpair.cuh, gbqv_runreg_dev.cuh (the build)

namespace gbqv {
namespace {

// Tile shapes.  complex64: 256 threads (8 thread bits), 5 register bits (32
// amplitudes a thread), two CTAs per SM each with one tile buffer, so that
// one CTA's loads and barriers overlap the other's arithmetic.  complex128:
// 512 threads (9 thread bits), 3 register bits, one CTA per SM with two tile
// buffers (the next tile loads while this one is computed).  The
// interpreting kernel at 32 register amplitudes needs more than 128
// registers a thread for its dispatch: one CTA per SM, two buffers.
int reg_tbits(bool dbl) { return dbl ? 9 : 8; }
template <typename T, int RB>
struct RegShape {
  static constexpr int kThreads = sizeof(T) == 8 ? 256 : 512;
  static constexpr int kTbits = sizeof(T) == 8 ? 8 : 9;
  static constexpr int kCtas = (sizeof(T) == 8 && RB <= 4) ? 2 : 1;
  static constexpr int kBufs = kCtas == 1 ? 2 : 1;
};
// the specialised kernel's: 128 registers suffice at complex64
struct JitShape {
  int threads, tbits, ctas, bufs;
};
JitShape jit_shape(bool dbl) { return dbl ? JitShape{512, 9, 1, 2} : JitShape{256, 8, 2, 1}; }
constexpr int kRegMaxOps = 24;
constexpr int kRegMaxSegs = kRegMaxOps + 1;

enum RegKind : int {
  RK_DENSE1 = 0,       // 1-qubit dense, target on register bit a
  RK_DENSE1_REAL = 1,  // the same with a real matrix (every binding)
  RK_DENSE1_LANE = 2,  // 1-qubit dense, target on lane bit a
  RK_DENSE2 = 3,       // 2-qubit dense on register bits a < b (matrix bit 0 <-> a)
  RK_DIAG1 = 4,        // 1-qubit diagonal on register bit a
  RK_DIAG = 5,         // diagonal on any bits
  RK_MCX = 6,          // multi-controlled X, target on register bit a
  RK_MCX_LANE = 7,     // multi-controlled X, target on lane bit a
  RK_DIAG_T = 8,       // diagonal whose qubits are all thread bits: one factor per thread
  RK_DENSE1_REAL_LANE = 9,  // RK_DENSE1_LANE with a real matrix
};

struct RegOp {
  int kind, k, a, b;
  int bound, mat_off;   // matrix in the per-binding block (bound) or the shared pool
  uint32_t ctm, crm;    // X controls: bits of the thread index / of the register index
  int8_t dtpos[5];      // diagonal: thread-bit position of op qubit j, -1 on a register bit
  uint8_t div[32];      // diagonal: index bits that register i contributes
};

struct RegSeg {
  int first, count;     // ops [first, first + count)
  uint16_t rp[32];      // tile index bits of register i
  uint8_t tb[16];       // tile bit held by thread-index bit q (q < 9)
};
static_assert(sizeof(RegSeg) % 8 == 0 && sizeof(RegOp) % 8 == 0, "shared-memory layout keeps 8-byte alignment");

struct RegParams {
  int m, c, rb, nops, nsegs, pool_elems, bound_elems, state_bits;
  uint64_t nbind, ntiles;
  uint64_t tile_lowmask[kMaxQubits];
  int T[24];
  RegOp ops[kRegMaxOps];
  RegSeg segs[kRegMaxSegs];
};

#include "gbqv_runreg_dev.cuh"

template <typename T, int R, int A>
__device__ __forceinline__ void dense2_b(T (&v)[R], const T *m, int b) {
  constexpr int RB = R == 32 ? 5 : R == 16 ? 4 : R == 8 ? 3 : 2;
  switch (b) {
    case 1: if constexpr (A < 1 && 1 < RB) reg_dense2<T, R, A, 1>(v, m); break;
    case 2: if constexpr (A < 2 && 2 < RB) reg_dense2<T, R, A, 2>(v, m); break;
    case 3: if constexpr (A < 3 && 3 < RB) reg_dense2<T, R, A, 3>(v, m); break;
    case 4: if constexpr (A < 4 && 4 < RB) reg_dense2<T, R, A, 4>(v, m); break;
    default: break;
  }
}

template <typename T, int R>
__device__ __forceinline__ void apply_reg_op(T (&v)[R], const RegOp &op, const T *mat, int tid) {
  constexpr int RB = R == 32 ? 5 : R == 16 ? 4 : R == 8 ? 3 : 2;
  const int lane = tid & 31;
  switch (op.kind) {
    case RK_DENSE1:
    case RK_DENSE1_REAL:
    case RK_DIAG1:
    case RK_MCX: {
      const bool tcond = ((uint32_t)tid & op.ctm) == op.ctm;
#define GBQV_REG_CASE(J)                                                    \
  case J:                                                                   \
    if constexpr (J < RB) {                                                 \
      if (op.kind == RK_DENSE1) reg_dense1<T, R, J>(v, mat);                \
      else if (op.kind == RK_DENSE1_REAL) reg_dense1_real<T, R, J>(v, mat); \
      else if (op.kind == RK_DIAG1) reg_diag1<T, R, J>(v, mat);             \
      else reg_mcx<T, R, J>(v, tcond, op.crm);                              \
    }                                                                       \
    break;
      switch (op.a) {
        GBQV_REG_CASE(0)
        GBQV_REG_CASE(1)
        GBQV_REG_CASE(2)
        GBQV_REG_CASE(3)
        GBQV_REG_CASE(4)
        default: break;
      }
#undef GBQV_REG_CASE
      return;
    }
    case RK_DENSE2:
      switch (op.a) {
        case 0: dense2_b<T, R, 0>(v, mat, op.b); break;
        case 1: dense2_b<T, R, 1>(v, mat, op.b); break;
        case 2: dense2_b<T, R, 2>(v, mat, op.b); break;
        case 3: dense2_b<T, R, 3>(v, mat, op.b); break;
        default: break;
      }
      return;
    case RK_DENSE1_LANE:
      lane_dense1<T, R>(v, mat, op.a, lane);
      return;
    case RK_DENSE1_REAL_LANE:
      lane_dense1_real<T, R>(v, mat, op.a, lane);
      return;
    case RK_DIAG_T: {
      uint32_t td = 0;
      for (int j = 0; j < op.k; ++j) td |= (((uint32_t)tid >> op.dtpos[j]) & 1u) << j;
      thread_diag<T, R>(v, mat, td);
      return;
    }
    case RK_MCX_LANE:
      lane_mcx<T, R>(v, op.a, ((uint32_t)tid & op.ctm) == op.ctm, op.crm);
      return;
    case RK_DIAG: {
      uint32_t td = 0;
      for (int j = 0; j < op.k; ++j)
        if (op.dtpos[j] >= 0) td |= (((uint32_t)tid >> op.dtpos[j]) & 1u) << j;
#pragma unroll
      for (int i = 0; i < R; ++i) v[i] = cmul(v[i], mat[td | op.div[i]]);
      return;
    }
    default: return;
  }
}

// One or two tile buffers (RegShape): with two, tile t + gridDim.x is
// fetched with cp.async into one while tile t is computed in registers (and
// re-laid out) through the other; with one, tile t is fetched, computed and
// written back while the SM's other CTA overlaps it.
template <typename T, int RB>
__global__ void __launch_bounds__(RegShape<T, RB>::kThreads, RegShape<T, RB>::kCtas)
    k_run_reg(T *__restrict__ psi, const RegParams *__restrict__ P, const T *__restrict__ pool,
              const T *__restrict__ bpool) {
  constexpr int R = 1 << RB, NT = RegShape<T, RB>::kThreads, TBITS = RegShape<T, RB>::kTbits,
                NBUF = RegShape<T, RB>::kBufs;
  constexpr uint32_t kPer = 16 / sizeof(T);  // amplitudes per 16-byte copy
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = P->m, c = P->c, nsegs = P->nsegs, nops = P->nops;
  const int tid = threadIdx.x;
  const uint32_t L = 1u << m, cmask = (1u << c) - 1;
  T *buf0 = reinterpret_cast<T *>(smem_raw);
  T *buf1 = buf0 + (NBUF == 2 ? L : 0);
  T *mats = buf0 + NBUF * L;
  T *bmats = mats + P->pool_elems;
  RegOp *ops = reinterpret_cast<RegOp *>(bmats + P->bound_elems);
  RegSeg *segs = reinterpret_cast<RegSeg *>(ops + nops);
  uint64_t *hi = reinterpret_cast<uint64_t *>((reinterpret_cast<uintptr_t>(segs + nsegs) + 7) & ~uintptr_t(7));
  for (int i = tid; i < P->pool_elems; i += NT) mats[i] = pool[i];
  {
    const int *src = reinterpret_cast<const int *>(P->ops);
    int *dst = reinterpret_cast<int *>(ops);
    for (int i = tid; i < nops * (int)(sizeof(RegOp) / 4); i += NT) dst[i] = src[i];
    src = reinterpret_cast<const int *>(P->segs);
    dst = reinterpret_cast<int *>(segs);
    for (int i = tid; i < nsegs * (int)(sizeof(RegSeg) / 4); i += NT) dst[i] = src[i];
  }
  const uint32_t nhi = 1u << (m - c);
  for (uint32_t h = tid; h < nhi; h += NT) {
    uint64_t a = 0;
    for (int j = c; j < m; ++j)
      if ((h >> (j - c)) & 1) a |= 1ULL << P->T[j];
    hi[h] = a;
  }
  __syncthreads();
  const bool bound = P->bound_elems > 0;
  // a padding state of a bound stack is neither read nor written
  auto skip = [&](uint64_t gb) { return bound && (gb >> P->state_bits) >= P->nbind; };
  auto fetch = [&](uint64_t t, T *buf) {
    const uint64_t gb = tile_base(t, P->tile_lowmask, m);
    if (skip(gb)) return;
    for (uint32_t ch = tid; ch < L / kPer; ch += NT) {
      const uint32_t l = ch * kPer;  // kPer consecutive tile indices: consecutive amplitudes (c >= 4)
      cp_async16(buf + l, psi + (gb | hi[l >> c] | (l & cmask)));
    }
  };
  uint64_t t = blockIdx.x;
  if (NBUF == 2) {
    if (t < P->ntiles) fetch(t, buf0);
    cp_async_commit();
  }
  for (int k = 0; t < P->ntiles; t += gridDim.x, ++k) {
    T *tile = (NBUF == 2 && (k & 1)) ? buf1 : buf0;
    const uint64_t gbase = tile_base(t, P->tile_lowmask, m);
    if (NBUF == 2) {
      if (t + gridDim.x < P->ntiles) fetch(t + gridDim.x, (k & 1) ? buf0 : buf1);
      cp_async_commit();
      cp_async_wait<1>();  // this tile's copies (all but the group just issued)
      __syncthreads();
      if (skip(gbase)) continue;  // same value in every thread of the CTA
    } else {
      if (skip(gbase)) continue;
      fetch(t, tile);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    if (bound) {
      const T *src = bpool + (gbase >> P->state_bits) * (uint64_t)P->bound_elems;
      for (int i = tid; i < P->bound_elems; i += NT) bmats[i] = src[i];
      __syncthreads();
    }
    T v[R];
    uint32_t tpart = 0;
    for (int s = 0; s < nsegs; ++s) {
      const RegSeg &S = segs[s];
      if (s > 0) {
        const RegSeg &Sp = segs[s - 1];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < R; ++i) tile[tpart | Sp.rp[i]] = v[i];
        __syncthreads();
      }
      tpart = 0;
#pragma unroll
      for (int q = 0; q < TBITS; ++q) tpart |= (((uint32_t)tid >> q) & 1u) << S.tb[q];
#pragma unroll
      for (int i = 0; i < R; ++i) v[i] = tile[tpart | S.rp[i]];
      for (int o = S.first; o < S.first + S.count; ++o) {
        const RegOp &op = ops[o];
        apply_reg_op<T, R>(v, op, (op.bound ? bmats : mats) + op.mat_off, tid);
      }
    }
    {
      const RegSeg &Sl = segs[nsegs - 1];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < R; ++i) tile[tpart | Sl.rp[i]] = v[i];
    }
    __syncthreads();
    for (uint32_t l = tid; l < L; l += NT) psi[gbase | hi[l >> c] | (l & cmask)] = tile[l];
    __syncthreads();  // the buffer is fetched into again; bmats are rewritten next tile
  }
  cp_async_wait<0>();
}

template <typename T> T to_dev(const cd &z);
template <> double2 to_dev<double2>(const cd &z) { return make_double2(z.real(), z.imag()); }
template <> float2 to_dev<float2>(const cd &z) { return make_float2((float)z.real(), (float)z.imag()); }

// dense 2-qubit matrix with its two index bits exchanged
std::vector<cd> swap_bits2(const cd *m) {
  static const int s[4] = {0, 2, 1, 3};
  std::vector<cd> o(16);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) o[s[r] + 4 * s[c]] = m[r + 4 * c];
  return o;
}

template <typename T, int RB>
void launch_reg_t(Device &dev, RegParams &P, const std::vector<T> &pool, const std::vector<T> &bpool) {
  const size_t pbytes = sizeof(RegParams), poolb = pool.size() * sizeof(T), bpoolb = bpool.size() * sizeof(T);
  const size_t pool_off = (pbytes + 255) & ~size_t(255);
  const size_t bpool_off = (pool_off + poolb + 255) & ~size_t(255);
  grow(dev.mat, dev.mat_cap, bpool_off + bpoolb + 256);
  char *base = reinterpret_cast<char *>(dev.mat);
  cuda_check(cudaMemcpyAsync(base, &P, pbytes, cudaMemcpyHostToDevice, dev.stream), "run upload");
  if (poolb)
    cuda_check(cudaMemcpyAsync(base + pool_off, pool.data(), poolb, cudaMemcpyHostToDevice, dev.stream), "run upload");
  if (bpoolb)
    cuda_check(cudaMemcpyAsync(base + bpool_off, bpool.data(), bpoolb, cudaMemcpyHostToDevice, dev.stream),
               "run upload");
  constexpr int NT = RegShape<T, RB>::kThreads;
  size_t smem = sizeof(T) * (RegShape<T, RB>::kBufs * (1u << P.m) + pool.size() + (size_t)P.bound_elems);
  smem += sizeof(RegOp) * P.nops + sizeof(RegSeg) * P.nsegs;
  smem = (smem + 7) & ~size_t(7);
  smem += sizeof(uint64_t) * (1u << (P.m - P.c));
  static bool attr_set = false;
  if (!attr_set) {
    cuda_check(cudaFuncSetAttribute(k_run_reg<T, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
               "run kernel attribute");
    attr_set = true;
  }
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run_reg<T, RB>, NT, smem),
             "occupancy");
  per_sm = std::max(per_sm, 1);
  const uint64_t grid = std::min<uint64_t>(P.ntiles, (uint64_t)sm_count() * per_sm);
  k_run_reg<T, RB><<<(unsigned)grid, NT, smem, dev.stream>>>(
      reinterpret_cast<T *>(dev.state), reinterpret_cast<const RegParams *>(base),
      reinterpret_cast<const T *>(base + pool_off), reinterpret_cast<const T *>(base + bpool_off));
  check_launch("run kernel");
}

// ---------------------------------------------------------------------------
// Runs specialised to their op sequence.  The interpreting kernel above reads
// each op's kind and bits from shared memory and dispatches through a switch;
// the register array then has to sit in the same registers after every case,
// and the moves and dispatch cost more instructions than the arithmetic
// (MOV was the most frequent opcode of k_run_reg<float2,4>).  A run whose
// structure (ops, bits, matrix offsets, segments) recurs is compiled once by
// NVRTC into a kernel where every op is a straight call with its bits as
// template arguments; the matrices stay data.  Tiered: the interpreting kernel
// serves a structure's first execution, its second compiles (about a
// second), later ones reuse the module.  Without NVRTC (or on a compile
// error) the interpreting kernel keeps serving, on the GPU.

struct Nvrtc {
  using Prog = void *;
  int (*create)(Prog *, const char *, const char *, int, const char *const *, const char *const *) = nullptr;
  int (*compile)(Prog, int, const char *const *) = nullptr;
  int (*cubin_size)(Prog, size_t *) = nullptr;
  int (*cubin)(Prog, char *) = nullptr;
  int (*log_size)(Prog, size_t *) = nullptr;
  int (*log)(Prog, char *) = nullptr;
  int (*destroy)(Prog *) = nullptr;
  bool ok = false;
};

const Nvrtc &nvrtc() {
  static Nvrtc n = [] {
    Nvrtc r;
    void *h = dlopen("libnvrtc.so.13", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libnvrtc.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return r;
    auto sym = [&](auto &f, const char *name) { f = reinterpret_cast<std::remove_reference_t<decltype(f)>>(dlsym(h, name)); };
    sym(r.create, "nvrtcCreateProgram");
    sym(r.compile, "nvrtcCompileProgram");
    sym(r.cubin_size, "nvrtcGetCUBINSize");
    sym(r.cubin, "nvrtcGetCUBIN");
    sym(r.log_size, "nvrtcGetProgramLogSize");
    sym(r.log, "nvrtcGetProgramLog");
    sym(r.destroy, "nvrtcDestroyProgram");
    r.ok = r.create && r.compile && r.cubin_size && r.cubin && r.log_size && r.log && r.destroy;
    return r;
  }();
  return n;
}

struct DriverModule {
  CUresult (*load)(CUmodule *, const void *) = nullptr;
  CUresult (*get)(CUfunction *, CUmodule, const char *) = nullptr;
  CUresult (*attr)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                     void **, void **) = nullptr;
  bool ok = false;
};

const DriverModule &driver_module() {
  static DriverModule d = [] {
    DriverModule r;
    auto entry = [](const char *name) -> void * {
      void *ptr = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion(name, &ptr, 12000, cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess)
        ptr = nullptr;
      cudaGetLastError();
      return ptr;
    };
    r.load = reinterpret_cast<decltype(r.load)>(entry("cuModuleLoadData"));
    r.get = reinterpret_cast<decltype(r.get)>(entry("cuModuleGetFunction"));
    r.attr = reinterpret_cast<decltype(r.attr)>(entry("cuFuncSetAttribute"));
    r.launch = reinterpret_cast<decltype(r.launch)>(entry("cuLaunchKernel"));
    r.ok = r.load && r.get && r.attr && r.launch;
    return r;
  }();
  return d;
}

// Kernel arguments of a specialised run (by value).
struct JitArgs {
  uint64_t ntiles, nbind;
  uint64_t lowmask[24];
  int T[24];
  int state_bits;
};

const char *kJitKernel = R"GBQV(
struct JitArgs {
  uint64_t ntiles, nbind;
  uint64_t lowmask[24];
  int T[24];
  int state_bits;
};
extern "C" __global__ void __launch_bounds__(NT, NCTA)
    k_run_jit(TT *__restrict__ psi, const TR *__restrict__ pool, const TR *__restrict__ bpool, const JitArgs A) {
  constexpr uint32_t L = 1u << M, cmask = (1u << C) - 1, kPer = 16 / sizeof(TT);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31;
  TT *buf0 = reinterpret_cast<TT *>(smem_raw);
  TT *buf1 = buf0 + (NBUF == 2 ? L : 0);
  TR *mats = reinterpret_cast<TR *>(buf0 + NBUF * L);
  TR *bmats = mats + POOL;
  uint64_t *hi = reinterpret_cast<uint64_t *>(smem_raw + HIOFF);
  for (int i = tid; i < POOL; i += NT) mats[i] = pool[i];
  for (uint32_t h = tid; h < (1u << (M - C)); h += NT) {
    uint64_t a = 0;
    for (int j = C; j < M; ++j)
      if ((h >> (j - C)) & 1) a |= 1ULL << A.T[j];
    hi[h] = a;
  }
  __syncthreads();
  auto skip = [&](uint64_t gb) { return BOUND > 0 && (gb >> A.state_bits) >= A.nbind; };
  auto fetch = [&](uint64_t t, TT *buf) {
    const uint64_t gb = tile_base(t, A.lowmask, M);
    if (skip(gb)) return;
    for (uint32_t ch = tid; ch < L / kPer; ch += NT) {
      const uint32_t l = ch * kPer;
      cp_async16(buf + l, psi + (gb | hi[l >> C] | (l & cmask)));
    }
  };
  uint64_t t = blockIdx.x;
  if (NBUF == 2) {
    if (t < A.ntiles) fetch(t, buf0);
    cp_async_commit();
  }
  for (int k = 0; t < A.ntiles; t += gridDim.x, ++k) {
    TT *tile = (NBUF == 2 && (k & 1)) ? buf1 : buf0;
    const uint64_t gbase = tile_base(t, A.lowmask, M);
    if (NBUF == 2) {
      if (t + gridDim.x < A.ntiles) fetch(t + gridDim.x, (k & 1) ? buf0 : buf1);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      if (skip(gbase)) continue;
    } else {
      if (skip(gbase)) continue;
      fetch(t, tile);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    if (BOUND > 0) {
      const TR *src = bpool + (gbase >> A.state_bits) * (uint64_t)BOUND;
      for (int i = tid; i < BOUND; i += NT) bmats[i] = src[i];
      __syncthreads();
    }
    TR v[R];
    uint32_t tpart;
SEGMENTS
    __syncthreads();
    for (uint32_t l = tid; l < L; l += NT) psi[gbase | hi[l >> C] | (l & cmask)] = tile[l];
    __syncthreads();
  }
  cp_async_wait<0>();
}
)GBQV";

// The CUDA source of a run's specialised kernel; pairs: complex128 with the
// register amplitudes as float pairs (fcx), the memory stays double2.
std::string jit_source(bool dbl, bool pairs, const RegParams &P) {
  const int R = 1 << P.rb;
  std::ostringstream o;
  o << "typedef unsigned int uint32_t;\ntypedef unsigned long long uint64_t;\ntypedef unsigned short uint16_t;\n"
       "typedef unsigned char uint8_t;\ntypedef signed char int8_t;\ntypedef int int32_t;\n"
    << kFpairSrc << "\n" << kRunRegDevSrc << "\n";
  const size_t tsz = dbl ? 16 : 8;
  const JitShape sh = jit_shape(dbl);
  const size_t hioff =
      (tsz * ((size_t)sh.bufs * (1u << P.m) + (size_t)P.pool_elems + (size_t)P.bound_elems) + 7) & ~size_t(7);
  o << "typedef " << (dbl ? "double2" : "float2") << " TT;\n"
    << "typedef " << (pairs ? "fcx" : "TT") << " TR;\n"
    << "constexpr int NT = " << sh.threads << ", NCTA = " << sh.ctas << ", NBUF = " << sh.bufs << ";\n"
    << "constexpr int R = " << R << ", M = " << P.m << ", C = " << P.c << ", POOL = " << P.pool_elems
    << ", BOUND = " << P.bound_elems << ";\nconstexpr uint32_t HIOFF = " << hioff << ";\n";
  std::ostringstream seg;
  auto tpart_expr = [&](const RegSeg &S) {
    std::ostringstream e;
    for (int q = 0; q < sh.tbits; ++q) e << (q ? " | " : "") << "((((uint32_t)tid >> " << q << ") & 1u) << " << (int)S.tb[q] << ")";
    return e.str();
  };
  for (int si = 0; si < P.nsegs; ++si) {
    const RegSeg &S = P.segs[si];
    seg << "    {\n";
    if (si > 0) {
      const RegSeg &Sp = P.segs[si - 1];
      seg << "      __syncthreads();\n";
      for (int i = 0; i < R; ++i) seg << "      tile[tpart | " << Sp.rp[i] << "u] = from_reg(v[" << i << "], TT());\n";
      seg << "      __syncthreads();\n";
    }
    seg << "      tpart = " << tpart_expr(S) << ";\n";
    for (int i = 0; i < R; ++i)
      seg << "      v[" << i << "] = " << (pairs ? "to_reg_pair" : "to_reg") << "(tile[tpart | " << S.rp[i] << "u]);\n";
    for (int oi = S.first; oi < S.first + S.count; ++oi) {
      const RegOp &op = P.ops[oi];
      const std::string mat = std::string(op.bound ? "bmats" : "mats") + " + " + std::to_string(op.mat_off);
      const std::string tcond = "((((uint32_t)tid) & " + std::to_string(op.ctm) + "u) == " + std::to_string(op.ctm) + "u)";
      switch (op.kind) {
        case RK_DENSE1: seg << "      reg_dense1<TR, R, " << op.a << ">(v, " << mat << ");\n"; break;
        case RK_DENSE1_REAL: seg << "      reg_dense1_real<TR, R, " << op.a << ">(v, " << mat << ");\n"; break;
        case RK_DIAG1: seg << "      reg_diag1<TR, R, " << op.a << ">(v, " << mat << ");\n"; break;
        case RK_MCX: seg << "      reg_mcx<TR, R, " << op.a << ">(v, " << tcond << ", " << op.crm << "u);\n"; break;
        case RK_DENSE2: seg << "      reg_dense2<TR, R, " << op.a << ", " << op.b << ">(v, " << mat << ");\n"; break;
        case RK_DENSE1_LANE: seg << "      lane_dense1<TR, R>(v, " << mat << ", " << op.a << ", lane);\n"; break;
        case RK_DENSE1_REAL_LANE: seg << "      lane_dense1_real<TR, R>(v, " << mat << ", " << op.a << ", lane);\n"; break;
        case RK_MCX_LANE: seg << "      lane_mcx<TR, R>(v, " << op.a << ", " << tcond << ", " << op.crm << "u);\n"; break;
        case RK_DIAG_T:
        case RK_DIAG: {
          std::ostringstream td;
          td << "0u";
          for (int j = 0; j < op.k; ++j)
            if (op.dtpos[j] >= 0) td << " | ((((uint32_t)tid >> " << (int)op.dtpos[j] << ") & 1u) << " << j << ")";
          if (op.kind == RK_DIAG_T) {
            seg << "      thread_diag<TR, R>(v, " << mat << ", " << td.str() << ");\n";
          } else {
            seg << "      {\n        const uint32_t td = " << td.str() << ";\n        const TR *dm = " << mat << ";\n";
            for (int i = 0; i < R; ++i) seg << "        v[" << i << "] = cmul(v[" << i << "], dm[td | " << (int)op.div[i] << "u]);\n";
            seg << "      }\n";
          }
          break;
        }
        default: throw Error(1, "run op kind without a specialised form");
      }
    }
    seg << "    }\n";
  }
  const RegSeg &Sl = P.segs[P.nsegs - 1];
  seg << "    __syncthreads();\n";
  for (int i = 0; i < R; ++i) seg << "    tile[tpart | " << Sl.rp[i] << "u] = from_reg(v[" << i << "], TT());\n";
  std::string k = kJitKernel;
  const size_t at = k.find("SEGMENTS\n");
  k.replace(at, 9, seg.str());
  o << k;
  return o.str();
}

// process-wide counts: specialised kernels compiled, and launched
std::atomic<uint64_t> g_jit_compiled{0}, g_jit_launched{0};

struct JitEntry {
  int uses = 0;
  bool failed = false;
  CUfunction fn = nullptr;
  size_t smem_attr = 0;
};

std::mutex &jit_mutex() {
  static std::mutex m;
  return m;
}
std::unordered_map<std::string, JitEntry> &jit_cache() {
  static std::unordered_map<std::string, JitEntry> c;
  return c;
}

// NVRTC: the source to a cubin for sm_103a; false (with the compiler's log)
// on failure.
bool jit_cubin(const std::string &src, std::vector<char> &cubin, std::string &log) {
  const Nvrtc &n = nvrtc();
  if (!n.ok) {
    log = "NVRTC is not available";
    return false;
  }
  Nvrtc::Prog prog = nullptr;
  if (n.create(&prog, src.c_str(), "gbqv_run_jit.cu", 0, nullptr, nullptr) != 0) {
    log = "nvrtcCreateProgram failed";
    return false;
  }
  const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17"};
  const int rc = n.compile(prog, 2, opts);
  size_t ls = 0;
  n.log_size(prog, &ls);
  log.assign(ls, '\0');
  if (ls) n.log(prog, &log[0]);
  if (rc == 0) {
    size_t cs = 0;
    n.cubin_size(prog, &cs);
    cubin.resize(cs);
    n.cubin(prog, cubin.data());
  }
  n.destroy(&prog);
  return rc == 0 && !cubin.empty();
}

// Compile and load: the kernel, or null (log says why).
CUfunction jit_compile(const std::string &src, std::string &log) {
  const DriverModule &d = driver_module();
  if (!d.ok) {
    log = "the driver's module entry points are not available";
    return nullptr;
  }
  std::vector<char> cubin;
  if (!jit_cubin(src, cubin, log)) return nullptr;
  CUmodule mod = nullptr;  // kept loaded for the life of the process (the cache holds its function)
  CUfunction fn = nullptr;
  if (d.load(&mod, cubin.data()) != CUDA_SUCCESS || d.get(&fn, mod, "k_run_jit") != CUDA_SUCCESS) {
    log += "\nmodule load failed";
    return nullptr;
  }
  return fn;
}

// The specialised kernel for P, or null (interpreting kernel) under the
// tiering rule or when compiling fails.
CUfunction jit_kernel(const Device &dev, bool dbl, bool pairs, const RegParams &P) {
  if (dev.run_jit == 0) return nullptr;
  const std::string src = jit_source(dbl, pairs, P);
  std::lock_guard<std::mutex> g(jit_mutex());
  JitEntry &e = jit_cache()[src];
  ++e.uses;
  if (e.fn || e.failed) return e.fn;
  if (dev.run_jit == 1 && e.uses < 2) return nullptr;
  std::string log;
  e.fn = jit_compile(src, log);
  e.failed = !e.fn;
  if (e.fn) ++g_jit_compiled;
  return e.fn;
}

// A synthetic run (every op kind, three segments) compiled with NVRTC
// without loading it: the host-side check of the source generator.
int jit_compile_check(bool dbl, std::string &log) {
  auto P = std::make_unique<RegParams>();
  std::memset(P.get(), 0, sizeof(RegParams));
  P->rb = dbl ? 3 : 5;
  P->m = P->rb + reg_tbits(dbl);
  P->c = 4;
  P->nsegs = 3;
  const int kinds[] = {RK_DENSE1, RK_DENSE1_REAL, RK_DENSE1_LANE, RK_DENSE2, RK_DIAG1, RK_DIAG,
                       RK_MCX,    RK_MCX_LANE,    RK_DIAG_T,      RK_DENSE1_REAL_LANE};
  P->nops = 10;
  for (int o = 0; o < P->nops; ++o) {
    RegOp &op = P->ops[o];
    op.kind = kinds[o];
    op.k = op.kind == RK_DENSE2 || op.kind == RK_DIAG || op.kind == RK_DIAG_T ? 2 : 1;
    op.a = op.kind == RK_DENSE2 ? 0 : 1;
    op.b = 2;
    op.bound = o & 1;
    op.mat_off = 4 * o;
    op.ctm = op.kind == RK_MCX || op.kind == RK_MCX_LANE ? 0x20u : 0u;
    op.crm = op.kind == RK_MCX ? 0x1u : 0u;
    op.dtpos[0] = op.kind == RK_DIAG ? -1 : 5;
    op.dtpos[1] = 6;
    for (int i = 0; i < 32; ++i) op.div[i] = (uint8_t)(i & 1);
  }
  for (int sgi = 0; sgi < 3; ++sgi) {
    RegSeg &S = P->segs[sgi];
    S.first = sgi == 0 ? 0 : sgi == 1 ? 4 : 7;
    S.count = sgi == 0 ? 4 : 3;
    for (int i = 0; i < (1 << P->rb); ++i) S.rp[i] = (uint16_t)(i << sgi);
    for (int q = 0; q < reg_tbits(dbl); ++q) S.tb[q] = (uint8_t)(q < sgi ? q : q + P->rb);
  }
  P->pool_elems = 40;
  P->bound_elems = 40;
  std::vector<char> cubin;
  return jit_cubin(jit_source(dbl, dbl, *P), cubin, log) ? 0 : 1;
}

template <typename T, int RB>
bool launch_reg_jit(Device &dev, RegParams &P, const std::vector<T> &pool_in, const std::vector<T> &bpool_in) {
  // complex128 runs hold their registers as float pairs unless native FP64
  // arithmetic was asked for (gbqv_set_tensor_c128(h, 0)); their matrices are
  // uploaded as pairs too (same 16 bytes per entry)
  const bool pairs = sizeof(T) == 16 && dev.tensor_c128 != 0;
  CUfunction fn = jit_kernel(dev, sizeof(T) == 16, pairs, P);
  if (!fn) return false;
  std::vector<T> pool_p, bpool_p;
  if (pairs) {
    auto split = [](const std::vector<T> &in, std::vector<T> &out) {
      out.resize(in.size());
      for (size_t i = 0; i < in.size(); ++i) {
        const double2 z = reinterpret_cast<const double2 &>(in[i]);
        float f[4];
        const double v[2] = {z.x, z.y};
        for (int c = 0; c < 2; ++c) {
          f[2 * c] = (float)v[c];
          f[2 * c + 1] = (float)(v[c] - (double)f[2 * c]);
        }
        std::memcpy(&out[i], f, sizeof(f));
      }
    };
    split(pool_in, pool_p);
    split(bpool_in, bpool_p);
  }
  const std::vector<T> &pool = pairs ? pool_p : pool_in, &bpool = pairs ? bpool_p : bpool_in;
  const size_t poolb = pool.size() * sizeof(T), bpoolb = bpool.size() * sizeof(T);
  const size_t bpool_off = (poolb + 255) & ~size_t(255);
  grow(dev.mat, dev.mat_cap, bpool_off + bpoolb + 256);
  char *base = reinterpret_cast<char *>(dev.mat);
  if (poolb) cuda_check(cudaMemcpyAsync(base, pool.data(), poolb, cudaMemcpyHostToDevice, dev.stream), "run upload");
  if (bpoolb)
    cuda_check(cudaMemcpyAsync(base + bpool_off, bpool.data(), bpoolb, cudaMemcpyHostToDevice, dev.stream),
               "run upload");
  const JitShape sh = jit_shape(sizeof(T) == 16);
  size_t smem = (sizeof(T) * ((size_t)sh.bufs * (1u << P.m) + pool.size() + (size_t)P.bound_elems) + 7) & ~size_t(7);
  smem += sizeof(uint64_t) * (1u << (P.m - P.c));
  const DriverModule &d = driver_module();
  {
    std::lock_guard<std::mutex> g(jit_mutex());
    // one attribute per function, raised to the largest size it has launched with
    JitEntry *e = nullptr;
    for (auto &kv : jit_cache())
      if (kv.second.fn == fn) e = &kv.second;
    if (e && e->smem_attr < smem) {
      if (d.attr(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem) != CUDA_SUCCESS)
        throw Error(3, "run kernel attribute");
      e->smem_attr = smem;
    }
  }
  JitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ntiles = P.ntiles;
  a.nbind = P.nbind;
  a.state_bits = P.state_bits;
  for (int j = 0; j < P.m; ++j) {
    a.lowmask[j] = P.tile_lowmask[j];
    a.T[j] = P.T[j];
  }
  T *psi = reinterpret_cast<T *>(dev.state);
  const T *pp = reinterpret_cast<const T *>(base), *bp = reinterpret_cast<const T *>(base + bpool_off);
  void *args[] = {&psi, &pp, &bp, &a};
  const uint64_t grid = std::min<uint64_t>(P.ntiles, (uint64_t)sm_count() * sh.ctas);
  if (d.launch(fn, (unsigned)grid, 1, 1, (unsigned)sh.threads, 1, 1, (unsigned)smem, dev.stream, args, nullptr) !=
      CUDA_SUCCESS)
    throw Error(3, "specialised run kernel launch failed");
  check_launch("specialised run kernel");
  ++g_jit_launched;
  return true;
}

// Register bits for a new segment: `need` plus the tile bits whose next use
// as a dense / X-target bit comes soonest (ties: higher bits first, so low
// bits stay thread bits and shared-memory accesses stay contiguous).
std::vector<int> choose_regs(const std::vector<int> &need, int rb, int m,
                             const std::vector<std::vector<int>> &dense_bits, size_t from) {
  std::vector<int> regs = need;
  std::vector<std::pair<size_t, int>> cand;
  for (int b = 0; b < m; ++b) {
    if (std::find(regs.begin(), regs.end(), b) != regs.end()) continue;
    size_t next = SIZE_MAX;
    for (size_t o = from; o < dense_bits.size() && next == SIZE_MAX; ++o)
      if (std::find(dense_bits[o].begin(), dense_bits[o].end(), b) != dense_bits[o].end()) next = o;
    cand.push_back({next, -b});
  }
  std::sort(cand.begin(), cand.end());
  for (auto &cb : cand) {
    if ((int)regs.size() >= rb) break;
    regs.push_back(-cb.second);
  }
  return regs;
}

}  // namespace

bool run_jit_available() { return nvrtc().ok; }
void run_jit_counts(uint64_t &compiled, uint64_t &launched) {
  compiled = g_jit_compiled.load();
  launched = g_jit_launched.load();
}
int run_jit_compile_check(bool dbl, std::string &log) { return jit_compile_check(dbl, log); }

// A run on the register-tile kernel; false when the run has an op it does
// not take (a dense op on more than 2 qubits) or the tile is too small.
bool launch_run_reg(Device &dev, const std::vector<const RunOp *> &ops, const std::vector<int> &tile_qubits, int c,
                    const RunBound *bound) {
  const int m = (int)tile_qubits.size();
  const int tbits = reg_tbits(dev.dbl);
  const int rb = m - tbits;
  const int maxrb = dev.dbl ? 3 : 5;
  if (rb < 2 || rb > maxrb || (int)ops.size() > kRegMaxOps || ops.empty()) return false;
  for (const RunOp *op : ops) {
    if (op->kind == 0 && op->qubits.size() > 2) return false;
    if (op->qubits.size() > 5) return false;
  }
  const int n = dev.n;
  std::vector<int> local(n, -1);
  for (int j = 0; j < m; ++j) local[tile_qubits[j]] = j;
  // per op: local qubits, and the bits it needs as register bits (dense qubits, X target)
  std::vector<std::vector<int>> lq(ops.size()), dense_bits(ops.size());
  for (size_t o = 0; o < ops.size(); ++o) {
    for (auto q : ops[o]->qubits) lq[o].push_back(local[q]);
    if (ops[o]->kind == 0) dense_bits[o] = lq[o];
    if (ops[o]->kind == 2) dense_bits[o] = {lq[o].back()};
  }
  auto thread_bits = [&](const std::vector<int> &regs) {
    std::vector<int> tb;
    for (int b = 0; b < m; ++b)
      if (std::find(regs.begin(), regs.end(), b) == regs.end()) tb.push_back(b);
    return tb;  // ascending: thread-index bit q holds tile bit tb[q]
  };
  // segments: one set of register bits each
  std::vector<std::vector<int>> seg_regs;
  std::vector<std::vector<size_t>> seg_ops;
  std::vector<int> regs = choose_regs(dense_bits[0], rb, m, dense_bits, 0);
  seg_regs.push_back(regs);
  seg_ops.push_back({});
  for (size_t o = 0; o < ops.size(); ++o) {
    const std::vector<int> tb = thread_bits(regs);
    bool ok = true;
    for (int b : dense_bits[o]) {
      const bool in_reg = std::find(regs.begin(), regs.end(), b) != regs.end();
      const int tpos = (int)(std::find(tb.begin(), tb.end(), b) - tb.begin());
      const bool lane_ok = dense_bits[o].size() == 1 && tpos < 5;  // 1-qubit dense / X target on a lane bit
      if (!in_reg && !lane_ok) ok = false;
    }
    if (!ok) {
      regs = choose_regs(dense_bits[o], rb, m, dense_bits, o + 1);
      seg_regs.push_back(regs);
      seg_ops.push_back({});
    }
    seg_ops.back().push_back(o);
  }
  auto P = std::make_unique<RegParams>();
  std::memset(P.get(), 0, sizeof(RegParams));
  P->m = m;
  P->c = c;
  P->rb = rb;
  P->nops = (int)ops.size();
  P->nsegs = (int)seg_regs.size();
  P->ntiles = 1ULL << (n - m);
  for (int j = 0; j < m; ++j) {
    P->T[j] = tile_qubits[j];
    P->tile_lowmask[j] = (1ULL << tile_qubits[j]) - 1;
  }
  using HostMat = std::vector<cd>;
  std::vector<HostMat> op_mat(ops.size()), op_bmat(ops.size());
  int bound_elems = 0, pool_elems = 0;
  size_t oi = 0;
  for (size_t s = 0; s < seg_regs.size(); ++s) {
    const std::vector<int> &rg = seg_regs[s];
    const std::vector<int> tb = thread_bits(rg);
    RegSeg &S = P->segs[s];
    S.first = (int)oi;
    S.count = (int)seg_ops[s].size();
    for (int i = 0; i < (1 << rb); ++i) {
      uint32_t a = 0;
      for (int p = 0; p < rb; ++p)
        if ((i >> p) & 1) a |= 1u << rg[p];
      S.rp[i] = (uint16_t)a;
    }
    for (int q = 0; q < tbits; ++q) S.tb[q] = (uint8_t)tb[q];
    auto rpos = [&](int b) { return (int)(std::find(rg.begin(), rg.end(), b) - rg.begin()); };
    auto tpos = [&](int b) { return (int)(std::find(tb.begin(), tb.end(), b) - tb.begin()); };
    for (size_t o : seg_ops[s]) {
      const RunOp &op = *ops[o];
      RegOp &d = P->ops[oi++];
      const int k = (int)lq[o].size();
      d.k = k;
      d.bound = !op.bmat.empty();
      op_mat[o] = op.mat;
      op_bmat[o] = op.bmat;
      if (op.kind == 0 && k == 1) {
        const int b = lq[o][0];
        bool real = true;
        for (const cd &z : op.mat) real &= z.imag() == 0.0;
        for (const cd &z : op.bmat) real &= z.imag() == 0.0;
        if (rpos(b) < rb) {
          d.kind = real ? RK_DENSE1_REAL : RK_DENSE1;
          d.a = rpos(b);
        } else {
          d.kind = real ? RK_DENSE1_REAL_LANE : RK_DENSE1_LANE;
          d.a = tpos(b);
        }
      } else if (op.kind == 0) {  // k == 2
        int a = rpos(lq[o][0]), b = rpos(lq[o][1]);
        if (a > b) {
          std::swap(a, b);
          op_mat[o] = swap_bits2(op.mat.data());
          if (!op.bmat.empty()) {
            HostMat bm(op.bmat.size());
            for (size_t j = 0; j < op.bmat.size() / 16; ++j) {
              HostMat t = swap_bits2(op.bmat.data() + 16 * j);
              std::copy(t.begin(), t.end(), bm.begin() + 16 * j);
            }
            op_bmat[o] = bm;
          }
        }
        d.kind = RK_DENSE2;
        d.a = a;
        d.b = b;
      } else if (op.kind == 1) {
        if (k == 1 && rpos(lq[o][0]) < rb) {
          d.kind = RK_DIAG1;
          d.a = rpos(lq[o][0]);
        } else {
          bool thread_only = true;
          for (int j = 0; j < k; ++j) thread_only &= rpos(lq[o][j]) >= rb;
          d.kind = thread_only ? RK_DIAG_T : RK_DIAG;
          for (int j = 0; j < k; ++j) d.dtpos[j] = (int8_t)(rpos(lq[o][j]) < rb ? -1 : tpos(lq[o][j]));
          for (int i = 0; i < (1 << rb); ++i) {
            uint32_t x = 0;
            for (int j = 0; j < k; ++j)
              if (rpos(lq[o][j]) < rb) x |= (uint32_t)((i >> rpos(lq[o][j])) & 1) << j;
            d.div[i] = (uint8_t)x;
          }
        }
      } else {  // multi-controlled X
        const int tq = lq[o].back();
        if (rpos(tq) < rb) {
          d.kind = RK_MCX;
          d.a = rpos(tq);
        } else {
          d.kind = RK_MCX_LANE;
          d.a = tpos(tq);
        }
        for (int j = 0; j + 1 < k; ++j) {
          const int b = lq[o][j];
          if (rpos(b) < rb)
            d.crm |= 1u << rpos(b);
          else
            d.ctm |= 1u << tpos(b);
        }
      }
      if (op.kind != 2) {
        d.mat_off = d.bound ? bound_elems : pool_elems;
        (d.bound ? bound_elems : pool_elems) += (int)op.mat.size();
      }
    }
  }
  P->pool_elems = pool_elems;
  P->bound_elems = bound_elems;
  // matrices in op order, as the offsets above
  auto fill = [&](auto tag) {
    using T = decltype(tag);
    std::vector<T> pool, bpool;
    std::vector<size_t> order;
    for (size_t s = 0; s < seg_ops.size(); ++s)
      for (size_t o : seg_ops[s]) order.push_back(o);
    for (size_t o : order)
      if (ops[o]->kind != 2 && op_bmat[o].empty())
        for (const cd &z : op_mat[o]) pool.push_back(to_dev<T>(z));
    if (bound_elems) {
      P->state_bits = bound->state_bits;
      P->nbind = bound->count;
      bpool.reserve((size_t)bound_elems * bound->count);
      for (uint64_t j = 0; j < bound->count; ++j)
        for (size_t o : order) {
          if (op_bmat[o].empty()) continue;
          const size_t msz = op_mat[o].size();
          if (op_bmat[o].size() < (bound->first + j + 1) * msz) throw Error(1, "bound run op has too few bindings");
          const cd *src = op_bmat[o].data() + (bound->first + j) * msz;
          for (size_t e = 0; e < msz; ++e) bpool.push_back(to_dev<T>(src[e]));
        }
    }
    switch (rb) {
      case 2:
        if (!launch_reg_jit<T, 2>(dev, *P, pool, bpool)) launch_reg_t<T, 2>(dev, *P, pool, bpool);
        break;
      case 3:
        if (!launch_reg_jit<T, 3>(dev, *P, pool, bpool)) launch_reg_t<T, 3>(dev, *P, pool, bpool);
        break;
      case 4:
        if constexpr (sizeof(T) == 8)
          if (!launch_reg_jit<T, 4>(dev, *P, pool, bpool)) launch_reg_t<T, 4>(dev, *P, pool, bpool);
        break;
      case 5:
        if constexpr (sizeof(T) == 8)
          if (!launch_reg_jit<T, 5>(dev, *P, pool, bpool)) launch_reg_t<T, 5>(dev, *P, pool, bpool);
        break;
      default: break;
    }
  };
  if (bound_elems && !bound) throw Error(1, "bound run op outside a bound run");
  if (dev.dbl)
    fill(double2{});
  else
    fill(float2{});
  return true;
}

}  // namespace gbqv
