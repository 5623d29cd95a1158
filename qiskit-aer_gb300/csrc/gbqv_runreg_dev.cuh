// gbqv_runreg_dev.cuh — device arithmetic of the register-tile run kernel:
// complex helpers, the ops on the register-held amplitudes v[0..R) of a
// thread (1-2 qubit dense ops, diagonals, multi-controlled X), the same on
// lane bits through warp shuffles, and the asynchronous tile copies.
//
// Shared by two compilers: gbqv_runreg.cu includes it (inside its namespace)
// for the interpreting kernel k_run_reg, and gbqv_runjit.cpp hands its text to
// the runtime compiler (NVRTC) for the kernels specialised to one run's op
// sequence.  It therefore includes only gbqv_fpair.cuh (which NVRTC receives
// as text ahead of this one) and uses only builtin vector types and the
// fixed-width integer names the includer provides.
#ifndef GBQV_RUNREG_DEV_CUH
#define GBQV_RUNREG_DEV_CUH

#ifndef __CUDACC_RTC__
#include "gbqv_fpair.cuh"
#endif

// register form of a memory amplitude and back (the identity except for
// float-pair registers)
__device__ __forceinline__ float2 to_reg(float2 a) { return a; }
__device__ __forceinline__ double2 to_reg(double2 a) { return a; }
__device__ __forceinline__ float2 from_reg(float2 a, float2) { return a; }
__device__ __forceinline__ double2 from_reg(double2 a, double2) { return a; }
__device__ __forceinline__ float shfl_scalar(float v, int mask) { return __shfl_xor_sync(0xffffffffu, v, mask); }
__device__ __forceinline__ double shfl_scalar(double v, int mask) { return __shfl_xor_sync(0xffffffffu, v, mask); }
__device__ __forceinline__ fpair shfl_scalar(fpair v, int mask) {
  return fpair(__shfl_xor_sync(0xffffffffu, v.hi, mask), __shfl_xor_sync(0xffffffffu, v.lo, mask));
}

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
  T r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename T>
__device__ __forceinline__ void cfma(T &acc, T a, T b) {
  acc.x = rfma(a.x, b.x, acc.x);
  acc.x = rfma(-a.y, b.y, acc.x);
  acc.y = rfma(a.x, b.y, acc.y);
  acc.y = rfma(a.y, b.x, acc.y);
}
// m0 * a0 + m1 * a1, and sum_c m[stride c] * x[c]: multiply-add chains at
// complex64 / complex128 (the order of the shared-memory run kernel), one
// compensated dot product per real part for float pairs (gbqv_fpair.cuh)
template <typename T>
__device__ __forceinline__ T cdot2(T m0, T a0, T m1, T a1) {
  T r;
  r.x = 0;
  r.y = 0;
  cfma(r, m0, a0);
  cfma(r, m1, a1);
  return r;
}
template <typename T>
__device__ __forceinline__ T cdot4(const T *m, int stride, const T (&x)[4]) {
  T r;
  r.x = 0;
  r.y = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) cfma(r, m[stride * c], x[c]);
  return r;
}

template <typename T>
__device__ __forceinline__ T czero() {
  T z;
  z.x = 0;
  z.y = 0;
  return z;
}
template <typename T>
__device__ __forceinline__ T shfl_x(T v, int mask) {
  T r;
  r.x = shfl_scalar(v.x, mask);
  r.y = shfl_scalar(v.y, mask);
  return r;
}

// ---- ops on the register-held amplitudes v[0..R) ----
template <typename T, int R, int J>
__device__ __forceinline__ void reg_dense1(T (&v)[R], const T *m) {
  const T m00 = m[0], m10 = m[1], m01 = m[2], m11 = m[3];
#pragma unroll
  for (int p = 0; p < R / 2; ++p) {
    const int i0 = ((p >> J) << (J + 1)) | (p & ((1 << J) - 1)), i1 = i0 | (1 << J);
    const T a0 = v[i0], a1 = v[i1];
    v[i0] = cdot2(m00, a0, m01, a1);
    v[i1] = cdot2(m10, a0, m11, a1);
  }
}
// real matrix: the complex FMAs above with every imaginary matrix term zero
template <typename T, int R, int J>
__device__ __forceinline__ void reg_dense1_real(T (&v)[R], const T *m) {
  const auto m00 = m[0].x, m10 = m[1].x, m01 = m[2].x, m11 = m[3].x;
#pragma unroll
  for (int p = 0; p < R / 2; ++p) {
    const int i0 = ((p >> J) << (J + 1)) | (p & ((1 << J) - 1)), i1 = i0 | (1 << J);
    const T a0 = v[i0], a1 = v[i1];
    T r0, r1;
    r0.x = rfma(m01, a1.x, m00 * a0.x);
    r0.y = rfma(m01, a1.y, m00 * a0.y);
    r1.x = rfma(m11, a1.x, m10 * a0.x);
    r1.y = rfma(m11, a1.y, m10 * a0.y);
    v[i0] = r0;
    v[i1] = r1;
  }
}
template <typename T, int R, int J>
__device__ __forceinline__ void reg_diag1(T (&v)[R], const T *d) {
  const T d0 = d[0], d1 = d[1];
#pragma unroll
  for (int i = 0; i < R; ++i) v[i] = cmul(v[i], ((i >> J) & 1) ? d1 : d0);
}
template <typename T, int R, int J>
__device__ __forceinline__ void reg_mcx(T (&v)[R], bool tcond, uint32_t crm) {
#pragma unroll
  for (int p = 0; p < R / 2; ++p) {
    const int i0 = ((p >> J) << (J + 1)) | (p & ((1 << J) - 1)), i1 = i0 | (1 << J);
    const bool sw = tcond && (((uint32_t)i0 & crm) == crm);
    const T a0 = v[i0], a1 = v[i1];
    v[i0] = sw ? a1 : a0;
    v[i1] = sw ? a0 : a1;
  }
}
template <typename T, int R, int A, int B>
__device__ __forceinline__ void reg_dense2(T (&v)[R], const T *m) {
#pragma unroll
  for (int q = 0; q < R / 4; ++q) {
    // insert zeros at A then B (A < B)
    int i = ((q >> A) << (A + 1)) | (q & ((1 << A) - 1));
    i = ((i >> B) << (B + 1)) | (i & ((1 << B) - 1));
    const int idx[4] = {i, i | (1 << A), i | (1 << B), i | (1 << A) | (1 << B)};
    T x[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = v[idx[c]];
#pragma unroll
    for (int r = 0; r < 4; ++r) v[idx[r]] = cdot4(m + r, 4, x);
  }
}

// ---- ops on lane bits (warp shuffles) and on thread bits ----
// 1-qubit dense op on lane bit a: this lane holds row `bit` of the pair, new
// = m[bit][bit] * own + m[bit][1-bit] * partner's
template <typename T, int R>
__device__ __forceinline__ void lane_dense1(T (&v)[R], const T *mat, int a, int lane) {
  const int bit = (lane >> a) & 1;
  const T ms = bit ? mat[3] : mat[0], mo = bit ? mat[1] : mat[2];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const T o = shfl_x(v[i], 1 << a);
    v[i] = cdot2(ms, v[i], mo, o);
  }
}
template <typename T, int R>
__device__ __forceinline__ void lane_dense1_real(T (&v)[R], const T *mat, int a, int lane) {
  const int bit = (lane >> a) & 1;
  const auto ms = bit ? mat[3].x : mat[0].x, mo = bit ? mat[1].x : mat[2].x;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const T o = shfl_x(v[i], 1 << a);
    T r;
    r.x = rfma(mo, o.x, ms * v[i].x);
    r.y = rfma(mo, o.y, ms * v[i].y);
    v[i] = r;
  }
}
// multi-controlled X with its target on lane bit a
template <typename T, int R>
__device__ __forceinline__ void lane_mcx(T (&v)[R], int a, bool tcond, uint32_t crm) {
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const T o = shfl_x(v[i], 1 << a);
    if (tcond && (((uint32_t)i & crm) == crm)) v[i] = o;
  }
}
// diagonal whose qubits are all thread bits: one factor per thread
template <typename T, int R>
__device__ __forceinline__ void thread_diag(T (&v)[R], const T *mat, uint32_t td) {
  const T d = mat[td];
#pragma unroll
  for (int i = 0; i < R; ++i) v[i] = cmul(v[i], d);
}

// 16-byte asynchronous global -> shared copies (LDGSTS): the next tile
// streams in while the current one is computed.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ uint64_t tile_base(uint64_t t, const uint64_t *lowmask, int m) {
  for (int j = 0; j < m; ++j) {
    const uint64_t msk = lowmask[j];
    t = ((t & ~msk) << 1) | (t & msk);
  }
  return t;
}

#endif  // GBQV_RUNREG_DEV_CUH
