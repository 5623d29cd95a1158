// gbqv_fpair.cuh — float pairs: ~48-bit real arithmetic on the FP32 pipe,
// for complex128 work that would otherwise run on GB300's 1.2 TFLOP/s FP64
// pipe (the specialised register-tile runs, gbqv_runreg.cu, and the adjoint
// sweep, gbqv_kernels.cu).  Includes nothing; also handed to NVRTC as text.
#ifndef GBQV_FPAIR_CUH
#define GBQV_FPAIR_CUH

// ---- float pairs: ~48-bit real arithmetic on the FP32 pipe ----
// A complex128 run spends 8 FP64 operations per amplitude and 1-qubit op, and
// FP64 runs at 1.2 TFLOP/s on GB300.  In its specialised kernel the register
// amplitudes are held as pairs of floats (hi + lo, non-overlapping) with
// error-free products (FMA) and sums (two-sum), ~48 significant bits: error
// about 2^-47 of the operands' magnitude per operation, far inside the 1e-12
// parity tolerance.  The tile in shared memory and the state in HBM stay
// complex128.
struct fpair {
  float hi, lo;
  __device__ __forceinline__ fpair() {}
  __device__ __forceinline__ fpair(float h) : hi(h), lo(0.0f) {}
  __device__ __forceinline__ fpair(float h, float l) : hi(h), lo(l) {}
};
__device__ __forceinline__ fpair fp_fast2sum(float a, float b) {
  const float s = a + b;
  return fpair(s, b - (s - a));
}
__device__ __forceinline__ fpair operator+(fpair a, fpair b) {
  const float s = a.hi + b.hi, bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  return fp_fast2sum(s, e + a.lo + b.lo);
}
__device__ __forceinline__ fpair operator-(fpair a) { return fpair(-a.hi, -a.lo); }
__device__ __forceinline__ fpair operator-(fpair a, fpair b) { return a + (-b); }
__device__ __forceinline__ fpair operator*(fpair a, fpair b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fp_fast2sum(p, e);
}
// a * b + c for every register scalar type (the templates below call rfma)
__device__ __forceinline__ float rfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ fpair rfma(fpair a, fpair b, fpair c) { return a * b + c; }

// Sums of products with one normalisation at the end: the compensated dot
// product (Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26 (2005), Dot2) on
// the pairs' high parts, each product's low terms (a.hi b.lo + a.lo b.hi,
// as in operator*) and the sums' rounding errors gathered in one float.  The
// error is about 2^-46 of the sum of |products|; a complex multiply-add
// chain over four products costs 46 FP32 operations per real result
// against 72 with operator* and operator+.
struct fp_dot {
  float s, e;
};
__device__ __forceinline__ fp_dot fp_dot_first(fpair a, fpair b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  fp_dot d;
  d.s = p;
  d.e = e;
  return d;
}
__device__ __forceinline__ void fp_dot_add(fp_dot &d, fpair a, fpair b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = d.s + p, bb = s - d.s;
  d.e += ((d.s - (s - bb)) + (p - bb)) + e;
  d.s = s;
}
__device__ __forceinline__ fpair fp_dot_done(fp_dot d) {  // two-sum: the errors may outweigh a cancelled sum
  const float s = d.s + d.e, bb = s - d.s;
  return fpair(s, (d.s - (s - bb)) + (d.e - bb));
}

// double -> pair: hi = the significand cut to 24 bits, lo = the remaining 29
// bits rounded to a float (integer code, no FP64 operation); |d| below
// 2^-126 flushes to 0
__device__ __forceinline__ fpair fpair_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned h = (unsigned)(b >> 32), l = (unsigned)b;
  const int e = (int)((h >> 20) & 0x7ffu);
  if (e < 897) return fpair(0.0f, 0.0f);
  const unsigned sgn = h & 0x80000000u;
  const float hi = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
  float lo = __uint2float_rn(l & 0x1fffffffu);  // the remainder r, worth r * 2^(e - 1075)
  lo = e >= 949 ? lo * __uint_as_float((unsigned)(e - 948) << 23) : 0.0f;
  return fpair(hi, sgn ? -lo : lo);
}
// float -> double, exactly, in integer code (zero and subnormal floats give 0)
__device__ __forceinline__ double float_to_double_bits(float f) {
  const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xffu;
  if (e == 0) return 0.0;
  return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
}
// pair -> double: one FP64 add, rounded to nearest
__device__ __forceinline__ double fpair_to_double(fpair p) {
  return float_to_double_bits(p.hi) + float_to_double_bits(p.lo);
}
struct fcx {
  fpair x, y;
};

// m0 * a0 + m1 * a1 (complex) as one compensated dot product per real part
__device__ __forceinline__ fcx cdot2(fcx m0, fcx a0, fcx m1, fcx a1) {
  fp_dot re = fp_dot_first(m0.x, a0.x), im = fp_dot_first(m0.x, a0.y);
  fp_dot_add(re, -m0.y, a0.y);
  fp_dot_add(im, m0.y, a0.x);
  fp_dot_add(re, m1.x, a1.x);
  fp_dot_add(im, m1.x, a1.y);
  fp_dot_add(re, -m1.y, a1.y);
  fp_dot_add(im, m1.y, a1.x);
  fcx r;
  r.x = fp_dot_done(re);
  r.y = fp_dot_done(im);
  return r;
}
// sum over c < 4 of m[c] * x[c]
__device__ __forceinline__ fcx cdot4(const fcx *m, int stride, const fcx (&x)[4]) {
  fp_dot re = fp_dot_first(m[0].x, x[0].x), im = fp_dot_first(m[0].x, x[0].y);
  fp_dot_add(re, -m[0].y, x[0].y);
  fp_dot_add(im, m[0].y, x[0].x);
#pragma unroll
  for (int c = 1; c < 4; ++c) {
    const fcx mc = m[stride * c];
    fp_dot_add(re, mc.x, x[c].x);
    fp_dot_add(im, mc.x, x[c].y);
    fp_dot_add(re, -mc.y, x[c].y);
    fp_dot_add(im, mc.y, x[c].x);
  }
  fcx r;
  r.x = fp_dot_done(re);
  r.y = fp_dot_done(im);
  return r;
}

__device__ __forceinline__ fcx to_reg_pair(double2 a) {
  fcx r;
  r.x = fpair_from_double(a.x);
  r.y = fpair_from_double(a.y);
  return r;
}
__device__ __forceinline__ double2 from_reg(fcx a, double2) {
  double2 r;
  r.x = fpair_to_double(a.x);
  r.y = fpair_to_double(a.y);
  return r;
}

#endif  // GBQV_FPAIR_CUH
