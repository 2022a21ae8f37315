// fe_df64.cuh -- FP64-class Jacobian arithmetic on GB300's FP32 pipes.
//
// GB300 issues FP64 at ~1/64 of its FP32 rate, and the element kernels are
// bound by it.  A "df64" value is the unevaluated sum hi + lo of two binary32
// numbers with |lo| <= ulp(hi) / 2: a 48-bit significand, relative rounding
// error ~2^-48 (3.6e-15) per operation -- three orders of magnitude inside
// the 1e-12 parity contract of the Jacobian, at ~18 FP32 instructions per
// multiply-add instead of one FP64 FMA.  The algorithms are the classical
// error-free transformations: Knuth's two-sum for addition, the FMA
// two-product for multiplication, renormalised with Dekker's fast two-sum
// (Dekker 1971; the double-double arithmetic of Hida, Li & Bailey 2001,
// applied to binary32).  Every FP32 operation is written with an explicit
// rounding intrinsic so that the compiler cannot contract or reorder it:
// the transformations are exact only as written.
//
// Conversions between binary64 and binary32 are done on the integer pipe
// (exponent rebias, fraction shift, round half up on the magnitude), so a
// conversion costs the FP64 pipe one exact subtraction; zeros, values
// outside the binary32 normal range, infinities and NaN take the ordinary
// conversion.  Range: full df64 accuracy for |x| in ~[1e-30, 3e38].
//
// Device code for nvcc (the library) and nvrtc (generated kernels); the CPU
// emulation of generated kernels compiles it as host C++ with shims for the
// intrinsics.
#ifndef FE_DF64_CUH
#define FE_DF64_CUH

// binary32 -> binary64, exact (sign, exponent + 1023 - 127, fraction << 29)
__device__ __forceinline__ double fe_widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (e - 1u < 254u)
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
  if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)sign);
  return (double)f;
}
__device__ __forceinline__ double fe_widen(double d) { return d; }

// binary64 -> nearest binary32 (ties away from zero), by integer operations
__device__ __forceinline__ float fe_narrow(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned long long mag = u & 0x7fffffffffffffffULL;
  const unsigned sign = (unsigned)(u >> 63) << 31;
  if (mag == 0ULL) return __uint_as_float(sign);
  const unsigned long long e = mag >> 52;
  if (e - 897ULL < 254ULL) {  // binary32 exponent field 1..254
    const unsigned long long r = mag + (1ULL << 28);  // round at the 29th fraction bit; carries into e
    const unsigned long long e2 = r >> 52;
    if (e2 <= 1150ULL)
      return __uint_as_float(sign | (unsigned)((e2 - 896ULL) << 23) | (unsigned)((r >> 29) & 0x7fffffULL));
  }
  return (float)d;
}

struct fe_df64 {
  float hi, lo;
  __device__ fe_df64() {}
  __device__ fe_df64(float h, float l) : hi(h), lo(l) {}
  __device__ fe_df64(int z) : hi((float)z), lo(0.0f) {}
  // split: hi = nearest binary32, lo = the exact remainder rounded
  __device__ explicit fe_df64(double d) {
    hi = fe_narrow(d);
    lo = fe_narrow(d - fe_widen(hi));
  }
};

// value as binary64 (one FP64 add)
__device__ __forceinline__ double fe_widen(fe_df64 a) { return fe_widen(a.hi) + fe_widen(a.lo); }

__device__ __forceinline__ fe_df64 operator+(fe_df64 a, fe_df64 b) {
  // two-sum of the high parts (exact), plus the low parts, then renormalise
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  const float e0 = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  const float e = __fadd_rn(e0, __fadd_rn(a.lo, b.lo));
  const float h = __fadd_rn(s, e);
  return fe_df64(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ fe_df64 operator*(fe_df64 a, fe_df64 b) {
  // two-product of the high parts (exact with an FMA), plus the cross terms
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float h = __fadd_rn(p, e);
  return fe_df64(h, __fsub_rn(e, __fsub_rn(h, p)));
}

__device__ __forceinline__ fe_df64 &operator+=(fe_df64 &a, fe_df64 b) {
  a = a + b;
  return a;
}

__device__ __forceinline__ fe_df64 operator-(fe_df64 a) { return fe_df64(-a.hi, -a.lo); }
__device__ __forceinline__ fe_df64 operator-(fe_df64 a, fe_df64 b) { return a + (-b); }

// a / b: the binary32 quotient of the high parts, corrected once by the
// remainder a - q1 b formed in df64 (Dekker 1971, the one-correction
// double-double division of Hida, Li & Bailey 2001); ~2^-44 relative
__device__ __forceinline__ fe_df64 operator/(fe_df64 a, fe_df64 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const fe_df64 r = a - fe_df64(q1, 0.0f) * b;
  const float q2 = __fdiv_rn(r.hi, b.hi);
  const float h = __fadd_rn(q1, q2);
  return fe_df64(h, __fsub_rn(q2, __fsub_rn(h, q1)));
}

// acc += b * c as a compensated dot-product step (Ogita, Rump & Oishi 2005,
// "Accurate sum and dot product", algorithm Dot2, with df64 operands): the
// exact two-product of the high parts and the cross terms form the product's
// error, the exact two-sum of the running high part and the product forms
// the sum's error, and both errors accumulate in acc.lo without a
// renormalisation per step (12 FP32 instructions instead of 18).  acc.lo then
// holds up to ~(terms) ulp(acc.hi), and the rounding of the additions into it
// grows as (terms)^2 u^2 (u = 2^-24); fe_norm restores |lo| <= ulp(hi) / 2.
// The generated contractions renormalise after every group of a few
// multiply-adds (one knot's terms of one entry), which keeps the error
// bound linear in the number of groups: n m u^2 sum|terms| for n groups of m.
__device__ __forceinline__ void fe_mac(fe_df64 &acc, fe_df64 b, fe_df64 c) {
  const float p = __fmul_rn(b.hi, c.hi);
  float pe = __fmaf_rn(b.hi, c.hi, -p);
  pe = __fmaf_rn(b.hi, c.lo, pe);
  pe = __fmaf_rn(b.lo, c.hi, pe);
  const float s = __fadd_rn(acc.hi, p);
  const float v = __fsub_rn(s, acc.hi);
  const float e = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, v)), __fsub_rn(p, v));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pe));
}

// renormalise (Dekker's fast two-sum; |lo| is small against |hi|)
__device__ __forceinline__ fe_df64 fe_norm(fe_df64 a) {
  const float h = __fadd_rn(a.hi, a.lo);
  return fe_df64(h, __fsub_rn(a.lo, __fsub_rn(h, a.hi)));
}

// acc + b * c as one fused multiply-add in the accumulator's precision (the
// generated Jacobian contractions chain these into the accumulator instead
// of adding a separately formed sum of products to it: one FP64 add fewer
// per update)
__device__ __forceinline__ double fe_fma(double b, double c, double acc) { return fma(b, c, acc); }
__device__ __forceinline__ float fe_fma(float b, float c, float acc) { return __fmaf_rn(b, c, acc); }

// the stored (CSR / element-matrix) value of an accumulator
__device__ __forceinline__ float fe_jstore(float v) { return v; }
__device__ __forceinline__ double fe_jstore(double v) { return v; }
__device__ __forceinline__ double fe_jstore(fe_df64 v) { return fe_widen(v); }

#endif
