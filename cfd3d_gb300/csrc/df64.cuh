// df64.cuh -- double-float ("float-float") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), carrying a
// ~48-bit significand.  The operations are the classical error-free transformations:
// Knuth's TwoSum, Dekker's fast two-sum, and the FMA-based exact product
// (a*b = p + fma(a, b, -p)), as used in double-double libraries (Dekker 1971; Bailey's
// QD).  On GB300 the FP32 pipes issue ~60x the FP64 rate, so an IF97 Gibbs sum in
// df64 costs a fraction of the same sum in FP64 at ~1e-14 relative accuracy.
// The exponent range is FP32's: IF97 terms that underflow here are below 1e-38 and
// contribute nothing at this precision.
#pragma once

namespace cfd {

// float <-> double conversions on the integer pipes.  On a GB300 the hardware conversions
// issue on the FP64 pipe at its rate (2 per clock per SM, measured: 625 G conversions/s
// either way).  These give the same bits -- IEEE 754 round to nearest, ties to even -- from
// integer instructions for the normal range and signed zeros (measured 1.5 / 2.2 T
// conversions/s alone), and hand the rest (subnormals, infinities, NaNs, values outside the
// float range) to the hardware conversion.  Inside a kernel they cost a dozen integer
// instructions, two branches and registers per cast: the eddy viscosity, whose work is
// mostly casts of its neighbours' states, gains from them; the update, the residual and
// the time step measured slower with them, and keep the hardware's.
__device__ __forceinline__ float to_f32(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;             // the float's biased exponent
  const unsigned keep = ((hi & 0xfffffu) << 3) | (lo >> 29);  // 23 significand bits
  const unsigned rem = lo & 0x1fffffffu;                      // the 29 bits rounded off
  const unsigned up = (rem > 0x10000000u) | ((rem == 0x10000000u) & keep);
  // (a carry out of the significand steps the exponent, to infinity past the largest float)
  if (e >= 1 && e <= 254) return __uint_as_float((hi & 0x80000000u) | (((unsigned)e << 23) + keep + (up & 1u)));
  if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
  return __double2float_rn(x);
}
__device__ __forceinline__ double to_f64(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e != 0u && e != 0xffu)
    return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return (double)x;
}

struct df64 {
  float hi, lo;
  __device__ __forceinline__ df64() {}
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit df64(double a) {
    hi = static_cast<float>(a);
    lo = static_cast<float>(a - static_cast<double>(hi));
  }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64(s, e);
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64(s, e);
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  float e = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, e);
  e = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // long division with one correction step
  float q1 = __fdiv_rn(a.hi, b.hi);
  df64 r = a - b * df64(q1, 0.0f);
  float q2 = __fdiv_rn(r.hi, b.hi);
  df64 q = fast_two_sum(q1, q2);
  r = a - b * q;
  float q3 = __fdiv_rn(r.hi, b.hi);
  return q + df64(q3, 0.0f);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { a = a + b; return a; }

}  // namespace cfd
