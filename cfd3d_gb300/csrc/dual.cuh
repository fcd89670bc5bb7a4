// dual.cuh -- forward-mode dual numbers for the local Jacobians of the discrete adjoint.
//
// Dual<N> carries a value and its derivatives along N seed directions.  The adjoint
// kernels evaluate the same templated routines as the forward kernels (reconstruction,
// fluxes, sources, boundary operations) on Dual<N> inputs seeded with the identity, which
// yields the routine's local Jacobian; contracted with the cotangent it gives the routine's
// vector-Jacobian product.  Branches (limiter cases, min/max, upwind direction, clips) are
// taken on the values, as in the forward evaluation, so the derivative is that of the
// branch the forward residual took.  Values are formed without FMA contraction, like the
// reconstruction's uncontracted arithmetic, so that ties at clip bounds resolve the same way.
#pragma once
#include <cmath>
#include "iapws.cuh"

namespace cfd {

template <int N>
struct Dual {
  double v;
  double d[N];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(x) {
#pragma unroll 1
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  __device__ __forceinline__ static Dual seed(double x, int i) {
    Dual r(x);
    r.d[i] = 1.0;
    return r;
  }
  __device__ __forceinline__ explicit operator double() const { return v; }
};

#define DUAL_LOOP _Pragma("unroll 1") for (int i = 0; i < N; ++i)

template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = __dadd_rn(a.v, b.v); DUAL_LOOP r.d[i] = a.d[i] + b.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = __dsub_rn(a.v, b.v); DUAL_LOOP r.d[i] = a.d[i] - b.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v; DUAL_LOOP r.d[i] = -a.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = __dmul_rn(a.v, b.v); DUAL_LOOP r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
  DUAL_LOOP r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
// mixed operands
template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v = __dadd_rn(r.v, b); return r; }
template <int N> __device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v = __dadd_rn(a, r.v); return r; }
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v = __dsub_rn(r.v, b); return r; }
template <int N> __device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) {
  Dual<N> r; r.v = __dsub_rn(a, b.v); DUAL_LOOP r.d[i] = -b.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = __dmul_rn(a.v, b); DUAL_LOOP r.d[i] = a.d[i] * b; return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v / b;
  const double ib = 1.0 / b;
  DUAL_LOOP r.d[i] = a.d[i] * ib;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a / b.v;
  const double f = -r.v / b.v;
  DUAL_LOOP r.d[i] = f * b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> __device__ __forceinline__ Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N> __device__ __forceinline__ Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { a = a * b; return a; }

// comparisons on values
template <int N> __device__ __forceinline__ bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> __device__ __forceinline__ bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> __device__ __forceinline__ bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> __device__ __forceinline__ bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> __device__ __forceinline__ bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> __device__ __forceinline__ bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> __device__ __forceinline__ bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
template <int N> __device__ __forceinline__ bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N> __device__ __forceinline__ bool operator!=(const Dual<N>& a, double b) { return a.v != b; }
template <int N> __device__ __forceinline__ bool operator!=(const Dual<N>& a, const Dual<N>& b) { return a.v != b.v; }
template <int N> __device__ __forceinline__ bool operator==(const Dual<N>& a, const Dual<N>& b) { return a.v == b.v; }
template <int N> __device__ __forceinline__ bool operator==(const Dual<N>& a, double b) { return a.v == b; }

// elementary functions
template <int N> __device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r; r.v = ::sqrt(a.v);
  const double f = (r.v > 0.0) ? 0.5 / r.v : 0.0;
  DUAL_LOOP r.d[i] = f * a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> exp(const Dual<N>& a) {
  Dual<N> r; r.v = ::exp(a.v); DUAL_LOOP r.d[i] = r.v * a.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> log(const Dual<N>& a) {
  Dual<N> r; r.v = ::log(a.v); const double f = 1.0 / a.v; DUAL_LOOP r.d[i] = f * a.d[i]; return r;
}
template <int N> __device__ __forceinline__ Dual<N> tanh(const Dual<N>& a) {
  Dual<N> r; r.v = ::tanh(a.v); const double f = 1.0 - r.v * r.v; DUAL_LOOP r.d[i] = f * a.d[i]; return r;
}
// x^y with a constant exponent
template <int N> __device__ __forceinline__ Dual<N> pow(const Dual<N>& a, double y) {
  Dual<N> r; r.v = ::pow(a.v, y);
  const double f = (a.v != 0.0) ? y * r.v / a.v : 0.0;
  DUAL_LOOP r.d[i] = f * a.d[i];
  return r;
}
// x^y with both varying: d = x^y (y' log x + y x'/x)
template <int N> __device__ __forceinline__ Dual<N> pow(const Dual<N>& a, const Dual<N>& y) {
  Dual<N> r; r.v = ::pow(a.v, y.v);
  const double lx = (a.v > 0.0) ? ::log(a.v) : 0.0;
  const double f = (a.v != 0.0) ? y.v * r.v / a.v : 0.0;
  DUAL_LOOP r.d[i] = r.v * lx * y.d[i] + f * a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) { return (a.v < 0.0) ? -a : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return (b.v < a.v) ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return (b.v > a.v) ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N>& a, double b) { return (b < a.v) ? Dual<N>(b) : a; }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N>& a, double b) { return (b > a.v) ? Dual<N>(b) : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(double a, const Dual<N>& b) { return (b.v < a) ? b : Dual<N>(a); }
template <int N> __device__ __forceinline__ Dual<N> fmax(double a, const Dual<N>& b) { return (b.v > a) ? b : Dual<N>(a); }
template <int N> __device__ __forceinline__ Dual<N> copysign(double a, const Dual<N>& b) { return Dual<N>(::copysign(a, b.v)); }
template <int N> __device__ __forceinline__ bool isfinite(const Dual<N>& a) { return ::isfinite(a.v); }

// uncontracted arithmetic of the reconstruction: duals have no FMA ambiguity
template <int N> __device__ __forceinline__ Dual<N> nmul(const Dual<N>& a, const Dual<N>& b) { return a * b; }
template <int N> __device__ __forceinline__ Dual<N> nadd(const Dual<N>& a, const Dual<N>& b) { return a + b; }
template <int N> __device__ __forceinline__ Dual<N> nsub(const Dual<N>& a, const Dual<N>& b) { return a - b; }

#undef DUAL_LOOP

// IF97 Gibbs sums on dual arguments: g = sum n x^I y^J with its first three derivatives
// accumulated in FP64 term by term, then each accumulated derivative g_a becomes a dual
// number with d(g_a) = g_ax dx + g_ay dy.  Exact, and the term loop stays plain FP64.
template <int N>
struct GibbsByParts<Dual<N>> {
  static constexpr bool value = true;
  template <const IJN* TAB, size_t K>
  static __device__ __forceinline__ void term(double x, double xi, double y, double yi, double* S) {
    constexpr int I = TAB[K].i;
    constexpr int J = TAB[K].j;
    constexpr double n = TAB[K].n;
    const double t = n * cpow<I>(x, xi) * cpow<J>(y, yi);
    constexpr double i1 = I, i2 = double(I) * (I - 1), i3 = double(I) * (I - 1) * (I - 2);
    constexpr double j1 = J, j2 = double(J) * (J - 1), j3 = double(J) * (J - 1) * (J - 2);
    if constexpr (I != 0) S[0] += i1 * t * xi;
    if constexpr (J != 0) S[1] += j1 * t * yi;
    if constexpr (I != 0 && I != 1) S[2] += i2 * t * (xi * xi);
    if constexpr (I != 0 && J != 0) S[3] += i1 * j1 * t * (xi * yi);
    if constexpr (J != 0 && J != 1) S[4] += j2 * t * (yi * yi);
    if constexpr (I != 0 && I != 1 && I != 2) S[5] += i3 * t * (xi * xi * xi);
    if constexpr (I != 0 && I != 1 && J != 0) S[6] += i2 * j1 * t * (xi * xi * yi);
    if constexpr (I != 0 && J != 0 && J != 1) S[7] += i1 * j2 * t * (xi * yi * yi);
    if constexpr (J != 0 && J != 1 && J != 2) S[8] += j3 * t * (yi * yi * yi);
  }
  template <const IJN* TAB, size_t... K>
  static __device__ __forceinline__ void sum(const Dual<N>& x, const Dual<N>& xi, const Dual<N>& y,
                                             const Dual<N>& yi, GAcc<Dual<N>>& a) {
    // S: g_x, g_y, g_xx, g_xy, g_yy, g_xxx, g_xxy, g_xyy, g_yyy
    double S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    (term<TAB, K>(x.v, xi.v, y.v, yi.v, S), ...);
    const int from[5][3] = {{0, 2, 3}, {1, 3, 4}, {2, 5, 6}, {3, 6, 7}, {4, 7, 8}};
    Dual<N>* out[5] = {&a.x, &a.y, &a.xx, &a.xy, &a.yy};
    for (int q = 0; q < 5; ++q) {
      Dual<N> r(S[from[q][0]]);
      for (int i = 0; i < N; ++i) r.d[i] = S[from[q][1]] * x.d[i] + S[from[q][2]] * y.d[i];
      *out[q] = *out[q] + r;
    }
  }
};

}  // namespace cfd
