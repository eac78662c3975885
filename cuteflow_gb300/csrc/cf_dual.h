/*
 * cf_dual.h -- forward-mode dual numbers for the discrete adjoint.
 *
 * Dual<N> carries a value and N directional derivatives.  The value lane performs exactly the
 * IEEE operations the plain FP64 forward performs (same order, no contraction: the kernels are
 * compiled with -fmad=false), so comparisons taken on values select the same branches as the
 * forward step, and the derivative lanes are the exact local derivatives of that branch.  The
 * templated step arithmetic (cf_flux.h) instantiated with Dual<N> therefore yields the local
 * Jacobians the reverse sweep needs (dt frozen).
 */
#ifndef CF_DUAL_H
#define CF_DUAL_H

#include "cf_flux.h"
#include "cf_xd.h"

#ifdef __CUDACC__
#define CFD_HD __host__ __device__ __forceinline__
#else
#define CFD_HD inline
#endif

namespace cf {

#ifdef __CUDACC__
using ::fabs;
using ::sqrt;
#endif

template <int N>
struct Dual {
  double v;
  double d[N];
  CFD_HD Dual() : v(0.0) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  CFD_HD Dual(double x) : v(x) {  // NOLINT: constants promote implicitly
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  /* the i-th independent variable with value x */
  static CFD_HD Dual var(double x, int i) {
    Dual r(x);
    r.d[i] = 1.0;
    return r;
  }
};

template <int N>
CFD_HD double val(const Dual<N>& x) { return x.v; }

template <int N>
CFD_HD Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
CFD_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
CFD_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
CFD_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(a.d[i], b.v, a.v * b.d[i]);
  return r;
}
/* a / b: the value lane is the IEEE quotient and the derivative lanes use the reciprocal, both
 * from the integer-pipe division of cf_xd.h (the FP64 pipe keeps the lanes' FMAs) */
template <int N>
CFD_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  const double y = em_div(1.0, b.v);
  r.v = em_div(a.v, b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(-r.v, b.d[i], a.d[i]) * y;
  return r;
}
/* mixed with constants */
template <int N> CFD_HD Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v + b; return r; }
template <int N> CFD_HD Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v = a + b.v; return r; }
template <int N> CFD_HD Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v - b; return r; }
template <int N>
CFD_HD Dual<N> operator-(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
template <int N>
CFD_HD Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
CFD_HD Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i];
  return r;
}
template <int N>
CFD_HD Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v / b;  /* mostly constants (/ 2, / 4), which the compiler folds */
  const double y = 1.0 / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * y;
  return r;
}
template <int N>
CFD_HD Dual<N> operator/(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = em_div(a, b.v);
  const double y = em_div(1.0, b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -r.v * b.d[i] * y;
  return r;
}
/* comparisons act on values, on the ordered integer keys of cf_xd.h (the IEEE results: NaN
 * compares false, -0 equals +0), which keeps them off the FP64 pipe the derivative lanes use */
template <int N> CFD_HD bool operator<(const Dual<N>& a, const Dual<N>& b) { return xlt(a.v, b.v); }
template <int N> CFD_HD bool operator>(const Dual<N>& a, const Dual<N>& b) { return xlt(b.v, a.v); }
template <int N> CFD_HD bool operator<=(const Dual<N>& a, const Dual<N>& b) { return xle(a.v, b.v); }
template <int N> CFD_HD bool operator>=(const Dual<N>& a, const Dual<N>& b) { return xle(b.v, a.v); }
template <int N> CFD_HD bool operator<(const Dual<N>& a, double b) { return xlt(a.v, b); }
template <int N> CFD_HD bool operator>(const Dual<N>& a, double b) { return xlt(b, a.v); }
template <int N> CFD_HD bool operator<=(const Dual<N>& a, double b) { return xle(a.v, b); }
template <int N> CFD_HD bool operator>=(const Dual<N>& a, double b) { return xle(b, a.v); }
template <int N> CFD_HD bool operator<(double a, const Dual<N>& b) { return xlt(a, b.v); }
template <int N> CFD_HD bool operator>(double a, const Dual<N>& b) { return xlt(b.v, a); }
template <int N> CFD_HD bool operator==(const Dual<N>& a, const Dual<N>& b) { return xeq(a.v, b.v); }
template <int N> CFD_HD bool operator!=(const Dual<N>& a, const Dual<N>& b) { return !xeq(a.v, b.v); }

template <int N>
CFD_HD Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = em_sqrt(a.v);
  const double y = r.v > 0.0 ? em_div(0.5, r.v) : 0.0; /* sqrt(0) only where the depth is exactly zero */
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * y;
  return r;
}
template <int N>
CFD_HD Dual<N> fabs(const Dual<N>& a) {
  return (a.v < 0.0) ? -a : a;
}

/* the reciprocal of a depth with its derivative (the stored RN(1/h) carries none) */
template <int N>
CFD_HD Dual<N> recip_h(const Dual<N>& h, double) { return 1.0 / h; }

/* Quotient by a known reciprocal (div_rn in cf_flux.h): the value lane is the step's own
 * rounding; the lanes differentiate a / d. */
template <int N>
CFD_HD Dual<N> div_rn(const Dual<N>& a, const Dual<N>& d, const Dual<N>& y) {
  Dual<N> r;
  r.v = em_div(a.v, d.v);  /* the IEEE quotient, as div_rn's */
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(-r.v, d.d[i], a.d[i]) * y.v;
  return r;
}
template <int N>
CFD_HD Dual<N> div_rn(const Dual<N>& a, double d, double y) {
  Dual<N> r;
  r.v = em_div(a.v, d);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * y;
  return r;
}

/* x^(-1/3): d/dx = -r / (3 x) with r = x^(-1/3) */
template <int N>
CFD_HD Dual<N> rcbrt(const Dual<N>& x) {
  Dual<N> r;
  r.v = rcbrt(x.v);
  const double k = -em_div(r.v, 3.0 * x.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * k;
  return r;
}

}  // namespace cf

#endif
