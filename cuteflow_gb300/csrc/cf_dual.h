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

/* The transposed edge stage of an interior first-order HLLC edge (IFLUX 1, flux_mode 0): given the
 * adjoint weights w[10] of its two slots (side A: flux 1-3, bed x, y; then side B), the
 * contributions lamA, lamB to the adjoints of (h, hu, hv) of its two elements, i.e. J^T w for the
 * edge's Jacobian J, at a fraction of the cost of differentiating the whole edge in six lanes:
 *   - the change to the edge frame and the hydrostatic reconstruction have closed-form
 *     derivatives (u_n = (hu nx + hv ny) / h, u_t = (hv nx - hu ny) / h; reconstructed depths pass
 *     or are clamped to 0);
 *   - the flux core depends on (hl, ul, hr, ur) and on the tangential velocities only through its
 *     tangential components, which are x1 vl or x1 vr (side A) and y1 vl or y1 vr (side B) with
 *     the region telling which (first_order_flux reports it): the core runs on Dual<4> numbers over
 *     (hl, ul, hr, ur), and the tangential derivatives are x1, y1;
 *   - the bed sources g/2 (ha^2 - h^2) len have closed-form derivatives.
 * The value lanes repeat the step's IEEE operations, so every branch is the forward's.  Returns
 * false, and the caller differentiates the edge in full, where a side's raw and masked depths
 * differ (0 < h <= tolisec; the reference then evaluates the two sides differently). */
CFD_HD bool adj_edge_hllc(const MemberDev& M, const EdgeGeo& G, const double4& UA, const double4& UB, double zml,
                          double zmr, const double w[10], double lamA[3], double lamB[3]) {
  const double g = M.gp, tolisec = M.tolisec, nx = G.nx, ny = G.ny, len = G.len;
  /* the comparisons on integer keys (xlt, xeq, and XD<false> for the frame change: the same IEEE
   * results and the same double arithmetic) keep them off the FP64 pipe that bounds this kernel */
  const auto kmax = [](double a, double b) { return xlt(a, b) ? b : a; };   /* Fortran max */
  const double zij = kmax(zml, zmr);
  XD<false> hl_, ul_, vl_, hr_, ur_, vr_;
  to_frame(XD<false>(UA.x), XD<false>(UA.y), XD<false>(UA.z), UA.w, nx, ny, tolisec, hl_, ul_, vl_);
  to_frame(XD<false>(UB.x), XD<false>(UB.y), XD<false>(UB.z), UB.w, nx, ny, tolisec, hr_, ur_, vr_);
  const double hautl = val(hl_), vitul = val(ul_), vitvl = val(vl_);
  const double hautr = val(hr_), vitur = val(ur_), vitvr = val(vr_);
  if (!xeq(hautl, UA.x) || !xeq(hautr, UB.x)) return false;
  /* hydrostatic reconstruction (flux_riemann.cuf:176-181, :200-210); which variables carry a
   * derivative (a clamped or masked one is a constant of the inputs) */
  const double el = hautl + zml - zij, er = UB.x + zmr - zij;
  double hl = kmax(0.0, el), hr = kmax(0.0, er);
  double ul = vitul, vl = vitvl, ur = vitur, vr = vitvr;
  const bool pl = !xlt(hl, tolisec), pr = !xlt(hr, tolisec);
  if (!pl) { hl = 0.; ul = 0.; vl = 0.; }
  if (!pr) { hr = 0.; ur = 0.; vr = 0.; }
  const bool wa = xlt(tolisec, UA.x), wb = xlt(tolisec, UB.x);   /* frame velocities differentiable */
  const bool s_hl = pl && xlt(0.0, el), s_ul = pl && wa, s_hr = pr && xlt(0.0, er), s_ur = pr && wb;
  const Dual<4> Hl = s_hl ? Dual<4>::var(hl, 0) : Dual<4>(hl), Ul = s_ul ? Dual<4>::var(ul, 1) : Dual<4>(ul);
  const Dual<4> Hr = s_hr ? Dual<4>::var(hr, 2) : Dual<4>(hr), Ur = s_ur ? Dual<4>::var(ur, 3) : Dual<4>(ur);
  TwoFluxT<Dual<4>> F;
  HllcRegions rg;
  first_order_flux<1>(g, nx, ny, Hl, Ul, Dual<4>(vl), Hr, Ur, Dual<4>(vr), F, &rg);
  /* w^T d(slot fluxes)/d(hl, ul, hr, ur): the slots hold F * len */
  double gc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
    gc[i] = len * (w[0] * F.a1.d[i] + w[1] * F.a2.d[i] + w[2] * F.a3.d[i] + w[5] * F.b1.d[i] + w[6] * F.b2.d[i] +
                   w[7] * F.b3.d[i]);
  /* tangential velocities: a2 = nx x2 - ny x3, a3 = ny x2 + nx x3 with x3 = x1 v (x1 = a1);
   * b2 = -(nx y2 - ny y3), b3 = -(ny y2 + nx y3) with y3 = y1 v (y1 = -b1) */
  double gvl = 0.0, gvr = 0.0;
  if (rg.valid) {
    const double ga = len * (w[2] * nx - w[1] * ny) * F.a1.v;
    const double gb = len * (w[7] * nx - w[6] * ny) * F.b1.v;   /* (ny w6 - nx w7) y1 with y1 = -b1 */
    if (rg.a_vr) gvr += ga; else gvl += ga;
    if (rg.b_vr) gvr += gb; else gvl += gb;
  }
  /* to the conserved variables: d(h_m, u_n, u_t)/d(h, hu, hv) with y = RN(1/h) */
  lamA[0] = lamA[1] = lamA[2] = 0.0;
  lamB[0] = lamB[1] = lamB[2] = 0.0;
  {
    const double gh = s_hl ? gc[0] : 0.0, gu = s_ul ? gc[1] : 0.0, gv = s_ul ? gvl : 0.0;
    if (wa) {
      const double y = UA.w;
      lamA[0] = gh - (gu * vitul + gv * vitvl) * y;
      lamA[1] = (gu * nx - gv * ny) * y;
      lamA[2] = (gu * ny + gv * nx) * y;
    }
  }
  {
    const double gh = s_hr ? gc[2] : 0.0, gu = s_ur ? gc[3] : 0.0, gv = s_ur ? gvr : 0.0;
    lamB[0] = gh;   /* the B side reconstructs from the raw depth */
    if (wb) {
      const double y = UB.w;
      lamB[0] -= (gu * vitur + gv * vitvr) * y;
      lamB[1] = (gu * nx - gv * ny) * y;
      lamB[2] = (gu * ny + gv * nx) * y;
    }
  }
  /* bed sources (source_terms.cuf:90-97): ta = g/2 (ha^2 - hA^2) len into (ta nx, ta ny) of
   * side A, tb likewise into -(tb nx, tb ny) of side B */
  {
    const double ea = UA.x + zml - zij, eb = UB.x + zmr - zij;
    const double ha = kmax(0.0, ea), hb = kmax(0.0, eb);
    const double dta = g / 2.0 * (2.0 * (xlt(0.0, ea) ? ha : 0.0) - 2.0 * UA.x) * len;
    const double dtb = g / 2.0 * (2.0 * (xlt(0.0, eb) ? hb : 0.0) - 2.0 * UB.x) * len;
    lamA[0] += (w[3] * nx + w[4] * ny) * dta;
    lamB[0] -= (w[8] * nx + w[9] * ny) * dtb;
  }
  return true;
}

}  // namespace cf

#endif
