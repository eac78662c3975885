/*
 * cf_flux.h -- per-edge and per-element arithmetic of the step, shared by the sm_103a kernels
 * (cf_kernels.cu, cf_adjoint.cu) and, compiled for the host, by the CPU test harness that checks
 * it against the oracle edge by edge.  Everything here is __host__ __device__ and FP64.
 *
 * Bit-exact reproduction.  The reference's WAF flux is discontinuous at the bit level: where
 * the reconstructed depths of an edge are equal to the last bit (still water),
 * r = dupw / (dloc + eps) (flux_riemann.cuf:876-878) changes sign with the side that
 * evaluates it, and a one-ulp change of the state moves the limiter between its branches.
 * A result "within round-off" of the reference therefore does not stay within 1e-9 of it.
 * This code evaluates every expression in the reference's order of operations, with true
 * divisions, and the kernels are compiled without FMA contraction (-fmad=false), so a step
 * on the GPU reproduces the CPU restatement of the reference bit for bit.  The second side of
 * an edge is obtained from the first by exact IEEE identities ((-a)*b = -(a*b),
 * (-a)-(-b) = b-a, commutativity), never by re-rounded arithmetic.
 *
 * Scalar type.  The state-dependent arithmetic is written once, as templates on the scalar
 * type T.  T = double is the step.  T = Dual<N> (cf_dual.h) carries N derivative lanes next to
 * a value lane that performs the same IEEE operations in the same order, so it takes the same
 * branches (wet/dry masks, wave regions, limiter cases) as the step and its lanes are the exact
 * local Jacobian of that branch: the discrete adjoint is built from it.  Geometry, time and
 * time step stay double (the adjoint holds dt fixed).
 */
#ifndef CF_FLUX_H
#define CF_FLUX_H

#include <cmath>
#include <cstring>

#include "cf_internal.h"

#ifdef __CUDACC__
#define CF_HD __host__ __device__
#define CF_INLINE __forceinline__
#else
#define CF_HD
#define CF_INLINE inline
#endif

namespace cf {

#ifndef __CUDACC__
using std::copysign;
using std::fabs;
using std::fma;
using std::fmax;
using std::frexp;
using std::ldexp;
using std::sqrt;
#endif

/* ---- loads --------------------------------------------------------------------------- */

CF_HD CF_INLINE double4 ld4(const double4* p) {
#ifdef __CUDA_ARCH__
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 a = __ldg(q), b = __ldg(q + 1);
  return make_double4(a.x, a.y, b.x, b.y);
#else
  return *p;
#endif
}

template <class T>
CF_HD CF_INLINE T ldro(const T* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

/* The two 32-bit words of a bit pattern, through an opaque move on the device.  A test written on
 * a double's whole 64-bit pattern, such as (b << 1) == 0 or (b & exponent) != exponent, is
 * recognised by the compiler as a comparison of the double and issued as an FP64-pipe instruction
 * (measured: one per test); on the words it stays on the integer pipes. */
CF_HD CF_INLINE void words_u(uint64_t b, uint32_t& lo, uint32_t& hi) {
#ifdef __CUDA_ARCH__
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(b));
#else
  lo = (uint32_t)b;
  hi = (uint32_t)(b >> 32);
#endif
}
/* b is the pattern of a finite double */
CF_HD CF_INLINE bool finite_u(uint64_t b) {
  uint32_t lo, hi;
  words_u(b, lo, hi);
  (void)lo;
  return (hi & 0x7ff00000u) != 0x7ff00000u;
}
/* b is the pattern of +0 or -0 */
CF_HD CF_INLINE bool zero_u(uint64_t b) {
  uint32_t lo, hi;
  words_u(b, lo, hi);
  return ((hi << 1) | lo) == 0;
}

CF_HD CF_INLINE bool finite_bits(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return finite_u(b);
}

/* value of a scalar (the Dual overload is in cf_dual.h) */
CF_HD CF_INLINE double val(double x) { return x; }

template <class T>
CF_HD CF_INLINE T dmax(const T& a, const T& b) { return (a < b) ? b : a; } /* Fortran max */
template <class T>
CF_HD CF_INLINE T dmin(const T& a, const T& b) { return (b < a) ? b : a; } /* Fortran min */

/* x / 2, x / 4 and 2 x.  A scaling by a power of two rounds once whichever way it is written, so
 * these give the bits of the quotient or product they stand for; the integer-product type (cf_xd.h)
 * overloads them with an exponent change. */
template <class T>
CF_HD CF_INLINE T halve(const T& x) { return x * 0.5; }
template <class T>
CF_HD CF_INLINE T quarter(const T& x) { return x * 0.25; }
template <class T>
CF_HD CF_INLINE T twice(const T& x) { return x * 2.0; }

/* a / d rounded to nearest, given y = RN(1/d): q = RN(a y), r = a - d q (exact through the
 * FMA), RN(q + r y) (Markstein's correction step; P. Markstein, "Computation of elementary
 * functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34, 1990).  It equals the
 * IEEE quotient for finite non-zero a (no mismatch in 3e8 adversarial samples, see the tests);
 * a zero numerator is returned as q = a y, which carries the quotient's sign.  Three FP64
 * instructions instead of a full division wherever 1/d is known: for precomputed geometry,
 * and for denominators shared by several quotients (y = 1/d computed once). */
CF_HD CF_INLINE double div_rn(double a, double d, double y) {
  const double q = a * y;
  const double r = fma(-d, q, a);
  const double q1 = fma(r, y, q);
  uint64_t ab;
  memcpy(&ab, &a, sizeof(ab));
  return zero_u(ab) ? q : q1;
}

/* ---- x**(-1/3) -------------------------------------------------------------------------- */

/* x^(-1/3), the Manning factor h^(-1/3) (source_terms.cuf:112-127; the reference calls pow, which
 * is not correctly rounded and differs between math libraries), as one fixed sequence of IEEE and
 * integer operations that the oracle repeats exactly, with no division:
 *   x = m 2^(3k), m in [1, 8): the exponent split in integer arithmetic (Kahan, "Computing a real
 *       cube root", 1991, splits the exponent by three the same way);
 *   a single-precision seed for m^(-1/3): a cubic in the leading mantissa bits u = 1 + f
 *       (least-squares fit of u^(-1/3) on [1, 2), relative error 2.5e-4) times 2^(-r/3), then one
 *       Newton step y <- y + y (1 - m y^3) / 3 (relative error ~2e-7);
 *   one third-order step in double precision, y <- y + y (e/3 + 2 e^2/9) with e = 1 - m y^3 (the
 *       series of (1 - e)^(-1/3) to second order; the truncation is below 1e-19 relative);
 *   y 2^(-k) by an exponent shift.
 * Rounding bound 1.2 ulp (the two products forming y^3 give e an error of 2^-52, a third of it
 * reaches y; then the final rounding); measured within 1 ulp of the exact value (tests).  Seven
 * FP64-pipe instructions.  Zero, subnormal, infinite, negative and NaN x (never reached by the
 * step, whose depths here exceed tolisec > 0) take rcbrt_special. */
CF_HD CF_INLINE double rcbrt_core(uint64_t b) {
  const uint32_t ex = (uint32_t)(b >> 52);
  const uint32_t ep = ex + 177u;            /* unbiased exponent + 1200 */
  const uint32_t k3 = ep / 3u;
  const uint32_t r = ep - 3u * k3;          /* exponent = 3 (k3 - 400) + r */
  const uint64_t frac = b & ((1ull << 52) - 1);
  const uint64_t mb = frac | ((uint64_t)(1023u + r) << 52);
  const uint32_t ub = (127u << 23) | (uint32_t)(frac >> 29);
  const uint32_t mfb = ub + (r << 23);
  double m;
  float u, mf;
  memcpy(&m, &mb, sizeof(m));
  memcpy(&u, &ub, sizeof(u));
  memcpy(&mf, &mfb, sizeof(mf));
  float y = fmaf(fmaf(fmaf(-0x1.99153cp-5f, u, 0x1.45621ap-2f), u, -0x1.9eb31ap-1f), u, 0x1.8ab91ap+0f);
  y = y * (r == 0u ? 1.0f : (r == 1u ? 0x1.965feap-1f : 0x1.428a30p-1f));
  const float e32 = fmaf(-mf, y * y * y, 1.0f);
  y = fmaf(y, e32 * 0x1.555556p-2f, y);
  const double yd = (double)y;
  const double e = fma(-m, yd * yd * yd, 1.0);
  const double c = e * fma(e, 2.0 / 9.0, 1.0 / 3.0);
  const double res = fma(yd, c, yd);
  uint64_t rb;
  memcpy(&rb, &res, sizeof(rb));
  rb = (uint64_t)((int64_t)rb - ((int64_t)k3 - 400) * (int64_t)(1ull << 52));
  double out;
  memcpy(&out, &rb, sizeof(out));
  return out;
}

/* x^(-1/3) outside the normal positive numbers: +0 -> +inf, subnormal -> scaled by 2^54 into the
 * normal range (x^(-1/3) = (2^54 x)^(-1/3) 2^18, exact scalings), +inf -> 0, negative or NaN ->
 * NaN (Fortran's real power of a negative base). */
CF_HD CF_INLINE double rcbrt_special(double x) {
  if (!(x >= 0.0)) {
    const uint64_t qnan = 0x7ff8000000000000ull;
    double n;
    memcpy(&n, &qnan, sizeof(n));
    return (x != x) ? x : n;
  }
  if (x == 0.0) return 1.0 / x;
  if (x > 1.0) return 0.0;
  const double s = x * 0x1p54;
  uint64_t b;
  memcpy(&b, &s, sizeof(b));
  return rcbrt_core(b) * 0x1p18;
}

CF_HD CF_INLINE double rcbrt(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  if ((uint32_t)(b >> 52) - 1u >= 2046u) return rcbrt_special(x);
  return rcbrt_core(b);
}

/* ---- edge-frame states ------------------------------------------------------------------ */

/* RN(1/h) of an element's depth: the state carries it (the element kernel stores it with the
 * new depth), so the quotients by h below are Markstein's exact three-instruction form.  A
 * linearization computes it from h (cf_dual.h overloads this for its dual numbers). */
template <class T>
CF_HD CF_INLINE T recip_h(const T&, double yh) { return T(yh); }

/* Masked primitive state in the frame (n, t) of an edge (flux_riemann.cuf:105-112); yh = RN(1/h). */
template <class T>
CF_HD CF_INLINE void to_frame(T h, T hu, T hv, double yh, double nx, double ny, double tolisec, T& hm, T& un,
                              T& ut) {
  if (h > tolisec) {
    const T y = recip_h(h, yh);
    un = div_rn(hu * nx + hv * ny, h, y);
    ut = div_rn(hv * nx - hu * ny, h, y);
    hm = h;
  } else {
    hm = T(0.0);
    un = T(0.0);
    ut = T(0.0);
  }
}

/* Only the masked depth and tangential velocity (what the WAF upwind states use). */
template <class T>
CF_HD CF_INLINE void to_frame_t(T h, T hu, T hv, double yh, double nx, double ny, double tolisec, T& hm, T& ut) {
  if (h > tolisec) {
    ut = div_rn(hv * nx - hu * ny, h, recip_h(h, yh));
    hm = h;
  } else {
    hm = T(0.0);
    ut = T(0.0);
  }
}

/* Wave speeds of all solvers (flux_riemann.cuf:930-983, 753-806, 1055-1108).  Returns false
 * when both depths are below eps: the reference then reads uninitialised speeds; the flux
 * defined for that case is zero. */
template <class T>
CF_HD CF_INLINE bool wave_speeds(double g, double eps, T hl, T ul, T hr, T ur, T& sl, T& sr, T& set) {
  if (hl < eps && hr < eps) return false;
  const T al = sqrt(g * hl);
  const T ar = sqrt(g * hr);
  const T het = halve(hl + hr) - quarter((ur - ul) * (hl + hr) / (al + ar));
  T pql, pqr;
  if (het < hl) pql = T(1.);
  else pql = (hl > eps) ? sqrt(halve(het + hl) * het / (hl * hl)) : T(0.);
  if (het < hr) pqr = T(1.);
  else pqr = (hr > eps) ? sqrt(halve(het + hr) * het / (hr * hr)) : T(0.);
  if (hl > eps) {
    sl = ul - al * pql;
    if (hr > eps) {
      sr = ur + ar * pqr;
    } else {
      sl = ul - al;
      sr = ul + twice(al);
    }
  } else {
    sl = ur - twice(ar);
    sr = ur + ar;
  }
  const T denom = hr * (ur - sr) - hl * (ul - sl);
  if (fabs(denom) < eps) set = halve(ul + ur) - (hr - hl) * (al + ar) / (hl + hr);
  else set = (sl * hr * (ur - sr) - sr * hl * (ul - sl)) / denom;
  return true;
}

template <class T>
struct TwoFluxT {
  /* global-frame flux of side A (normal out of A) and of side B (normal out of B) */
  T a1, a2, a3, b1, b2, b3;
};
typedef TwoFluxT<double> TwoFlux;

/* Side A's global flux from the edge-frame vector x; side B's from its vector y: B's frame
 * normal is -n and its vector is the mirror (-y1, y2, y3), which reprojects to
 * -(n1 y2 - n2 y3), -(n2 y2 + n1 y3) exactly. */
template <class T>
CF_HD CF_INLINE void reproject_both(double nx, double ny, T x1, T x2, T x3, T y1, T y2, T y3, TwoFluxT<T>& F) {
  F.a1 = x1;
  F.a2 = nx * x2 - ny * x3;
  F.a3 = ny * x2 + nx * x3;
  F.b1 = -y1;
  F.b2 = -(nx * y2 - ny * y3);
  F.b3 = -(ny * y2 + nx * y3);
}

/* First-order HLLC (IFLUX 1, flux_riemann.cuf:902-1026) and the star-state HLLC of Ata et
 * al. (IFLUX 2, :1029-1182), for both sides.  Side B's evaluation is the mirror image
 * (h -> h, u_n -> -u_n, u_t -> -u_t, s_L -> -s_R, s_R -> -s_L, s_* -> -s_*): it selects a
 * region with its own tests and its vector is the mirror of an A-frame vector. */
/* Which tangential velocity the HLLC (IFLUX 1) tangential fluxes of the two sides carry, for the
 * adjoint: the tangential component of side A's frame flux is x1 * (vl or vr) and side B's is
 * y1 * (vl or vr) in every region (FL: hl ul vl = fl1 vl, FR: fr1 vr, HLL: h1 times the velocity of
 * the upwind side of s*).  a_vr / b_vr: 1 when the side's velocity is vr; valid 0 when both sides
 * are dry (zero flux). */
struct HllcRegions {
  int valid, a_vr, b_vr;
};

template <int IFLUX, class T>
CF_HD CF_INLINE void first_order_flux(double g, double nx, double ny, T hl, T ul, T vl, T hr, T ur, T vr,
                                      TwoFluxT<T>& F, HllcRegions* regions = nullptr) {
  const double eps = (IFLUX == 1) ? EPS_HLLC : EPS_RIADH;
  T sl, sr, set;
  if (regions) regions->valid = 0;
  if (!wave_speeds(g, eps, hl, ul, hr, ur, sl, sr, set)) {
    F.a1 = F.a2 = F.a3 = F.b1 = F.b2 = F.b3 = T(0.0);
    return;
  }
  const T fl1 = hl * ul, fl2 = hl * (ul * ul) + halve(g * hl * hl), fl3 = hl * ul * vl;
  const T fr1 = hr * ur, fr2 = hr * (ur * ur) + halve(g * hr * hr), fr3 = hr * ur * vr;
  T x1, x2, x3, y1, y2, y3;
  if (IFLUX == 1) {
    /* A: sl > 0 -> FL | sr < 0 -> FR | HLL with the tangential component of the upwind side
     * of s*.  B: -sr > 0 -> FR | -sl < 0 -> FL | HLL, tangential by -s*. */
    const int ra = (sl > 0.) ? 0 : ((sr < 0.) ? 1 : 2);
    const int rb = (-sr > 0.) ? 1 : ((-sl < 0.) ? 0 : 2);
    T h1 = T(0.0), h2 = T(0.0);
    if (ra == 2 || rb == 2) {
      const T den = sr - sl + eps, yden = 1.0 / den;
      h1 = div_rn(sr * fl1 - sl * fr1 + sl * sr * (hr - hl), den, yden);
      h2 = div_rn(sr * fl2 - sl * fr2 + sl * sr * (hr * ur - hl * ul), den, yden);
    }
    if (ra == 0) { x1 = fl1; x2 = fl2; x3 = fl3; }
    else if (ra == 1) { x1 = fr1; x2 = fr2; x3 = fr3; }
    else { x1 = h1; x2 = h2; x3 = (set > 0.) ? h1 * vl : h1 * vr; }
    if (rb == 0) { y1 = fl1; y2 = fl2; y3 = fl3; }
    else if (rb == 1) { y1 = fr1; y2 = fr2; y3 = fr3; }
    else { y1 = h1; y2 = h2; y3 = (-set > 0.) ? h1 * vr : h1 * vl; }
    if (regions) {
      regions->valid = 1;
      regions->a_vr = (ra == 1 || (ra == 2 && !(set > 0.))) ? 1 : 0;
      regions->b_vr = (rb == 1 || (rb == 2 && (-set > 0.))) ? 1 : 0;
    }
  } else {
    const T pl = (fabs(sl - set) > eps) ? hl * (sl - ul) / (sl - set) : T(0.0);
    const T pr = (fabs(sr - set) > eps) ? hr * (sr - ur) / (sr - set) : T(0.0);
    const T el1 = fl1 + sl * (pl - hl), el2 = fl2 + sl * (pl * set - hl * ul), el3 = fl3 + sl * (pl * vl - hl * vl);
    const T er1 = fr1 + sr * (pr - hr), er2 = fr2 + sr * (pr * set - hr * ur), er3 = fr3 + sr * (pr * vr - hr * vr);
    /* A: 0<sl FL | 0<s* & 0>sl EL | 0>s* & 0<sr ER | FR.
     * B (sl'=-sr, s*'=-s*, sr'=-sl): 0<-sr FR | 0<-s* & 0>-sr ER | 0>-s* & 0<-sl EL | FL. */
    int ra, rb;
    if (0. < sl) ra = 0;
    else if (0. < set && 0. > sl) ra = 2;
    else if (0. > set && 0. < sr) ra = 3;
    else ra = 1;
    if (0. < -sr) rb = 1;
    else if (0. < -set && 0. > -sr) rb = 3;
    else if (0. > -set && 0. < -sl) rb = 2;
    else rb = 0;
#define CF_PICK(r, a1_, a2_, a3_)                      \
  if (r == 0) { a1_ = fl1; a2_ = fl2; a3_ = fl3; }     \
  else if (r == 1) { a1_ = fr1; a2_ = fr2; a3_ = fr3; } \
  else if (r == 2) { a1_ = el1; a2_ = el2; a3_ = el3; } \
  else { a1_ = er1; a2_ = er2; a3_ = er3; }
    CF_PICK(ra, x1, x2, x3)
    CF_PICK(rb, y1, y2, y3)
#undef CF_PICK
  }
  reproject_both(nx, ny, x1, x2, x3, y1, y2, y3, F);
}

/* WAF limiter (flux_riemann.cuf:465-524).  The superbee gaps at r = 0.5, 1, 2 are kept. */
template <class T>
CF_HD CF_INLINE T waf_limiter(int ilim, T r, T c) {
  T A = T(1.);
  if (ilim == 1) {
    if (r <= 0.) A = T(1.);
    else if (r > 0. && r < 0.5) A = 1. - twice(1. - fabs(c)) * r;
    else if (r > 0.5 && r < 1.) A = fabs(c);
    else if (r > 1. && r < 2.) A = 1. - (1. - fabs(c)) * r;
    else A = twice(fabs(c)) - 1.;
  } else if (ilim == 2) {
    if (r <= 0.) A = T(1.);
    else A = 1. - twice(1. - fabs(c)) * r / (1. + r);
  } else if (ilim == 3) {
    if (r <= 0.) A = T(1.);
    else A = 1. - (1. - fabs(c)) * r * (1. + r) / (1. + r * r);
  } else if (ilim == 4) {
    if (r <= 0.) A = T(1.);
    else if (r <= 1.) A = 1. - (1. - fabs(c)) * r;
    else A = fabs(c);
  }
  return A;
}

template <class T>
CF_HD CF_INLINE double sgn1(const T& x) { return copysign(1.0, val(x)); }

/* sgn1(x) * y, the reference's dsign(1.d0, x) * y: for every y that is not NaN the IEEE product
 * of +-1 and y is y with the sign of x multiplied in, a sign-bit flip (no FP64 instruction). */
CF_HD CF_INLINE double sgnmul(double x, double y) {
  uint64_t bx, by;
  memcpy(&bx, &x, sizeof(bx));
  memcpy(&by, &y, sizeof(by));
  by ^= bx & 0x8000000000000000ull;
  double r;
  memcpy(&r, &by, sizeof(r));
  return r;
}
template <class T>
CF_HD CF_INLINE T sgnmul(const T& x, const T& y) { return sgn1(x) * y; }

/* x, or (freeze) its value taken as a constant of the linearization; the same number either way. */
template <class T>
CF_HD CF_INLINE T held(const T& x, bool freeze) { return freeze ? T(val(x)) : x; }

/* Second-order WAF (IFLUX 3, flux_riemann.cuf:720-900) for both sides.  Inputs: the
 * reconstructed, masked edge-frame states of A (left) and B (right), the upwind
 * reconstructions (h, v) of each side, dt, and the distances d_mrl, d_mkvol (A), d_mkvoisin (B).
 * freeze_r (linearizations only) holds the limiter ratios r constant: r = dupw / (dloc + eps)
 * divides differences that are at round-off level in still water, and its derivative there
 * (~1/eps) carries no information. */
template <class T>
CF_HD CF_INLINE void waf_flux(double g, int ilim, double nx, double ny, double dt, double d_mrl, double y_mrl,
                              double d_mkvol, double y_mkvol, double d_mkvoisin, double y_mkvoisin, T hl, T ul,
                              T vl, T hr, T ur, T vr, T hl_upw, T vl_upw, T hr_upw, T vr_upw, TwoFluxT<T>& F,
                              bool freeze_r = false) {
  const double eps = EPS_SECOND;
  T sl, sr, set;
  if (!wave_speeds(g, eps, hl, ul, hr, ur, sl, sr, set)) {
    F.a1 = F.a2 = F.a3 = F.b1 = F.b2 = F.b3 = T(0.0);
    return;
  }
  const T fl1 = hl * ul, fl2 = hl * (ul * ul) + halve(g * hl * hl);
  const T fr1 = hr * ur, fr2 = hr * (ur * ur) + halve(g * hr * hr);
  const int ra = (sl > 0.) ? 0 : ((sr < 0.) ? 1 : 2);
  const int rb = (-sr > 0.) ? 1 : ((-sl < 0.) ? 0 : 2);
  T h1 = T(0.0), h2 = T(0.0);
  if (ra == 2 || rb == 2) {
    const T den = sr - sl + eps, yden = 1.0 / den;
    h1 = div_rn(sr * fl1 - sl * fr1 + sl * sr * (hr - hl), den, yden);
    h2 = div_rn(sr * fl2 - sl * fr2 + sl * sr * (hr * ur - hl * ul), den, yden);
  }
  const T ha1 = (ra == 0) ? fl1 : ((ra == 1) ? fr1 : h1);
  const T ha2 = (ra == 0) ? fl2 : ((ra == 1) ? fr2 : h2);
  const T hb1 = (rb == 0) ? fl1 : ((rb == 1) ? fr1 : h1);
  const T hb2 = (rb == 0) ? fl2 : ((rb == 1) ? fr2 : h2);

  const double dtoverdx = div_rn(dt, d_mrl, y_mrl);
  const T cr = sr * dtoverdx, cl = sl * dtoverdx, cet = set * dtoverdx;
  const T dloc = div_rn(hr - hl, d_mrl, y_mrl);          /* delta_loc_l = delta_loc_r */
  const T dloc_et = div_rn(vr - vl, d_mrl, y_mrl);
  const T upl = div_rn(hl - hl_upw, d_mkvol, y_mkvol);     /* upwind difference of side A */
  const T upr = div_rn(hr_upw - hr, d_mkvoisin, y_mkvoisin);  /* upwind difference of side B */
  const T upvl = div_rn(vl - vl_upw, d_mkvol, y_mkvol);
  const T upvr = div_rn(vr_upw - vr, d_mkvoisin, y_mkvoisin);
  const T ret_a = held(((set > 0.) ? upvl : upvr) / (dloc_et + eps), freeze_r);

  /* side A (:854-899) */
  {
    const T den = dloc + eps, yd = 1.0 / den;
    const T rl = held(div_rn((sl > 0.) ? upl : upr, den, yd), freeze_r);
    const T rr = held(div_rn((sr > 0.) ? upl : upr, den, yd), freeze_r);
    const T ll = waf_limiter(ilim, rl, cl);
    const T lr = waf_limiter(ilim, rr, cr);
    const T le = waf_limiter(ilim, ret_a, cet);
    const T wl = halve(1. + sgnmul(sl, ll));
    const T wlet = halve(1. + sgnmul(set, le));
    const T wlr = halve(sgnmul(sr, lr) - sgnmul(sl, ll));
    const T wr = halve(1. - sgnmul(sr, lr));
    const T wret = halve(1. - sgnmul(set, le));
    const T fw1 = wl * fl1 + wlr * ha1 + wr * fr1;
    const T fw2 = wl * fl2 + wlr * ha2 + wr * fr2;
    const T fw3 = (wlet * vl + wret * vr) * fw1;
    F.a1 = fw1;
    F.a2 = nx * fw2 - ny * fw3;
    F.a3 = ny * fw2 + nx * fw3;
  }
  /* side B: the same formulas on the mirrored states.  Its local difference is
   * (hl - hr)/d = -dloc, its upwind differences are minus A's (for the wave it tests), the
   * tangential ones coincide; its Courant numbers are -cr, -cl, -cet. */
  {
    const T den = -dloc + eps, yd = 1.0 / den;
    const T rl = held(div_rn((-sr > 0.) ? -upr : -upl, den, yd), freeze_r);
    const T rr = held(div_rn((-sl > 0.) ? -upr : -upl, den, yd), freeze_r);
    /* B's tangential ratio differs from A's only when s* == 0 (or is NaN) */
    const T ret_b = (set > 0. || set < 0.) ? ret_a : held(((-set > 0.) ? upvr : upvl) / (dloc_et + eps), freeze_r);
    const T ll = waf_limiter(ilim, rl, -cr);
    const T lr = waf_limiter(ilim, rr, -cl);
    const T le = waf_limiter(ilim, ret_b, -cet);
    const T wl = halve(1. + sgnmul(-sr, ll));
    const T wlet = halve(1. + sgnmul(-set, le));
    const T wlr = halve(sgnmul(-sl, lr) - sgnmul(-sr, ll));
    const T wr = halve(1. - sgnmul(-sl, lr));
    const T wret = halve(1. - sgnmul(-set, le));
    /* mirrored physical fluxes: FL' = (-fr1, fr2), FR' = (-fl1, fl2), HLL' = (-hb1, hb2) */
    const T fw1 = -(wl * fr1 + wlr * hb1 + wr * fl1);
    const T fw2 = wl * fr2 + wlr * hb2 + wr * fl2;
    const T fw3 = -(wlet * vr + wret * vl) * fw1;
    /* B's normal is -n: (fw1, -n1 fw2 + n2 fw3, -n2 fw2 - n1 fw3) */
    F.b1 = fw1;
    F.b2 = -nx * fw2 + ny * fw3;
    F.b3 = -ny * fw2 - nx * fw3;
  }
}

/* ---- MUSCL-Hancock (IFLUX 4) ----------------------------------------------------------- */

/* simple_limiter (flux_riemann.cuf:431-463) of an upwind slope r1 and a local slope r2:
 * 0 none, 1 superbee (Fortran's three-argument max / min as two nested ones), 2 van Leer,
 * 3 minmod.  Other ilimiteur values leave the reference's result unset; defined as 0. */
template <class T>
CF_HD CF_INLINE T simple_limiter(int ilim, T r1, T r2) {
  if (ilim == 1) {
    if (r2 > 0.) return dmax(T(0.), dmax(dmin(twice(r1), r2), dmin(r1, twice(r2))));
    return dmin(T(0.), dmin(dmax(twice(r1), r2), dmax(r1, twice(r2))));
  }
  if (ilim == 2) return (r1 * r2 + fabs(r1 * r2)) / (r1 + r2 + EPS_VLEER);
  if (ilim == 3) {
    if (r2 > 0.) return dmax(T(0.), dmin(r1, r2));
    return dmin(T(0.), dmax(r1, r2));
  }
  return T(0.);
}

/* Edge-frame MUSCL-Hancock flux of the side whose element is on the left
 * (solver_Riemann_muscl, flux_riemann.cuf:526-718): limited slopes of the left state (upwind
 * difference over d_up_l, local over d_mrl) and of the right state (local, upwind over
 * d_up_r), face values, the half-step predictor, then HLLC with eps = 1e-16 (single
 * precision).  Inputs are the hydrostatically reconstructed, masked states of both elements
 * and the upwind reconstructions of both sides, all in this side's frame. */
template <class T>
CF_HD CF_INLINE void muscl_side(double g, double tolisec, int ilim, double dtoverdx, double d_mrl, double y_mrl,
                                double d_up_l, double y_up_l, double d_up_r, double y_up_r, T hl, T ul, T vl, T hr,
                                T ur, T vr, T hl_upw, T ul_upw, T vl_upw, T hr_upw, T ur_upw, T vr_upw, T& x1, T& x2,
                                T& x3) {
  const double eps = EPS_SECOND;
  /* data reconstruction I (:560-609) */
  const T dloc1 = div_rn(hr - hl, d_mrl, y_mrl);
  const T dloc2 = div_rn(ur - ul, d_mrl, y_mrl);
  const T dloc3 = div_rn(vr - vl, d_mrl, y_mrl);
  const T dhl = simple_limiter(ilim, div_rn(hl - hl_upw, d_up_l, y_up_l), dloc1);
  const T hll = dmax(T(0.), hl - halve(dhl) * d_mrl);
  const T hlr = dmax(T(0.), hl + halve(dhl) * d_mrl);
  T ull, vll, ulr, vlr;
  if (hlr < tolisec || hll < tolisec) {
    ulr = vlr = ull = vll = T(0.);
  } else {
    const T dul = simple_limiter(ilim, div_rn(ul - ul_upw, d_up_l, y_up_l), dloc2);
    const T dvl = simple_limiter(ilim, div_rn(vl - vl_upw, d_up_l, y_up_l), dloc3);
    ull = ul - halve(dul) * d_mrl;
    vll = vl - halve(dvl) * d_mrl;
    ulr = ul + halve(dul) * d_mrl;
    vlr = vl + halve(dvl) * d_mrl;
  }
  const T dhr = simple_limiter(ilim, dloc1, div_rn(hr_upw - hr, d_up_r, y_up_r));
  const T hrr = dmax(T(0.), hr + halve(dhr) * d_mrl);
  const T hrl = dmax(T(0.), hr - halve(dhr) * d_mrl);
  T url, vrl, urr, vrr;
  if (hrl < tolisec || hrr < tolisec) {
    url = vrl = urr = vrr = T(0.);
  } else {
    const T dur = simple_limiter(ilim, dloc2, div_rn(ur_upw - ur, d_up_r, y_up_r));
    const T dvr = simple_limiter(ilim, dloc3, div_rn(vr_upw - vr, d_up_r, y_up_r));
    urr = ur + halve(dur) * d_mrl;
    vrr = vr + halve(dvr) * d_mrl;
    url = ur - halve(dur) * d_mrl;
    vrl = vr - halve(dvr) * d_mrl;
  }
  /* data reconstruction II (:615-621) */
  const T h1 = hlr + 0.5 * dtoverdx * (hll * ull - hlr * ulr);
  const T u1 = ulr + 0.5 * dtoverdx *
                         (hll * (ull * ull) + 0.5 * g * (hll * hll) - (hlr * (ulr * ulr) + 0.5 * g * (hlr * hlr)));
  const T v1 = vlr + 0.5 * dtoverdx * (hll * ull * vll - hlr * ulr * vlr);
  const T h2 = hrl + 0.5 * dtoverdx * (hrl * url - hrr * urr);
  const T u2 = url + 0.5 * dtoverdx *
                         (hrl * (url * url) + 0.5 * g * (hrl * hrl) - (hrr * (urr * urr) + 0.5 * g * (hrr * hrr)));
  const T v2 = vrl + 0.5 * dtoverdx * (hrl * url * vrl - hrr * urr * vrr);
  /* HLLC (:623-714) */
  T sl, sr, set;
  if (!wave_speeds(g, eps, h1, u1, h2, u2, sl, sr, set)) {
    x1 = x2 = x3 = T(0.);
    return;
  }
  if (sl > 0.) {
    x1 = h1 * u1;
    x2 = h1 * (u1 * u1) + halve(g * h1 * h1);
    x3 = h1 * u1 * v1;
  } else if (sr < 0.) {
    x1 = h2 * u2;
    x2 = h2 * (u2 * u2) + halve(g * h2 * h2);
    x3 = h2 * u2 * v2;
  } else {
    const T fl1 = h1 * u1, fl2 = h1 * (u1 * u1) + halve(g * h1 * h1);
    const T fr1 = h2 * u2, fr2 = h2 * (u2 * u2) + halve(g * h2 * h2);
    const T den = sr - sl + eps, yden = 1.0 / den;
    x1 = div_rn(sr * fl1 - sl * fr1 + sl * sr * (h2 - h1), den, yden);
    x2 = div_rn(sr * fl2 - sl * fr2 + sl * sr * (h2 * u2 - h1 * u1), den, yden);
    x3 = (set > 0.) ? x1 * v1 : x1 * v2;
  }
}

/* Discharge of an inlet at time t: debitglob, or a linear ramp from debitglob_start. */
CF_HD CF_INLINE double inlet_discharge(const MemberDev& M, int id, double t) {
  const double q1 = M.debit_end[id - 1];
  if (M.ramp_time > 0.0 && t < M.ramp_time) {
    const double q0 = M.debit_start[id - 1];
    return q0 + (q1 - q0) * (t / M.ramp_time);
  }
  return q1;
}

/* Boundary-edge flux of side A (flux_riemann.cuf:114-171).  surf: for phys_inflow (inlet 3),
 * calcul_surf_entree's sum of length * depth over the edge's inlet at the step's start. */
template <class T>
CF_HD CF_INLINE void boundary_flux(int iflux, const MemberDev& M, int kind, int id, double t, double nx, double ny,
                                   T h, T hu, T hv, double yh, double z, T& f1, T& f2, T& f3, T& q,
                                   double surf = 0.0) {
  const double g = M.gp, tolisec = M.tolisec;
  T hautl, vitul, vitvl;
  to_frame(h, hu, hv, yh, nx, ny, tolisec, hautl, vitul, vitvl);
  f1 = f2 = f3 = T(0.0);
  q = T(0.0);
  if (kind == -1) {
    if (M.inlet == 1) {
      f1 = hautl * vitul;
      f2 = nx * (hautl * (vitul * vitul) + halve(g * (hautl * hautl))) - ny * hautl * vitul * vitvl;
      f3 = ny * (hautl * (vitul * vitul) + halve(g * (hautl * hautl))) + nx * hautl * vitul * vitvl;
    } else if (M.inlet == 2) {
      const double debitnorm = -inlet_discharge(M, id, t) / M.long_entree[id - 1];
      f1 = T(debitnorm);
      f2 = nx * ((debitnorm * debitnorm) / (hautl + tolisec) + halve(g * (hautl * hautl)));
      f3 = ny * ((debitnorm * debitnorm) / (hautl + tolisec) + halve(g * (hautl * hautl)));
      q = T(-debitnorm);
    } else if (M.inlet == 3) {
      /* the inlet's discharge shared in proportion to depth (:127-138); the threshold is the
       * single-precision literal 1e-8 */
      const T debitnorm = (surf > (double)1e-8f) ? -(inlet_discharge(M, id, t) * hautl / surf) : T(0.0);
      f1 = debitnorm;
      f2 = nx * ((debitnorm * debitnorm) / (hautl + tolisec) + halve(g * (hautl * hautl)));
      f3 = ny * ((debitnorm * debitnorm) / (hautl + tolisec) + halve(g * (hautl * hautl)));
      q = -debitnorm;
    }
  } else if (kind == -3) {
    f2 = halve(nx * g * (hautl * hautl));
    f3 = halve(ny * g * (hautl * hautl));
  } else if (kind == -2) {
    if (M.outlet == 1) {
      if (vitul >= 0. && vitul / sqrt(g * hautl) < 1.0) {
        double ho = M.h_sortie[id - 1] - z;
        ho = dmax(0.0, ho);
        f1 = ho * vitul;
        f2 = nx * (ho * (vitul * vitul) + halve(g * (ho * ho))) - ny * ho * vitul * vitvl;
        f3 = ny * (ho * (vitul * vitul) + halve(g * (ho * ho))) + nx * ho * vitul * vitvl;
      } else {
        f2 = halve(nx * g * (hautl * hautl));
        f3 = halve(ny * g * (hautl * hautl));
      }
      q = f1;
    } else {
      /* transmissive outlet: the element is its own neighbour (:169-171), raw depth on the
       * right (:173-181); second-order schemes use first-order HLLC here (their centroid
       * distance to themselves is zero). */
      const double zij = dmax(z, z);
      T hsl = dmax(T(0.0), hautl + z - zij);
      T hsr = dmax(T(0.0), ((iflux <= 2) ? h : hautl) + z - zij);
      T ul = vitul, vl = vitvl, ur = vitul, vr = vitvl;
      if (hsl < tolisec) { hsl = T(0.); ul = T(0.); vl = T(0.); }
      if (hsr < tolisec) { hsr = T(0.); ur = T(0.); vr = T(0.); }
      TwoFluxT<T> F;
      if (iflux == 2) first_order_flux<2>(g, nx, ny, hsl, ul, vl, hsr, ur, vr, F);
      else first_order_flux<1>(g, nx, ny, hsl, ul, vl, hsr, ur, vr, F);
      f1 = F.a1; f2 = F.a2; f3 = F.a3;
    }
  }
}

/* Upwind reconstruction (h, v) of one side from the states of its upwind elements
 * (flux_riemann.cuf:240-366): a copy of element 1's masked state when d1 < 0 (one upwind
 * element, or the first-order fallback), else the centroid-distance weighted average of two. */
template <class T>
CF_HD CF_INLINE void upwind_mix(T h1, T hu1, T hv1, double yh1, T h2, T hu2, T hv2, double yh2, double d1,
                                double d2, double ysum, double nx, double ny, double tolisec, T& hu_, T& vu_) {
  T a, va;
  to_frame_t(h1, hu1, hv1, yh1, nx, ny, tolisec, a, va);
  if (T(d1) < 0.0) {
    hu_ = a;
    vu_ = va;
    return;
  }
  T b, vb;
  to_frame_t(h2, hu2, hv2, yh2, nx, ny, tolisec, b, vb);
  const double ds = d1 + d2;
  hu_ = div_rn(d1 * a + d2 * b, ds, ysum);
  vu_ = div_rn(d1 * va + d2 * vb, ds, ysum);
}

/* The bed elevation of an upwind reconstruction (flux_riemann.cuf:320-366): static, so the host
 * preprocessing evaluates it once per edge side. */
CF_HD CF_INLINE double upwind_bed(double z1, double z2, double d1, double d2, double ysum) {
  return (d1 < 0.0) ? z1 : div_rn(d1 * z1 + d2 * z2, d1 + d2, ysum);
}

/* The same, loading the elements' states (w = RN(1/h)), in the edge's arithmetic type T. */
template <class T>
CF_HD CF_INLINE void upwind_state(const double4* U, int i1, int i2, double d1, double d2, double ysum, double nx,
                                  double ny, double tolisec, T& hu_, T& vu_) {
  const double4 A1 = ld4(U + i1);
  if (T(d1) < 0.0) {
    upwind_mix(T(A1.x), T(A1.y), T(A1.z), A1.w, T(0.0), T(0.0), T(0.0), 0.0, d1, d2, ysum, nx, ny, tolisec, hu_,
               vu_);
    return;
  }
  const double4 A2 = ld4(U + i2);
  upwind_mix(T(A1.x), T(A1.y), T(A1.z), A1.w, T(A2.x), T(A2.y), T(A2.z), A2.w, d1, d2, ysum, nx, ny, tolisec, hu_,
             vu_);
}

/* The MUSCL form: (h, u_n, u_t) of one side's upwind reconstruction (flux_riemann.cuf:240-366
 * with the normal velocity as well). */
template <class T>
CF_HD CF_INLINE void upwind_state3(const double4* U, int i1, int i2, double d1, double d2, double ysum, double nx,
                                   double ny, double tolisec, T& hu_, T& uu_, T& vu_) {
  const double4 A1 = ld4(U + i1);
  T a, ua, va;
  to_frame(T(A1.x), T(A1.y), T(A1.z), A1.w, nx, ny, tolisec, a, ua, va);
  if (T(d1) < 0.0) {
    hu_ = a;
    uu_ = ua;
    vu_ = va;
    return;
  }
  const double4 A2 = ld4(U + i2);
  T b, ub, vb;
  to_frame(T(A2.x), T(A2.y), T(A2.z), A2.w, nx, ny, tolisec, b, ub, vb);
  const double ds = d1 + d2;
  hu_ = div_rn(d1 * a + d2 * b, ds, ysum);
  uu_ = div_rn(d1 * ua + d2 * ub, ds, ysum);
  vu_ = div_rn(d1 * va + d2 * vb, ds, ysum);
}

/* ---- one edge ------------------------------------------------------------------------- */

/* Static data of an interior edge beyond its normal: length, centroid distance and, for the
 * second-order scheme, the upwind distances and reciprocals. */
struct EdgeGeo {
  double nx, ny, len, d_mrl;
  double y_mrl, d_mkvol, y_mkvol, d_mkvoisin, y_mkvoisin;
  double ysum_a, ysum_b;  /* RN(1/(d1+d2)) of the upwind pairs of sides A and B */
};

/* Both sides' slot values of an interior edge: out[0..4] = side A {f1, f2, f3} * len and its
 * bed source {bx, by}; out[5..9] the same for side B.  hl_upw .. vr_upw are the upwind
 * reconstructions of sides A and B (second order only), zl_upw / zr_upw their bed elevations. */
template <int IFLUX, class T>
CF_HD CF_INLINE void interior_edge(const MemberDev& M, int ilim, int flux_mode, const EdgeGeo& G, double dt, T hA,
                                   T huA, T hvA, double zml, double yhA, T hB, T huB, T hvB, double zmr, double yhB,
                                   T hl_upw, T vl_upw, double zl_upw, T hr_upw, T vr_upw, double zr_upw, T out[10],
                                   bool freeze_r = false) {
  const double g = M.gp, tolisec = M.tolisec;
  const double nx = G.nx, ny = G.ny, len = G.len;
  const double zij = val(dmax(T(zml), T(zmr)));
  T hautl, vitul, vitvl, hautr, vitur, vitvr;
  to_frame(hA, huA, hvA, yhA, nx, ny, tolisec, hautl, vitul, vitvl);
  to_frame(hB, huB, hvB, yhB, nx, ny, tolisec, hautr, vitur, vitvr);
  TwoFluxT<T> F;
  if (IFLUX <= 2) {
    /* hydrostatic reconstruction (:176-181, :200-210): A from its masked depth, B from its
     * raw depth; the raw and masked depths differ only for 0 < h <= tolisec, where side B's
     * own evaluation (B masked, A raw) is computed separately. */
    T hijet = dmax(T(0.0), hautl + zml - zij);
    T hjiet = dmax(T(0.0), hB + zmr - zij);
    T ul = vitul, vl = vitvl, ur = vitur, vr = vitvr;
    if (hijet < tolisec) { hijet = T(0.); ul = T(0.); vl = T(0.); }
    if (hjiet < tolisec) { hjiet = T(0.); ur = T(0.); vr = T(0.); }
    first_order_flux<IFLUX>(g, nx, ny, hijet, ul, vl, hjiet, ur, vr, F);
    if (hautl != hA || hautr != hB) {
      T bl = dmax(T(0.0), hautr + zmr - zij), br = dmax(T(0.0), hA + zml - zij);
      T bul = -vitur, bvl = -vitvr, bur = -vitul, bvr = -vitvl;
      if (bl < tolisec) { bl = T(0.); bul = T(0.); bvl = T(0.); }
      if (br < tolisec) { br = T(0.); bur = T(0.); bvr = T(0.); }
      TwoFluxT<T> Gm;
      first_order_flux<IFLUX>(g, -nx, -ny, bl, bul, bvl, br, bur, bvr, Gm);
      F.b1 = Gm.a1;
      F.b2 = Gm.a2;
      F.b3 = Gm.a3;
    }
  } else {
    /* hydrostatic reconstruction of the four states (:370-400) */
    T hijet = dmax(T(0.0), hautl + zml - zij);
    T hlu = dmax(T(0.0), hl_upw + zl_upw - zij);
    T hjiet = dmax(T(0.0), hautr + zmr - zij);
    T hru = dmax(T(0.0), hr_upw + zr_upw - zij);
    T ul = vitul, vl = vitvl, ur = vitur, vr = vitvr, vlu = vl_upw, vru = vr_upw;
    if (hijet < tolisec) { hijet = T(0.); ul = T(0.); vl = T(0.); }
    if (hlu < tolisec) { hlu = T(0.); vlu = T(0.); }
    if (hjiet < tolisec) { hjiet = T(0.); ur = T(0.); vr = T(0.); }
    if (hru < tolisec) { hru = T(0.); vru = T(0.); }
    waf_flux(g, ilim, nx, ny, dt, G.d_mrl, G.y_mrl, G.d_mkvol, G.y_mkvol, G.d_mkvoisin, G.y_mkvoisin, hijet, ul, vl,
             hjiet, ur, vr, hlu, vlu, hru, vru, F, freeze_r);
  }
  if (flux_mode == 1) {
    F.b1 = -F.a1;
    F.b2 = -F.a2;
    F.b3 = -F.a3;
  }
  /* bed-slope source of both sides from the raw depths (source_terms.cuf:90-97) */
  const T ha = dmax(T(0.0), hA + zml - zij);
  const T hb = dmax(T(0.0), hB + zmr - zij);
  const T ta = g / 2.0 * (ha * ha - hA * hA) * len;
  const T tb = g / 2.0 * (hb * hb - hB * hB) * len;
  out[0] = F.a1 * len;
  out[1] = F.a2 * len;
  out[2] = F.a3 * len;
  out[3] = ta * nx;
  out[4] = ta * ny;
  out[5] = F.b1 * len;
  out[6] = F.b2 * len;
  out[7] = F.b3 * len;
  out[8] = -(tb * nx);
  out[9] = -(tb * ny);
}

/* interior_edge for MUSCL-Hancock (IFLUX 4): the reference evaluates the edge from each of its
 * elements in that element's frame.  Side B's frame normal is -n, so its inputs are A's
 * frame values with the elements swapped and the velocities negated, which is what B's own
 * masking and upwind averaging produce; each side's limited reconstruction is evaluated in
 * full (its slopes are not mirror images of the other side's).  upA / upB: (h, u_n, u_t) of
 * the upwind reconstructions of sides A and B in A's frame, zl_upw / zr_upw their beds. */
template <class T>
CF_HD CF_INLINE void interior_edge_muscl(const MemberDev& M, int ilim, int flux_mode, const EdgeGeo& G, double dt,
                                         T hA, T huA, T hvA, double zml, double yhA, T hB, T huB, T hvB, double zmr,
                                         double yhB, const T upA[3], double zl_upw, const T upB[3], double zr_upw,
                                         T out[10]) {
  const double g = M.gp, tolisec = M.tolisec;
  const double nx = G.nx, ny = G.ny, len = G.len;
  const double zij = val(dmax(T(zml), T(zmr)));
  T hautl, vitul, vitvl, hautr, vitur, vitvr;
  to_frame(hA, huA, hvA, yhA, nx, ny, tolisec, hautl, vitul, vitvl);
  to_frame(hB, huB, hvB, yhB, nx, ny, tolisec, hautr, vitur, vitvr);
  /* hydrostatic reconstruction of the four states (:370-400) */
  T hijet = dmax(T(0.0), hautl + zml - zij);
  T hlu = dmax(T(0.0), upA[0] + zl_upw - zij);
  T hjiet = dmax(T(0.0), hautr + zmr - zij);
  T hru = dmax(T(0.0), upB[0] + zr_upw - zij);
  T ul = vitul, vl = vitvl, ur = vitur, vr = vitvr;
  T ulu = upA[1], vlu = upA[2], uru = upB[1], vru = upB[2];
  if (hijet < tolisec) { hijet = T(0.); ul = T(0.); vl = T(0.); }
  if (hlu < tolisec) { hlu = T(0.); ulu = T(0.); vlu = T(0.); }
  if (hjiet < tolisec) { hjiet = T(0.); ur = T(0.); vr = T(0.); }
  if (hru < tolisec) { hru = T(0.); uru = T(0.); vru = T(0.); }
  const double dtoverdx = div_rn(dt, G.d_mrl, G.y_mrl);
  TwoFluxT<T> F;
  T x1, x2, x3;
  muscl_side(g, tolisec, ilim, dtoverdx, G.d_mrl, G.y_mrl, G.d_mkvol, G.y_mkvol, G.d_mkvoisin, G.y_mkvoisin, hijet,
             ul, vl, hjiet, ur, vr, hlu, ulu, vlu, hru, uru, vru, x1, x2, x3);
  F.a1 = x1;
  F.a2 = nx * x2 - ny * x3;
  F.a3 = ny * x2 + nx * x3;
  if (flux_mode == 1) {
    F.b1 = -F.a1;
    F.b2 = -F.a2;
    F.b3 = -F.a3;
  } else {
    T y1, y2, y3;
    muscl_side(g, tolisec, ilim, dtoverdx, G.d_mrl, G.y_mrl, G.d_mkvoisin, G.y_mkvoisin, G.d_mkvol, G.y_mkvol,
               hjiet, -ur, -vr, hijet, -ul, -vl, hru, -uru, -vru, hlu, -ulu, -vlu, y1, y2, y3);
    const double mx = -nx, my = -ny;
    F.b1 = y1;
    F.b2 = mx * y2 - my * y3;
    F.b3 = my * y2 + mx * y3;
  }
  /* bed-slope source of both sides from the raw depths (source_terms.cuf:90-97) */
  const T ha = dmax(T(0.0), hA + zml - zij);
  const T hb = dmax(T(0.0), hB + zmr - zij);
  const T ta = g / 2.0 * (ha * ha - hA * hA) * len;
  const T tb = g / 2.0 * (hb * hb - hB * hB) * len;
  out[0] = F.a1 * len;
  out[1] = F.a2 * len;
  out[2] = F.a3 * len;
  out[3] = ta * nx;
  out[4] = ta * ny;
  out[5] = F.b1 * len;
  out[6] = F.b2 * len;
  out[7] = F.b3 * len;
  out[8] = -(tb * nx);
  out[9] = -(tb * ny);
}

/* Static data of edge e in the form interior_edge takes. */
CF_HD CF_INLINE EdgeGeo edge_geo(const StepArgs& a, int e, bool second, const double4& geo) {
  EdgeGeo G;
  G.nx = geo.x;
  G.ny = geo.y;
  G.len = geo.z;
  G.d_mrl = geo.w;
  G.y_mrl = G.d_mkvol = G.y_mkvol = G.d_mkvoisin = G.y_mkvoisin = G.ysum_a = G.ysum_b = 0.0;
  if (second) {
    const double4 dk = ld4(a.edk + e);    /* d_mkvol, d_mkvoisin and their reciprocals */
    const double4 yi = ld4(a.einv + e);   /* 1/d_mrl, 1/(d1+d2) of A and of B */
    G.y_mrl = yi.x;
    G.d_mkvol = dk.x;
    G.y_mkvol = dk.z;
    G.d_mkvoisin = dk.y;
    G.y_mkvoisin = dk.w;
    G.ysum_a = yi.y;
    G.ysum_b = yi.z;
  }
  return G;
}
CF_HD CF_INLINE EdgeGeo edge_geo(const StepArgs& a, int e, bool second) { return edge_geo(a, e, second, ld4(a.egeo + e)); }

/* One slot's six values.  On the device three 16-byte stores: every slot array starts on a
 * 256-byte boundary (cudaMalloc, the no-allocation scratch) and a slot is 48 bytes, so every slot
 * starts on a 16-byte boundary.  On the host (the CPU harness) plain stores. */
CF_HD CF_INLINE void store_slot(Slot* p, double f1, double f2, double f3, double bx, double by, double q) {
#ifdef __CUDA_ARCH__
  double2* d = reinterpret_cast<double2*>(p);
  d[0] = make_double2(f1, f2);
  d[1] = make_double2(f3, bx);
  d[2] = make_double2(by, q);
#else
  p->f1 = f1;
  p->f2 = f2;
  p->f3 = f3;
  p->bx = bx;
  p->by = by;
  p->q = q;
#endif
}

/* The two slots of an interior edge from interior_edge's out[10]. */
CF_HD CF_INLINE void write_slots(Slot* sa, const double o[10]) {
  store_slot(sa, o[0], o[1], o[2], o[3], o[4], 0.0);
  store_slot(sa + 1, o[5], o[6], o[7], o[8], o[9], 0.0);
}

/* ---- dry regions ------------------------------------------------------------------------ */

CF_HD CF_INLINE uint64_t dbits_hd(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
}
CF_HD CF_INLINE double dbl_hd(uint64_t b) {
  double x;
  memcpy(&x, &b, sizeof(x));
  return x;
}

/* The two slots of an interior edge whose elements both hold the depth +0 (bit pattern 0), written
 * without evaluating the edge.  The general evaluation gives, for any bed elevations and any upwind
 * states:
 *   - masked depths 0, hydrostatic depths max(0, (+0 + z) - max(z, z')) = +0 (the difference is
 *     <= 0 or NaN, and max(0, .) returns the +0 operand); the first-order and WAF schemes
 *     (IFLUX 1-3) then see both depths below eps and assign +0 to every component of both sides'
 *     flux vectors (the second first-order evaluation is skipped: masked and raw depths agree);
 *   - MUSCL-Hancock (IFLUX 4): the local slopes are (+0 - +0) / d = +0, each limited slope is +0 (the
 *     limiters return their +0 operand for a +0 local slope and an upwind slope of either sign; a
 *     NaN slope of van Leer's 0 / 0 is removed by the max with 0), so the face depths, the clamped
 *     face velocities and the predicted states are +0 and the wave-speed routine gives the frame
 *     flux (+0, +0, +0); rotated back, a2 = nx 0 - ny 0, a3 = ny 0 + nx 0 (side B with -n), signed
 *     zeros formed here by the same operations (the time step must be finite);
 *   - with flux_mode 1 side B's fluxes are the negated side A's;
 *   - the bed source (g/2 (ha^2 - h^2)) len with ha = h = +0: (g/2 * +0) * len, a zero with the
 *     sign of g times the sign of len, then times nx, ny (side B negated).
 * Every product of a zero and a finite number is the zero with the product of the signs, so the
 * slots are these signed zeros whenever g, len, nx and ny are finite; otherwise (returns false)
 * the caller evaluates the edge. */
template <int IFLUX>
CF_HD CF_INLINE bool dry_edge_slots(double g, int flux_mode, const double4& geo, Slot* sa, double dt = 0.0) {
  const uint64_t S = 0x8000000000000000ull;
  const uint64_t bg = dbits_hd(g), bnx = dbits_hd(geo.x), bny = dbits_hd(geo.y), bl = dbits_hd(geo.z);
  if (!(finite_u(bg) & finite_u(bnx) & finite_u(bny) & finite_u(bl))) return false;
  if (IFLUX == 4 && !finite_u(dbits_hd(dt))) return false;
  const uint64_t sl = bl & S;                              /* the sign of len */
  const uint64_t st = (bg & S) ^ sl;                       /* ta = tb = (g/2 * +0) * len */
  /* the flux vectors (before * len): side A's frame flux rotated by n, side B's by -n */
  uint64_t a1 = 0, a2 = 0, a3 = 0, b1 = 0, b2 = 0, b3 = 0;
  if (IFLUX == 4) {
    const double x = geo.x * 0.0, y = geo.y * 0.0, mx = (-geo.x) * 0.0, my = (-geo.y) * 0.0;
    a2 = dbits_hd(x - y);
    a3 = dbits_hd(y + x);
    b2 = dbits_hd(mx - my);
    b3 = dbits_hd(my + mx);
  }
  if (flux_mode == 1) {
    b1 = a1 ^ S;
    b2 = a2 ^ S;
    b3 = a3 ^ S;
  }
  store_slot(sa, dbl_hd((a1 & S) ^ sl), dbl_hd((a2 & S) ^ sl), dbl_hd((a3 & S) ^ sl), dbl_hd(st ^ (bnx & S)),
             dbl_hd(st ^ (bny & S)), 0.0);
  store_slot(sa + 1, dbl_hd((b1 & S) ^ sl), dbl_hd((b2 & S) ^ sl), dbl_hd((b3 & S) ^ sl),
             dbl_hd(st ^ (bnx & S) ^ S), dbl_hd(st ^ (bny & S) ^ S), 0.0);
  return true;
}

/* An element area for which a dry element's update is exact zeros: a positive normal number (the
 * sign bit fails the test). */
CF_HD CF_INLINE bool area_ok(double area) {
  uint32_t lo, hi;
  words_u(dbits_hd(area), lo, hi);
  (void)lo;
  return (hi >> 20) - 1u < 2046u;
}

/* The conditions on the element's state and the member under which a dry element's update is
 * (+0, +0, +0, +0), besides area_ok: its depth is +-0, its discharges are finite, dt is finite and
 * tolisec >= 0. */
CF_HD CF_INLINE bool dry_state_ok(const MemberDev& M, const double4& U, double dt) {
  uint32_t tlo, thi;
  words_u(dbits_hd(M.tolisec), tlo, thi);
  /* +0..+inf: sign clear, magnitude at most the infinity's */
  const bool tol_ok = (thi >> 31) == 0 && (thi < 0x7ff00000u || (thi == 0x7ff00000u && tlo == 0));
  return zero_u(dbits_hd(U.x)) && tol_ok && finite_u(dbits_hd(U.y)) && finite_u(dbits_hd(U.z)) &&
         finite_u(dbits_hd(dt));
}

/* The conditions on the element itself under which a dry element's update is (+0, +0, +0, +0). */
CF_HD CF_INLINE bool dry_element_state(const MemberDev& M, const double4& U, const double4& st, double dt) {
  return area_ok(st.x) && dry_state_ok(M, U, dt);
}

/* True when the general update of an element provably returns the state (+0, +0, +0, +0) without
 * flagging it non-finite: dry_element_state holds and every flux and bed-source component of its
 * three slots is +-0.  Then every residual (0 + 0 - rc) / area and (sb + sf - rc) / area is +0 (the
 * friction source of a dry element is +0), each new component is the old one plus +-0 (finite),
 * and the new depth +-0 <= tolisec clamps the state to +0. */
CF_HD CF_INLINE bool dry_element(const MemberDev& M, const double4& U, const double4& st, const Slot& s0,
                                 const Slot& s1, const Slot& s2, double dt) {
  const uint64_t z = (dbits_hd(s0.f1) | dbits_hd(s0.f2) | dbits_hd(s0.f3) | dbits_hd(s0.bx) | dbits_hd(s0.by) |
                      dbits_hd(s1.f1) | dbits_hd(s1.f2) | dbits_hd(s1.f3) | dbits_hd(s1.bx) | dbits_hd(s1.by) |
                      dbits_hd(s2.f1) | dbits_hd(s2.f2) | dbits_hd(s2.f3) | dbits_hd(s2.bx) | dbits_hd(s2.by)) << 1;
  return z == 0 && dry_element_state(M, U, st, dt);
}

/* True when an element's three slots are signed zeros without reading them: nb (cnbr) flags three
 * interior edges with finite normals and lengths (and an area for which area_ok holds), the
 * member's g is finite, and the element and its three neighbours have depth +0 (bits 0), so that
 * every one of its edges took the edge kernel's dry shortcut (edge_body, dry_edge_slots; the
 * element kernel reads the same state and dt).  With dry_state_ok it gives dry_element's answer. */
template <class Ld>
CF_HD CF_INLINE bool dry_neighbourhood(const MemberDev& M, const int4& nb, const double4& U, Ld h_of) {
  if (!(nb.w && dbits_hd(U.x) == 0 && finite_u(dbits_hd(M.gp)))) return false;
  return (dbits_hd(h_of(nb.x)) | dbits_hd(h_of(nb.y)) | dbits_hd(h_of(nb.z))) == 0;
}

/* Fluxes (times the edge length) and bed sources of edge e into its two slots, from the
 * state U of step n: the body of the edge kernel. */
template <int IFLUX, class S = double>
CF_HD CF_INLINE void edge_body(const StepArgs& a, const MemberDev& M, int e, double dt, double t,
                               const double* surf = nullptr) {
  const int2 ab = ldro(a.ecell + e);
  /* the normal and length, which every path needs, load beside the element states (a dry edge
   * then waits for two memory round trips, not three) */
  const double4 geo = ld4(a.egeo + e);
  const double4 UA = ld4(a.Uin + ab.x);   /* {h, hu, hv, RN(1/h)} */
  Slot* sa = a.slots + 2 * (size_t)e;

  if (ab.y >= 0) {
    /* an edge between two dry elements (most of a flood plain that the water has not reached)
     * needs neither its geometry beyond the normal nor its upwind states */
    const double hB = ldro(reinterpret_cast<const double*>(a.Uin + ab.y));
    if ((dbits_hd(UA.x) | dbits_hd(hB)) == 0 && dry_edge_slots<IFLUX>(M.gp, a.flux_mode, geo, sa, dt)) return;
  }
  const double4 ez = ld4(a.ez + e);       /* bed of A, of B, of A's and B's upwind reconstructions */

  if (ab.y < 0) {
    const double len = geo.z;
    const int id = ldro(a.ebid + e);
    const double sf = (surf && ab.y == -1 && M.inlet == 3 && id >= 1 && id <= M.nin) ? surf[id - 1] : 0.0;
    double f1, f2, f3, q;
    boundary_flux(IFLUX, M, ab.y, id, t, geo.x, geo.y, UA.x, UA.y, UA.z, UA.w, ez.x, f1, f2, f3, q, sf);
    store_slot(sa, f1 * len, f2 * len, f3 * len, 0.0, 0.0, q * len);
    return;
  }

  const EdgeGeo G = edge_geo(a, e, IFLUX >= 3, geo);
  const double4 UB = ld4(a.Uin + ab.y);
  double o[10];
  if (IFLUX == 4) {
    const int4 up = ldro(a.eupw + e);
    const double4 dw = ld4(a.ewts + e);
    S upA[3], upB[3], om[10];
    upwind_state3(a.Uin, up.x, up.y, dw.x, dw.y, G.ysum_a, G.nx, G.ny, M.tolisec, upA[0], upA[1], upA[2]);
    upwind_state3(a.Uin, up.z, up.w, dw.z, dw.w, G.ysum_b, G.nx, G.ny, M.tolisec, upB[0], upB[1], upB[2]);
    interior_edge_muscl(M, a.ilimiteur, a.flux_mode, G, dt, S(UA.x), S(UA.y), S(UA.z), ez.x, UA.w, S(UB.x), S(UB.y),
                        S(UB.z), ez.y, UB.w, upA, ez.z, upB, ez.w, om);
#pragma unroll
    for (int i = 0; i < 10; ++i) o[i] = val(om[i]);
    write_slots(sa, o);
    return;
  }
  S hl_upw = S(0.0), vl_upw = S(0.0), hr_upw = S(0.0), vr_upw = S(0.0);
  if (IFLUX == 3) {
    const int4 up = ldro(a.eupw + e);
    const double4 dw = ld4(a.ewts + e);   /* d1, d2 of side A, d1, d2 of side B */
    upwind_state(a.Uin, up.x, up.y, dw.x, dw.y, G.ysum_a, G.nx, G.ny, M.tolisec, hl_upw, vl_upw);
    upwind_state(a.Uin, up.z, up.w, dw.z, dw.w, G.ysum_b, G.nx, G.ny, M.tolisec, hr_upw, vr_upw);
  }
  S os[10];
  interior_edge<(IFLUX == 4 ? 3 : IFLUX)>(M, a.ilimiteur, a.flux_mode, G, dt, S(UA.x), S(UA.y), S(UA.z), ez.x,
                                          UA.w, S(UB.x), S(UB.y), S(UB.z), ez.y, UB.w, hl_upw, vl_upw, ez.z, hr_upw,
                                          vr_upw, ez.w, os);
#pragma unroll
  for (int i = 0; i < 10; ++i) o[i] = val(os[i]);
  write_slots(sa, o);
}

/* ---- one element ------------------------------------------------------------------------ */

/* CFL time step of one element (cfl_condition.cuf:20-37); cflL = cfl * L_cfl. */
CF_HD CF_INLINE double cfl_dt_elem(const MemberDev& M, double cflL, double h, double hu, double hv, double yh) {
  double d = 1000000.0;
  if (h > M.tolisec) {
    const double vu = div_rn(hu, h, yh), vv = div_rn(hv, h, yh);
    const double nv = sqrt(vu * vu + vv * vv);
    const double vmax = dmax(0.01, nv + sqrt(M.gp * fabs(h)));
    d = dmin(cflL / vmax, 1000000.0);
  }
  if (M.is_dt_constant == 1) d = M.constant_dt;
  return d;
}

/* Manning friction of one element (source_terms.cuf:102-210): the source (sf2, sf3) of its
 * state q and the entries m = {m4, m5, m6, m7, m8, m9} of the rows 2 and 3 of the
 * semi-implicit matrix (I - dt/2 J)^-1 (row 1 is (1, 0, 0)).  A dry element, or
 * fricimplic 0, gives m = {0, 1, 0, 0, 0, 1}. */
template <class T>
CF_HD CF_INLINE void friction_terms(const MemberDev& M, double area, double dt, T manning, T q1, T q2, T q3, T& sf2,
                                    T& sf3, T m[6], double yq1) {
  const double gp = M.gp, tolisec = M.tolisec, tol = M.tol;
  sf2 = T(0.);
  sf3 = T(0.);
  m[0] = T(0.); m[1] = T(1.); m[2] = T(0.); m[3] = T(0.); m[4] = T(0.); m[5] = T(1.);
  if (q1 > tolisec) {
    const T yq = recip_h(q1, yq1);
    const T vitu = div_rn(q2, q1, yq), vitv = div_rn(q3, q1, yq);
    T normvit = sqrt(vitu * vitu + vitv * vitv);
    if (normvit < tol) normvit = T(tol);
    const T p13 = rcbrt(q1);                /* q1**(-1/3) */
    sf2 = -(gp * manning * manning * vitu * normvit * area * p13);
    sf3 = -(gp * manning * manning * vitv * normvit * area * p13);
    if (normvit > tol) {
      const T p43 = div_rn(p13, q1, yq);     /* q1**(-4/3) */
      if (M.fricimplic == 1) {
        const T yn = 1.0 / normvit;
        const T dtgn2h = dt / 2.0 * gp * manning * manning * p43;
        const T af21 = -(7.0 / 3.0 * dtgn2h * vitu * normvit);
        const T af22 = 1.0 + div_rn(dtgn2h * (twice(vitu * vitu) + vitv * vitv), normvit, yn);
        const T af23 = div_rn(dtgn2h * vitu * vitv, normvit, yn);
        const T af31 = -(7.0 / 3.0 * dtgn2h * vitv * normvit);
        const T af32 = af23;
        const T af33 = 1.0 + div_rn(dtgn2h * (vitu * vitu + twice(vitv * vitv)), normvit, yn);
        const T detaf = af22 * af33 - af23 * af32;
        const T yd = 1.0 / detaf;
        m[0] = div_rn(-(af21 * af33 - af23 * af31), detaf, yd);
        m[1] = div_rn(af33, detaf, yd);
        m[2] = div_rn(-af23, detaf, yd);
        m[3] = div_rn(af21 * af32 - af22 * af31, detaf, yd);
        m[4] = div_rn(-af32, detaf, yd);
        m[5] = div_rn(af22, detaf, yd);
      } else if (M.fricimplic == 2) {
        const T beta = -(dt * gp * manning * manning * normvit * p43);
        const T detaf = (1. - beta) * (1. - beta);
        m[1] = (1. - beta) / detaf;
        m[5] = (1. - beta) / detaf;
      }
    }
  }
}

/* Sources, friction and update of one element (source_terms.cuf:33-211,
 * finite_volumes_method.cuf:283-303) from its state q, the sums rc of its three edge fluxes
 * and sb of its bed sources, its area (and RN(1/area)) and its Manning n.  The wet/dry clamp
 * of the new depth is part of the map. */
template <class T>
CF_HD CF_INLINE void element_core(const MemberDev& M, double area, double yarea, T manning, T q1, T q2, T q3, T rc1,
                                  T rc2, T rc3, T sb2, T sb3, double dt, T& h, T& hu, T& hv, bool& nonfinite,
                                  double yq1) {
  T r1, r2, r3;
  if (M.friction == 1) {
    T sf2, sf3, m[6];
    friction_terms(M, area, dt, manning, q1, q2, q3, sf2, sf3, m, yq1);
    const T ri1 = div_rn(0. + 0. - rc1, area, yarea);
    const T ri2 = div_rn(sb2 + sf2 - rc2, area, yarea);
    const T ri3 = div_rn(sb3 + sf3 - rc3, area, yarea);
    if (M.fricimplic == 1 || M.fricimplic == 2) {
      r1 = 1. * ri1 + 0. * ri2 + 0. * ri3;
      r2 = m[0] * ri1 + m[1] * ri2 + m[2] * ri3;
      r3 = m[3] * ri1 + m[4] * ri2 + m[5] * ri3;
    } else {
      r1 = ri1;
      r2 = ri2;
      r3 = ri3;
    }
  } else {
    r1 = div_rn(0. - rc1, area, yarea);
    r2 = div_rn(sb2 - rc2, area, yarea);
    r3 = div_rn(sb3 - rc3, area, yarea);
  }
  h = q1 + dt * r1;
  hu = q2 + dt * r2;
  hv = q3 + dt * r3;
  nonfinite = !(finite_bits(val(h)) && finite_bits(val(hu)) && finite_bits(val(hv)));
  if (h <= M.tolisec) {
    h = T(0.);
    hu = T(0.);
    hv = T(0.);
  }
}

/* The element kernel's general body (element_update without its dry-region shortcut). */
template <class S = double>
CF_HD CF_INLINE double4 element_update_full(const MemberDev& M, const double4 U, const double4 st, const Slot& s0,
                                            const Slot& s1, const Slot& s2, double dt, bool& nonfinite) {
  /* fixed-order sums over the three edges (flux_riemann.cuf:411-426, source_terms.cuf:54-100) */
  const double rc1 = s0.f1 + s1.f1 + s2.f1;
  const double rc2 = s0.f2 + s1.f2 + s2.f2;
  const double rc3 = s0.f3 + s1.f3 + s2.f3;
  const double sb2 = s0.bx + s1.bx + s2.bx;
  const double sb3 = s0.by + s1.by + s2.by;
  S h, hu, hv;
  element_core(M, st.x, st.w, S(st.y), S(U.x), S(U.y), S(U.z), S(rc1), S(rc2), S(rc3), S(sb2), S(sb3), dt, h, hu,
               hv, nonfinite, U.w);
  /* the new state carries RN(1/h) for the next step's quotients by h */
  const double hn = val(h);
  return make_double4(hn, val(hu), val(hv), hn > 0.0 ? val(S(1.0) / h) : 0.0);
}

/* The element kernel's body: st = {area, manning n, cfl*L_cfl, 1/area}.  Returns the new
 * state; sets *nonfinite when it is not finite. */
template <class S = double>
CF_HD CF_INLINE double4 element_update(const MemberDev& M, const double4 U, const double4 st, const Slot& s0,
                                       const Slot& s1, const Slot& s2, double dt, bool& nonfinite) {
  if (dry_element(M, U, st, s0, s1, s2, dt)) {
    /* a dry element that no water reaches this step (its edges carry no flux) */
    nonfinite = false;
    return make_double4(0.0, 0.0, 0.0, 0.0);
  }
  return element_update_full<S>(M, U, st, s0, s1, s2, dt, nonfinite);
}

}  // namespace cf

#endif
