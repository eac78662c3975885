/*
 * cf_xd.h -- binary64 arithmetic that keeps GB300's FP64 pipe for the operations only it can do.
 *
 * GB300 issues two FP64 operations per clock per SM; its integer pipes issue ~30x more 32-bit
 * operations, run beside the FP64 pipe, and sit idle in an all-FP64 step (ncu: FP64 pipe 85 %
 * busy, ALU 1.4 %).  Exact substitutions move FP64-pipe work onto them:
 *
 *   comparisons  x < y etc. on ordered integer keys of the bit patterns (negative values
 *                mirrored, -0 and +0 one key, NaN compares false): the IEEE result, on the ALU;
 *   products     x * y by integer multiplication of the significands with round to nearest
 *                even (em_mul);
 *   quotients    a / b from a float reciprocal seed, a fixed-point refinement and the exact
 *                remainder, which decides the rounding (em_div);
 *   roots        sqrt(x) the same way from a float reciprocal-root seed (em_sqrt);
 *   scalings     x / 2, x / 4, 2 x and negation as exponent-field and sign-bit operations.
 * Each takes the FP64 instruction (out of line, so that the compiler does not evaluate it
 * speculatively on the fast path) wherever the integer path does not cover the case: a zero,
 * subnormal, infinite or NaN operand (a zero numerator of em_div is covered), a result outside
 * the normal range, and, for em_div and em_sqrt, a remainder check that fails.
 *
 * XD<MUL, OC> is a double that compares on integer keys and, with MUL, multiplies, divides (div_rn
 * included) and takes square roots with em_mul, em_div and em_sqrt; sums stay FP64
 * instructions.  Every result is the IEEE binary64 result of the same operation, so code
 * instantiated on XD<...> rounds exactly like the same code on double; which warps use the
 * integer arithmetic is a tuning choice, not a numerical one.
 */
#ifndef CF_XD_H
#define CF_XD_H

#include "cf_flux.h"

#ifdef __CUDACC__
#define XD_HD __host__ __device__ __forceinline__
#define XD_NOINLINE static __host__ __device__ __noinline__
#else
#define XD_HD inline
#define XD_NOINLINE static __attribute__((noinline))
#endif

namespace cf {

using ::fabs;
using ::sqrt;

XD_HD uint64_t xbits(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
}
XD_HD double xdbl(uint64_t b) {
  double x;
  memcpy(&x, &b, sizeof(x));
  return x;
}

XD_HD uint64_t xmulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

/* the FP64 instruction, for the operands and results the integer path does not cover */
XD_NOINLINE double xmul_slow(double a, double b) { return a * b; }

/* a * b, round to nearest even, in integer arithmetic (normal operands, normal result).  Out of
 * line: the edge kernel makes ~60 products per edge, and inlining each one multiplies the size of
 * a kernel whose instruction working set is already large (measured: WAF edge kernel 0.609 ms
 * inlined, 0.545 ms called, 1M triangles). */
XD_NOINLINE double em_mul(double a, double b) {
  const uint64_t ua = xbits(a), ub = xbits(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) return xmul_slow(a, b);
  const uint64_t M = (1ull << 52) - 1;
  const uint64_t ma = ((ua & M) | (1ull << 52)) << 11, mb = ((ub & M) | (1ull << 52)) << 1;
  const uint64_t hi = xmulhi(ma, mb);  /* the product's bits from 2^52 up: 53 or 54 bits */
  const uint64_t lo = ma * mb;         /* the product's bits below 2^52, shifted left by 12 */
  const uint32_t top = (uint32_t)(hi >> 53);
  const int e = (int)ea + (int)eb - 1023 + (int)top;
  uint64_t mant = hi >> top;
  const uint64_t rb = top ? (hi & 1u) : (lo >> 63);
  const uint64_t sticky = top ? (lo != 0) : ((lo << 1) != 0);
  mant += rb & (sticky | (mant & 1u));
  if ((uint32_t)(e - 1) >= 2046u) return xmul_slow(a, b);
  return xdbl((((uint64_t)(e - 1) << 52) + mant) | ((ua ^ ub) & (1ull << 63)));
}

/* the FP64 quotient, for the operands and results the integer path does not cover */
XD_NOINLINE double xdiv_slow(double a, double b) { return a / b; }

/* bits of an approximation to 1/f, f in [1, 2): on the device the single-precision reciprocal
 * (rcp.approx.ftz.f32, error at most one unit in the last place); on the host the IEEE float
 * quotient moved by -1, 0 or +1 unit, so host runs exercise the device's error bound */
XD_HD uint32_t xrcp_seed(float f, uint64_t salt) {
#ifdef __CUDA_ARCH__
  (void)salt;
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  return __float_as_uint(r);
#else
  const float r = 1.0f / f;
  uint32_t rb;
  memcpy(&rb, &r, sizeof(rb));
  return rb + (uint32_t)(salt % 3u) - 1u;
#endif
}

/* a / b rounded to nearest even, in integer arithmetic (normal operands, normal result; zero
 * numerators too).  With A, B the significands (2^52 <= A, B < 2^53) and t = (A < B), the
 * result's significand is N = RN(X / B), X = A 2^(52 + t), in [2^52, 2^53]:
 *  1. R0 ~ 2^84 / B from a float reciprocal of B's leading 24 bits (relative error < 2^-22;
 *     the reciprocal is clamped to the interval the exact one lies in);
 *  2. R ~ 2^115 / B = R0 2^31 (1 + e + e^2), e = 1 - B R0 / 2^84 (error e^3 plus truncations,
 *     below 2^-60), all in 64-bit fixed point;
 *  3. Q = floor(X R / 2^115), within one of floor(X / B); the remainder X - Q B is formed
 *     exactly (its magnitude is below 2^55, so 64-bit wrap-around arithmetic holds it) and
 *     brings Q to floor(X / B) with 0 <= remainder < B, which is checked: any other outcome takes
 *     the FP64 quotient;
 *  4. N = Q + 1 when twice the remainder exceeds B (or equals it, Q odd: a tie, which a quotient
 *     of two 53-bit numbers cannot produce).
 * Every result is the IEEE quotient's bits; the approximations of steps 1-2 only decide how
 * often the correction of step 3 is needed. */
XD_NOINLINE double em_div(double a, double b) {
  const uint64_t ua = xbits(a), ub = xbits(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  const uint64_t S = (ua ^ ub) & 0x8000000000000000ull;
  if (eb - 1u >= 2046u) return xdiv_slow(a, b);
  /* a zero numerator has a zero exponent field: its test runs behind the exponent test (written
   * on the whole pattern ahead of it, the compiler made it an FP64 comparison on every call) */
  if (ea - 1u >= 2046u) return zero_u(ua) ? xdbl(S) : xdiv_slow(a, b);  /* +-0 / normal: +-0 */
  const uint64_t M = (1ull << 52) - 1;
  const uint64_t A = (ua & M) | (1ull << 52), B = (ub & M) | (1ull << 52);
  const uint32_t t = (A < B) ? 1u : 0u;
  const int e = (int)ea - (int)eb + 1023 - (int)t;  /* the result's exponent field */
  if ((uint32_t)(e - 1) >= 2045u) return xdiv_slow(a, b);
  /* 1. */
  const uint32_t fb = 0x3f800000u | ((uint32_t)(B >> 29) & 0x7fffffu);
  float f;
  memcpy(&f, &fb, sizeof(f));
  const uint32_t rb = xrcp_seed(f, B);
  /* R0 = 2^32 r with r clamped to [1/2, 1 - 2^-32] (1/f lies in (1/2, 1]) */
  const uint64_t R0 = (rb >= 0x3f800000u) ? 0xffffffffull
                      : (rb < 0x3f000000u) ? 0x80000000ull : ((uint64_t)((rb & 0x7fffffu) | 0x800000u) << 8);
  /* 2. E0 = 2^84 e (|E0| < 2^63); T = 2^84 (e + e^2), the square from E0's leading bits */
  const int64_t E0 = (int64_t)(0ull - B * R0);
  const int64_t Eh = E0 >> 32;
  const int64_t T = E0 + ((Eh * Eh) >> 20);
  const int64_t Ph = (int64_t)R0 * (T >> 32);
  const uint64_t Pl = R0 * (uint64_t)(uint32_t)T;
  const int64_t P = Ph + (int64_t)(Pl >> 32);  /* floor(R0 T / 2^32) */
  const uint64_t R = (R0 << 31) + (uint64_t)(P >> 21);
  /* 3. */
  uint64_t Q = xmulhi(A << 11, R) >> (10 - t);
  int64_t rem = (int64_t)((A << (52 + t)) - Q * B);
  if (rem < 0) { Q -= 1; rem += (int64_t)B; }
  else if (rem >= (int64_t)B) { Q += 1; rem -= (int64_t)B; }
  if ((uint64_t)rem >= B) return xdiv_slow(a, b);
  /* 4. */
  const uint64_t r2 = (uint64_t)rem << 1;
  Q += (r2 > B || (r2 == B && (Q & 1u))) ? 1u : 0u;
  return xdbl((((uint64_t)(e - 1) << 52) + Q) | S);
}

XD_HD int64_t xmulhi_s(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}

/* the FP64 square root, for the operands the integer path does not cover */
XD_NOINLINE double xsqrt_slow(double x) { return ::sqrt(x); }

/* bits of an approximation to 1/sqrt(f), f in [1, 4): rsqrt.approx.ftz.f32 on the device; on the
 * host the quotient of 1 and the float root moved by -1, 0 or +1 unit */
XD_HD uint32_t xrsqrt_seed(float f, uint64_t salt) {
#ifdef __CUDA_ARCH__
  (void)salt;
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  return __float_as_uint(r);
#else
  const float r = 1.0f / std::sqrt(f);
  uint32_t rb;
  memcpy(&rb, &r, sizeof(rb));
  return rb + (uint32_t)(salt % 3u) - 1u;
#endif
}

/* sqrt(x) rounded to nearest even, in integer arithmetic (positive normal x; zeros too).  With X
 * the significand and p the parity of the unbiased exponent, the result's significand is
 * N = RN(sqrt(Y)), Y = X 2^(52 + p) in [2^104, 2^106):
 *  1. G0 ~ 2^32 / sqrt(X 2^(p - 52)) from the float reciprocal square root of X's leading 24
 *     bits (clamped to the interval (1/2, 1] the exact one lies in);
 *  2. e = 1 - Y G0^2 / 2^168 and S = X G0 2^(p - 32) (1 + e/2 + 3 e^2 / 8) (error 5 e^3 / 16 plus
 *     truncations), plus one, which puts S within one of floor(sqrt(Y));
 *  3. the remainder Y - S^2, exact in 64-bit wrap-around arithmetic (its magnitude is below
 *     2^57), brings S to floor(sqrt(Y)) with 0 <= remainder <= 2 S, which is checked: any other
 *     outcome takes the FP64 root;
 *  4. N = S + 1 when the remainder exceeds S (sqrt(Y) above S + 1/2; never equal to it).
 * Every result is the IEEE root's bits. */
XD_NOINLINE double em_sqrt(double x) {
  const uint64_t ux = xbits(x);
  const uint32_t ex = (uint32_t)(ux >> 52);  /* sign bit included: negative x fails the test */
  /* +-0 is its own root (tested behind the exponent test, as in em_div) */
  if (ex - 1u >= 2046u) return zero_u(ux) ? x : xsqrt_slow(x);
  const uint64_t X = (ux & ((1ull << 52) - 1)) | (1ull << 52);
  const uint32_t p = (ex & 1u) ^ 1u;
  const int er = (((int)ex - 1023 - (int)p) >> 1) + 1023;  /* the result's exponent field */
  /* 1. */
  const uint32_t fb = ((127u + p) << 23) | ((uint32_t)(X >> 29) & 0x7fffffu);
  float f;
  memcpy(&f, &fb, sizeof(f));
  const uint32_t gb = xrsqrt_seed(f, X);
  const uint64_t G0 = (gb >= 0x3f800000u) ? 0xffffffffull
                      : (gb < 0x3f000000u) ? 0x80000000ull : ((uint64_t)((gb & 0x7fffffu) | 0x800000u) << 8);
  /* 2. Ee = 2^63 e, C = 2^64 (e/2 + 3 e^2 / 8) */
  const uint64_t hi = xmulhi(X << 11, G0 * G0);  /* floor(X G0^2 / 2^53) ~ 2^(63 - p) (1 - e) */
  const int64_t Ee = (int64_t)((1ull << (63 - p)) - hi) << p;
  const int64_t Eh = Ee >> 20;
  const int64_t Cc = Ee + ((3 * Eh * Eh) >> 25);
  const uint64_t lo = X * G0, xh = xmulhi(X, G0);
  const int64_t Sb = (int64_t)((xh << (32 + p)) | (lo >> (32 - p)));  /* floor(X G0 2^(p - 32)) */
  uint64_t S = (uint64_t)(Sb + xmulhi_s(Sb, Cc)) + 1u;
  /* 3. */
  int64_t rem = (int64_t)((X << (52 + p)) - S * S);
  if (rem < 0) { rem += (int64_t)(2 * S - 1); S -= 1; }
  else if (rem > (int64_t)(2 * S)) { rem -= (int64_t)(2 * S + 1); S += 1; }
  if (rem < 0 || rem > (int64_t)(2 * S)) return xsqrt_slow(x);
  /* 4. */
  S += (rem > (int64_t)S) ? 1u : 0u;
  return xdbl(((uint64_t)(er - 1) << 52) + S);
}

/* The bit pattern a comparison keys on.  On the device an opaque register move: when a value that
 * an FP64 sum has just formed is compared on its bits, the compiler otherwise forms the sum twice,
 * once for the double and once for its bits (measured: 16 key comparisons of running sums took 35
 * FP64 additions instead of 18).  (The same move in every bit operation of this file made the WAF
 * edge slower: it also blocks the folding of its sign flips and scalings.) */
XD_HD uint64_t xbits_cmp(double x) {
  uint64_t b;
#ifdef __CUDA_ARCH__
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
#else
  memcpy(&b, &x, sizeof(b));
#endif
  return b;
}

/* ordered integer key of a non-NaN double: order of the values, -0 and +0 equal */
XD_HD long long xkey(uint64_t b) {
  const long long s = (long long)b >> 63;
  return (long long)((b & 0x7fffffffffffffffull) ^ (uint64_t)s) - s;
}
XD_HD bool xnan(uint64_t b) { return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }
/* a < b, a <= b, a == b (IEEE results, NaN compares false) on ordered keys; OC: the keys of the
 * opaque bit patterns (xbits_cmp), else of the plain ones */
template <bool OC> XD_HD uint64_t xbits_key(double x) { return OC ? xbits_cmp(x) : xbits(x); }
template <bool OC = true> XD_HD bool xlt(double a, double b) {
  const uint64_t ua = xbits_key<OC>(a), ub = xbits_key<OC>(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) < xkey(ub));
}
template <bool OC = true> XD_HD bool xle(double a, double b) {
  const uint64_t ua = xbits_key<OC>(a), ub = xbits_key<OC>(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) <= xkey(ub));
}
template <bool OC = true> XD_HD bool xeq(double a, double b) {
  const uint64_t ua = xbits_key<OC>(a), ub = xbits_key<OC>(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) == xkey(ub));
}

template <bool MUL, bool OC = true>
struct XD {
  double v;
  XD_HD XD() : v(0.0) {}
  XD_HD XD(double x) : v(x) {}  // NOLINT: constants promote implicitly
};

template <bool MUL, bool OC>
XD_HD double val(const XD<MUL, OC>& x) { return x.v; }

template <bool MUL>
XD_HD double xd_mul(double a, double b) {
  if (MUL) return em_mul(a, b);
  return a * b;
}
template <bool MUL>
XD_HD double xd_div(double a, double b) {
  if (MUL) return em_div(a, b);
  return a / b;
}

#define CF_XD_BIN(op, expr)                                                                               \
  template <bool MUL, bool OC> XD_HD XD<MUL, OC> operator op(const XD<MUL, OC>& a, const XD<MUL, OC>& b) { double x = a.v, y = b.v; return XD<MUL, OC>(expr); } \
  template <bool MUL, bool OC> XD_HD XD<MUL, OC> operator op(const XD<MUL, OC>& a, double y) { double x = a.v; return XD<MUL, OC>(expr); } \
  template <bool MUL, bool OC> XD_HD XD<MUL, OC> operator op(double x, const XD<MUL, OC>& b) { double y = b.v; return XD<MUL, OC>(expr); }
CF_XD_BIN(+, x + y)
CF_XD_BIN(-, x - y)
CF_XD_BIN(*, xd_mul<MUL>(x, y))
CF_XD_BIN(/, xd_div<MUL>(x, y))
#undef CF_XD_BIN

/* negation as a sign-bit flip: an FP64 negation that is not folded into its consumer is an FP64
 * instruction, and most consumers here are integer code (products, comparisons) */
template <bool MUL, bool OC> XD_HD XD<MUL, OC> operator-(const XD<MUL, OC>& a) { return XD<MUL, OC>(xdbl(xbits(a.v) ^ 0x8000000000000000ull)); }

#define CF_XD_CMP(op, expr)                                                                               \
  template <bool MUL, bool OC> XD_HD bool operator op(const XD<MUL, OC>& a, const XD<MUL, OC>& b) { double x = a.v, y = b.v; return expr; } \
  template <bool MUL, bool OC> XD_HD bool operator op(const XD<MUL, OC>& a, double y) { double x = a.v; return expr; } \
  template <bool MUL, bool OC> XD_HD bool operator op(double x, const XD<MUL, OC>& b) { double y = b.v; return expr; }
CF_XD_CMP(<, xlt<OC>(x, y))
CF_XD_CMP(>, xlt<OC>(y, x))
CF_XD_CMP(<=, xle<OC>(x, y))
CF_XD_CMP(>=, xle<OC>(y, x))
CF_XD_CMP(==, xeq<OC>(x, y))
CF_XD_CMP(!=, !xeq<OC>(x, y))
#undef CF_XD_CMP

template <bool MUL, bool OC> XD_HD XD<MUL, OC> sqrt(const XD<MUL, OC>& a) { return XD<MUL, OC>(MUL ? em_sqrt(a.v) : ::sqrt(a.v)); }
template <bool MUL, bool OC> XD_HD XD<MUL, OC> rcbrt(const XD<MUL, OC>& a) { return XD<MUL, OC>(rcbrt(a.v)); }
template <bool MUL, bool OC> XD_HD XD<MUL, OC> fabs(const XD<MUL, OC>& a) { return XD<MUL, OC>(xdbl(xbits(a.v) & 0x7fffffffffffffffull)); }
template <bool MUL, bool OC> XD_HD XD<MUL, OC> sgnmul(const XD<MUL, OC>& x, const XD<MUL, OC>& y) {
  return XD<MUL, OC>(xdbl(xbits(y.v) ^ (xbits(x.v) & 0x8000000000000000ull)));
}

/* x * 2^K (K = -2, -1, 1) by a change of the exponent field, for a normal x whose result is
 * normal: the exact scaling, the bits of the FP64 product.  Zeros keep their bits; subnormal,
 * infinite and NaN operands and results out of the normal range take the FP64 product. */
template <int K>
XD_HD double xscale(double x) {
  const uint64_t b = xbits(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  const uint32_t lo = (K < 0) ? (uint32_t)(1 - K) : 1u;          /* lowest exponent field handled */
  const uint32_t n = (K < 0) ? (uint32_t)(2046 + K) : (uint32_t)(2046 - K);  /* fields handled */
  if (e - lo < n) return xdbl(b + ((uint64_t)(int64_t)K << 52));
  if (zero_u(b)) return x;
  return xmul_slow(x, (K == -2) ? 0.25 : ((K == -1) ? 0.5 : 2.0));
}
template <bool MUL, bool OC> XD_HD XD<MUL, OC> halve(const XD<MUL, OC>& x) { return XD<MUL, OC>(MUL ? xscale<-1>(x.v) : x.v * 0.5); }
template <bool MUL, bool OC> XD_HD XD<MUL, OC> quarter(const XD<MUL, OC>& x) { return XD<MUL, OC>(MUL ? xscale<-2>(x.v) : x.v * 0.25); }
template <bool MUL, bool OC> XD_HD XD<MUL, OC> twice(const XD<MUL, OC>& x) { return XD<MUL, OC>(MUL ? xscale<1>(x.v) : x.v * 2.0); }

/* The quotient a / d that div_rn in cf_flux.h forms from y = RN(1/d) by Markstein's step: on the
 * integer path the division itself (the same bits, y unused), otherwise Markstein's step. */
template <bool MUL, bool OC>
XD_HD XD<MUL, OC> div_rn(const XD<MUL, OC>& a, double d, double y) {
  if (MUL) return XD<MUL, OC>(em_div(a.v, d));
  const double q = a.v * y;
  const double r = fma(-d, q, a.v);
  const double q1 = fma(r, y, q);
  return XD<MUL, OC>(zero_u(xbits(a.v)) ? q : q1);
}
template <bool MUL, bool OC>
XD_HD XD<MUL, OC> div_rn(const XD<MUL, OC>& a, const XD<MUL, OC>& d, const XD<MUL, OC>& y) {
  return div_rn(a, d.v, y.v);
}

}  // namespace cf

#endif
