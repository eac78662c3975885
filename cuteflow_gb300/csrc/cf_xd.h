/*
 * cf_xd.h -- binary64 arithmetic that keeps GB300's FP64 pipe for the operations only it can do.
 *
 * GB300 issues two FP64 operations per clock per SM; its integer pipes issue ~30x more 32-bit
 * operations, run beside the FP64 pipe, and sit idle in the step kernels (ncu: FP64 pipe 85 %
 * busy, ALU 1.4 %).  Two exact substitutions move FP64-pipe work onto them:
 *
 *   comparisons  x < y etc. on ordered integer keys of the bit patterns (negative values
 *                mirrored, -0 and +0 one key, NaN compares false): the IEEE result, on the ALU;
 *   products     x * y by integer multiplication of the significands with round to nearest
 *                even (em_mul): the IEEE product for normal operands with a normal result; any
 *                other operand (zero, subnormal, infinite, NaN) or result (overflow,
 *                underflow) takes the FP64 instruction, in an out-of-line function so that the
 *                compiler does not evaluate it speculatively on the fast path.
 *
 * XD<MUL> is a double that compares on integer keys and, with MUL, multiplies with em_mul;
 * sums, quotients and square roots stay FP64 instructions.  Every result is the IEEE binary64
 * result of the same operation, so code instantiated on XD<...> rounds exactly like the same
 * code on double; which warps use the integer multiply is a tuning choice, not a numerical one.
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

/* ordered integer key of a non-NaN double: order of the values, -0 and +0 equal */
XD_HD long long xkey(uint64_t b) {
  const long long s = (long long)b >> 63;
  return (long long)((b & 0x7fffffffffffffffull) ^ (uint64_t)s) - s;
}
XD_HD bool xnan(uint64_t b) { return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }
XD_HD bool xlt(double a, double b) {
  const uint64_t ua = xbits(a), ub = xbits(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) < xkey(ub));
}
XD_HD bool xle(double a, double b) {
  const uint64_t ua = xbits(a), ub = xbits(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) <= xkey(ub));
}
XD_HD bool xeq(double a, double b) {
  const uint64_t ua = xbits(a), ub = xbits(b);
  return !(xnan(ua) | xnan(ub)) & (xkey(ua) == xkey(ub));
}

template <bool MUL>
struct XD {
  double v;
  XD_HD XD() : v(0.0) {}
  XD_HD XD(double x) : v(x) {}  // NOLINT: constants promote implicitly
};

template <bool MUL>
XD_HD double val(const XD<MUL>& x) { return x.v; }

template <bool MUL>
XD_HD double xd_mul(double a, double b) {
  if (MUL) return em_mul(a, b);
  return a * b;
}

#define CF_XD_BIN(op, expr)                                                                               \
  template <bool MUL> XD_HD XD<MUL> operator op(const XD<MUL>& a, const XD<MUL>& b) { double x = a.v, y = b.v; return XD<MUL>(expr); } \
  template <bool MUL> XD_HD XD<MUL> operator op(const XD<MUL>& a, double y) { double x = a.v; return XD<MUL>(expr); } \
  template <bool MUL> XD_HD XD<MUL> operator op(double x, const XD<MUL>& b) { double y = b.v; return XD<MUL>(expr); }
CF_XD_BIN(+, x + y)
CF_XD_BIN(-, x - y)
CF_XD_BIN(*, xd_mul<MUL>(x, y))
CF_XD_BIN(/, x / y)
#undef CF_XD_BIN

template <bool MUL> XD_HD XD<MUL> operator-(const XD<MUL>& a) { return XD<MUL>(-a.v); }

#define CF_XD_CMP(op, expr)                                                                               \
  template <bool MUL> XD_HD bool operator op(const XD<MUL>& a, const XD<MUL>& b) { double x = a.v, y = b.v; return expr; } \
  template <bool MUL> XD_HD bool operator op(const XD<MUL>& a, double y) { double x = a.v; return expr; } \
  template <bool MUL> XD_HD bool operator op(double x, const XD<MUL>& b) { double y = b.v; return expr; }
CF_XD_CMP(<, xlt(x, y))
CF_XD_CMP(>, xlt(y, x))
CF_XD_CMP(<=, xle(x, y))
CF_XD_CMP(>=, xle(y, x))
CF_XD_CMP(==, xeq(x, y))
CF_XD_CMP(!=, !xeq(x, y))
#undef CF_XD_CMP

template <bool MUL> XD_HD XD<MUL> sqrt(const XD<MUL>& a) { return XD<MUL>(::sqrt(a.v)); }
template <bool MUL> XD_HD XD<MUL> rcbrt(const XD<MUL>& a) { return XD<MUL>(rcbrt(a.v)); }
template <bool MUL> XD_HD XD<MUL> fabs(const XD<MUL>& a) { return XD<MUL>(xdbl(xbits(a.v) & 0x7fffffffffffffffull)); }
template <bool MUL> XD_HD XD<MUL> sgnmul(const XD<MUL>& x, const XD<MUL>& y) {
  return XD<MUL>(xdbl(xbits(y.v) ^ (xbits(x.v) & 0x8000000000000000ull)));
}

/* Markstein's quotient (div_rn in cf_flux.h) with the product on the chosen path */
template <bool MUL>
XD_HD XD<MUL> div_rn(const XD<MUL>& a, double d, double y) {
  const double q = xd_mul<MUL>(a.v, y);
  const double r = fma(-d, q, a.v);
  const double q1 = fma(r, y, q);
  return XD<MUL>(((xbits(a.v) << 1) == 0) ? q : q1);
}
template <bool MUL>
XD_HD XD<MUL> div_rn(const XD<MUL>& a, const XD<MUL>& d, const XD<MUL>& y) {
  return div_rn(a, d.v, y.v);
}

}  // namespace cf

#endif
