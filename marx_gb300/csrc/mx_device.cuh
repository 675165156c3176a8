// Per-photon trace stages for the GB300 kernels.
//
// Each stage follows the reference function it replaces (paths inside MARX
// 5.5.3, cited per function) in FP64 for geometry and FP32 where the
// reference keeps float tables.  Unlike the oracle it is written for the
// GPU's scarce FP64 pipe: one reciprocal square root instead of a scaled
// hypot plus three divisions per normalisation, sincos pairs, precomputed
// per-shell sines and cosines, and |a/b|^2 = |a|^2/|b|^2 in the Fresnel
// reflectivity.  These change results only at the last-bit level; every
// comparison that decides a photon's fate (shell, reflectivity, order,
// chip) uses the same quantities and order as the reference.
#pragma once
#include <stdint.h>
#include "mx_model.h"

#include <cmath>
#include <cstring>
#ifdef __CUDACC__
#define MXD __host__ __device__ __forceinline__
#else
#define MXD inline
#endif

namespace mx {

constexpr double PI = 3.14159265358979323846264338327950288;

struct D3 { double x, y, z; };
MXD D3 mk(double x, double y, double z) { D3 r; r.x = x; r.y = y; r.z = z; return r; }
MXD D3 operator+(D3 a, D3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
MXD D3 operator-(D3 a, D3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
MXD D3 operator*(double s, D3 a) { return mk(s * a.x, s * a.y, s * a.z); }
MXD double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MXD D3 cross(D3 a, D3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

MXD double mx_rsqrt(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / std::sqrt(x);
#endif
}
MXD void mx_sincos(double x, double *s, double *c) {
#ifdef __CUDA_ARCH__
  sincos(x, s, c);
#else
  *s = std::sin(x); *c = std::cos(x);
#endif
}
// Comparisons of doubles on the integer pipe.  On GB300 a DSETP issues on
// the FP64 pipe, the one this trace is bound by; the order of IEEE doubles
// is the order of their bit patterns read as sign-magnitude integers.
// None of the helpers is meant for NaN.
MXD unsigned long long dbits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long) __double_as_longlong(x);
#else
  unsigned long long u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
// a < b for a, b >= +0 (no -0): the bit patterns compare as unsigned integers
MXD bool lt_pos(double a, double b) { return dbits(a) < dbits(b); }
// a signed integer key with key(a) < key(b) exactly when a < b, and
// key(-0) = key(+0) = 0
MXD long long dkey(double x) {
  const unsigned long long b = dbits(x);
  return (long long) ((long long) b < 0 ? 0x8000000000000000ull - b : b);
}
MXD bool is_zero(double x) { return (dbits(x) << 1) == 0; }   // x = +0 or -0
// -x when neg, else x: a sign-bit flip on the integer pipe (a negation that
// is not folded into the next operation issues as a DADD)
MXD double flip_sign(double x, bool neg) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(x) ^ ((long long) neg << 63));
#else
  return neg ? -x : x;
#endif
}
MXD bool neg_bit(double x) { return (long long) dbits(x) < 0; }   // sign bit: x < 0 or x = -0
// (unsigned) (4 x) for 0 <= x < 1 from the bits of x: the integer part of
// 1.m 2^(e+2).
MXD unsigned quarter_of(double x) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = dbits(x);
  const int e = (int) ((b >> 52) & 0x7ff) - 1023 + 2;   // 4x = 1.m 2^e
  if (e < 0) return 0u;
  if (e > 2) return (unsigned) (4.0 * x);
  return (unsigned) (((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - e));
#else
  return (unsigned) (4.0 * x);
#endif
}
// sqrt(x) for geometry: x times the library's reciprocal square root (within
// two ulps; six FP64 instructions and a multiply instead of the correctly
// rounded root's nine).  x = 0, infinities and NaN take sqrt.
MXD double sqrt_fast(double x) {
#ifdef __CUDA_ARCH__
  const unsigned e = (unsigned) (dbits(x) >> 52);   // sign and exponent
  if (e - 1u < 0x7feu) return x * rsqrt(x);         // positive, normal, finite
#endif
  return sqrt(x);
}
// sqrt(x) and 1 / sqrt(x) from one reciprocal square root (x positive,
// normal, finite); other x take sqrt and a division.
MXD void sqrt_rsqrt(double x, double &s, double &rs) {
#ifdef __CUDA_ARCH__
  const unsigned e = (unsigned) (dbits(x) >> 52);
  if (e - 1u < 0x7feu) { rs = rsqrt(x); s = x * rs; return; }
#endif
  s = sqrt(x);
  rs = 1.0 / s;
}
// (unsigned) x and (double) u on the integer pipe (the conversions issue
// on the FP64 pipe): x >= 0 below 2^32, u below 2^32.
MXD unsigned trunc_to_unsigned(double x) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = dbits(x);
  const int e = (int) ((b >> 52) & 0x7ff) - 1023;   // x = 1.m 2^e
  if (e < 0) return 0u;
  if (e > 31) return (unsigned) x;
  return (unsigned) (((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - e));
#else
  return (unsigned) x;
#endif
}
MXD double u2d(unsigned u) {
#ifdef __CUDA_ARCH__
  if (u == 0u) return 0.0;
  const int lz = __clz((int) u);                      // u = 1.m 2^(31 - lz)
  const unsigned long long m = ((unsigned long long) u << (lz + 21)) & 0xFFFFFFFFFFFFFull;
  return __longlong_as_double((long long) (((unsigned long long) (1023 + 31 - lz) << 52) | m));
#else
  return (double) u;
#endif
}
// JDMv_normalize (vector.c:99): a / |a|, a unchanged when |a| = 0.
MXD D3 normalized(D3 a) {
  double d = dot(a, a);
  if (is_zero(d)) return a;
  return mx_rsqrt(d) * a;
}
// a / |a| for a vector whose length is 1 to within 1e-8 (a rotation of a
// unit vector): with |a|^2 = 1 + e, 1/|a| = 1 - e/2 + 3e^2/8 - ..., and
// 1.5 - |a|^2 / 2 leaves out 3e^2/8 < 4e-17, below half an ulp.  Longer or
// shorter vectors take the full reciprocal square root.
MXD D3 normalized_unit(D3 a) {
  double d = dot(a, a);
  // |d - 1| < 1e-8 exactly when 0x1.ffffffaa19c47p-1 < d < 0x1.0000002af31ddp+0
  if (lt_pos(0x1.ffffffaa19c47p-1, d) && lt_pos(d, 0x1.0000002af31ddp+0)) return (1.5 - 0.5 * d) * a;
  return normalized(a);
}
// JDMv_rotate_unit_vector1 (vector.c:198): Rodrigues rotation of p about
// unit n by (c, s), renormalised.
MXD D3 rotate_unit(D3 p, D3 n, double c, double s) {
  double pn = dot(p, n);
  D3 u = c * p + (pn * (1.0 - c)) * n + s * cross(n, p);
  return normalized_unit(u);
}
// sin and cos of an angle that is usually tiny (mirror blur, aspect blur,
// dither offsets, facet misalignment, scattering).  Below 2^-5 rad the
// Taylor series of sin to x^7 and of cos to x^8 leave out terms below
// 3e-18 (sin, relative) and 3e-22 (cos): under a tenth of an ulp; below
// 1e-4 rad the series to x^3 and x^2 already do (the next terms are below
// 5e-18 relative).  Larger angles, rare in a warp, take the library
// sincos.
MXD void sincos_small(double x, double *s, double *c) {
  const double ax = fabs(x);
  if (lt_pos(ax, 1e-4)) {
    double x2 = x * x;
    *s = x + x * x2 * (-1.0 / 6.0);
    *c = 1.0 + x2 * -0.5;
  } else if (lt_pos(ax, 0x1p-5)) {
    double x2 = x * x;
    *s = x + x * x2 * (-1.0 / 6.0 + x2 * (1.0 / 120.0 + x2 * (-1.0 / 5040.0)));
    *c = 1.0 + x2 * (-0.5 + x2 * (1.0 / 24.0 + x2 * (-1.0 / 720.0 + x2 * (1.0 / 40320.0))));
  } else
    mx_sincos(x, s, c);
}
// sin(pi y), cos(pi y): the argument needs no reduction by pi.
MXD void mx_sincospi(double y, double *s, double *c) {
#ifdef __CUDA_ARCH__
  sincospi(y, s, c);
#else
  *s = std::sin(PI * y); *c = std::cos(PI * y);
#endif
}
MXD D3 rotate_unit_angle(D3 p, D3 n, double theta) {
  double s, c;
  mx_sincos(theta, &s, &c);
  return rotate_unit(p, n, c, s);
}
MXD D3 rotate_unit_small(D3 p, D3 n, double theta) {
  double s, c;
  sincos_small(theta, &s, &c);
  return rotate_unit(p, n, c, s);
}
MXD D3 mat_mul(const double *m, D3 v) {  // JDM3m_vector_mul (rotate.c:121), row-major 3x3
  return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

#ifdef __CUDA_ARCH__
#define MX_LDG(p) __ldg(p)
#define MX_DMUL(a, b) __dmul_rn(a, b)
#define MX_DADD(a, b) __dadd_rn(a, b)
#define MX_DDIV(a, b) __ddiv_rn(a, b)
#else
#define MX_LDG(p) (*(p))
#define MX_DMUL(a, b) ((a) * (b))
#define MX_DADD(a, b) ((a) + (b))
#define MX_DDIV(a, b) ((a) / (b))
#endif

// Conversions between float and double on the integer pipe.  On GB300 a
// F2F conversion issues on the FP64 pipe, the one this trace is bound by.
// f2d is exact (as the cast is); zeros, subnormals, infinities and NaN
// take the cast.
MXD double f2d(float f) {
#ifdef __CUDA_ARCH__
  const uint32_t u = __float_as_uint(f), a = u & 0x7fffffffu;
  uint32_t hi, lo;
  if (a >= 0x00800000u) {               // normal: rebias the exponent by 1023 - 127
    hi = (a >> 3) + (896u << 20);
    lo = a << 29;
    if (a >= 0x7f800000u) hi = 0x7ff00000u | ((a & 0x7fffffu) >> 3);   // infinity, NaN
  } else if (a != 0u) {                 // subnormal: a 2^-149 with a normalised
    const uint32_t lz = (uint32_t) __clz((int) a);
    const uint32_t m = (a << (lz - 8u)) & 0x7fffffu;
    hi = ((905u - lz) << 20) | (m >> 3);
    lo = m << 29;
  } else
    hi = lo = 0u;
  return __hiloint2double((int) ((u & 0x80000000u) | hi), (int) lo);
#else
  return (double) f;
#endif
}
// d truncated toward zero to float (relative error below 2^-23); magnitudes
// below 2^-126 become zero, above float range infinity; NaN stays NaN.  For
// single-precision screens only, never for a stored result.
MXD float d2f_trunc(double d) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = (unsigned long long) __double_as_longlong(d);
  const uint32_t hi = (uint32_t) (b >> 32), lo = (uint32_t) b, e = (hi >> 20) & 0x7ffu;
  uint32_t r = hi & 0x80000000u;
  if (e - 897u < 254u) r |= ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  else if (e >= 1151u) r |= 0x7f800000u | ((e == 2047u && ((hi & 0xfffffu) | lo)) ? 0x400000u : 0u);
  return __uint_as_float(r);
#else
  return (float) d;
#endif
}
// d rounded to the nearest float (ties to even), as the cast rounds it,
// on the integer pipe for results in the normal float range; other
// magnitudes (and NaN) take the cast.
MXD float d2f_rn(double d) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = (unsigned long long) __double_as_longlong(d);
  const uint32_t hi = (uint32_t) (b >> 32), e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 253u) {   // 2^-126 <= |d| < 2^126: the result is a normal float
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    uint32_t keep = (uint32_t) (m >> 29);                  // 24 bits with the leading one
    const uint32_t rem = (uint32_t) m & 0x1FFFFFFFu;
    keep += (rem > 0x10000000u || (rem == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    // a carry out of the 24 bits lands in the exponent field, as it should
    const uint32_t r = (hi & 0x80000000u) + ((e - 896u) << 23) + (keep - 0x800000u);
    return __uint_as_float(r);
  }
#endif
  return (float) d;
}
// 1 / d by Newton-Raphson iteration (y <- y + y (1 - d y)) from a
// single-precision seed: the float reciprocal of d is good to about 2^-23,
// each step squares the relative error, so two steps leave only the
// rounding of the last fused multiply-add (within one ulp of the quotient,
// not always the correctly rounded one).  Two MUFU/integer operations and
// four DFMA instead of the division's longer FP64 sequence.  Magnitudes
// outside [2^-125, 2^125), zeros, infinities and NaN take the division.
MXD double rcp_fast(double d) {
#ifdef __CUDA_ARCH__
  const unsigned e = (unsigned) (dbits(d) >> 52) & 0x7ffu;
  if (e - 898u < 250u) {
    double y = f2d(__frcp_rn(d2f_trunc(d)));
    double r = fma(-d, y, 1.0);
    y = fma(y, r, y);
    r = fma(-d, y, 1.0);
    return fma(y, r, y);
  }
#endif
  return 1.0 / d;
}
// ------------------------------------------------ sines on the FP32 pipe --
// GB300 issues FP64 at 1/64 of its FP32 rate, and a double-precision sine
// or cosine from the math library takes about twenty FP64-pipe
// instructions.  The angles below are reduced in double (a few exact FP64
// operations), then sin and cos of the reduced angle r, |r| <= pi/4, are
// evaluated in double-float arithmetic on the FP32 pipe: a value is the
// unevaluated sum hi + lo of two floats, sums and products are formed with
// the error-free transformations of Dekker (1971) and Knuth (TAOCP 4.2.2)
// using fused multiply-adds.  The polynomials are the Taylor series of sin
// and cos (truncation error below 5e-17 on |r| <= pi/4); their leading
// terms carry double-float coefficients (1/n! split into two floats), the
// last ones are summed in single precision where their size keeps the
// rounding below 2^-48.  The result is within 2^-44 of the true sine or
// cosine of the double argument.
#ifdef __CUDA_ARCH__
struct F2 { float h, l; };
__device__ __forceinline__ F2 quick_sum(float a, float b) {   // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), v = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}
__device__ __forceinline__ F2 df_add(F2 a, F2 b) {
  const F2 s = two_sum(a.h, b.h);
  return quick_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ F2 df_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return quick_sum(p, e);
}
__device__ __forceinline__ F2 df_mul_f(F2 a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return quick_sum(p, e);
}
// d as hi + lo: hi the truncation of d to float, lo that of the remainder
// (exact in double); |d - hi - lo| < 2^-46 |d|.  One FP64 subtraction.
__device__ __forceinline__ F2 df_from(double d) {
  const float h = d2f_trunc(d);
  return {h, d2f_trunc(d - f2d(h))};
}
__device__ __forceinline__ double df_to(F2 a) { return f2d(a.h) + f2d(a.l); }

// sin and cos of r (|r| <= pi/4 + a little) in double-float.
__device__ __forceinline__ void df_sincos(F2 r, F2 &sr, F2 &cr) {
  const F2 z = df_mul(r, r);
  const float zf = z.h;
  // S(z) = (sin r - r) / (r z) = -1/3! + z/5! - z^2/7! + ...: the terms
  // from z^4/11! on in single precision
  float g = __fmaf_rn(zf, -0x1.ae7f3ep-41f, 0x1.612462p-33f);
  g = __fmaf_rn(zf, g, -0x1.ae6456p-26f);
  F2 P = df_add(F2{0x1.71de3ap-19f, 0x1.55b1ccp-45f}, df_mul_f(z, g));
  P = df_add(F2{-0x1.a01a02p-13f, 0x1.7f97fap-39f}, df_mul(z, P));
  P = df_add(F2{0x1.111112p-7f, -0x1.dddddep-32f}, df_mul(z, P));
  P = df_add(F2{-0x1.555556p-3f, 0x1.555556p-28f}, df_mul(z, P));
  sr = df_add(r, df_mul(r, df_mul(z, P)));
  // C(z) = (cos r - 1) / z = -1/2! + z/4! - z^2/6! + ...: from z^5/12! on
  // in single precision
  float gc = __fmaf_rn(zf, 0x1.ae7f3ep-45f, -0x1.93974ap-37f);
  gc = __fmaf_rn(zf, gc, 0x1.1eed8ep-29f);
  F2 Q = df_add(F2{-0x1.27e4fcp-22f, 0x1.10ec14p-47f}, df_mul_f(z, gc));
  Q = df_add(F2{0x1.a01a02p-16f, -0x1.7f97fap-42f}, df_mul(z, Q));
  Q = df_add(F2{-0x1.6c16c2p-10f, 0x1.27d27ep-35f}, df_mul(z, Q));
  Q = df_add(F2{0x1.555556p-5f, -0x1.555556p-30f}, df_mul(z, Q));
  Q = df_add(F2{-0.5f, 0.0f}, df_mul(z, Q));
  cr = df_add(F2{1.0f, 0.0f}, df_mul(z, Q));
}

__device__ __forceinline__ F2 df_neg(F2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ F2 df_sub(F2 a, F2 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ F2 df_sqr(F2 a) { return df_mul(a, a); }
// sqrt(a), a > 0: the float root s corrected by (a - s^2) / (2 s), the
// residual from a fused multiply-add (one Newton step; Karp and Markstein
// 1997).
__device__ __forceinline__ F2 df_sqrt(F2 a) {
  const float s = __fsqrt_rn(a.h);
  const float e = __fadd_rn(__fmaf_rn(-s, s, a.h), a.l);
  return quick_sum(s, __fmul_rn(e, __fdiv_rn(0.5f, s)));
}
// 1 / sqrt(a), a > 0: the float estimate y and one Newton step
// y (1 + (1 - a y^2) / 2), with 1 - a y^2 formed in double-float.
__device__ __forceinline__ F2 df_rsqrt(F2 a) {
  const float y = __frsqrt_rn(a.h);
  const float p = __fmul_rn(y, y);
  const F2 q = df_mul(a, F2{p, __fmaf_rn(y, y, -p)});
  const float e = __fsub_rn(__fsub_rn(1.0f, q.h), q.l);
  return quick_sum(y, __fmul_rn(__fmul_rn(0.5f, y), e));
}
// a / b: the float quotient corrected by the remainder a - q b.
__device__ __forceinline__ F2 df_div(F2 a, F2 b) {
  const float q = __fdiv_rn(a.h, b.h);
  const F2 r = df_sub(a, df_mul_f(b, q));
  return quick_sum(q, __fdiv_rn(r.h, b.h));
}

// The Fresnel numerator and denominator of reflectivity_parts in
// double-float arithmetic on the FP32 pipe (beta, delta are floats), with
// the same branches.  n^2 - sin^2 is formed without cancelling two numbers
// near 1 (where the double evaluation loses up to 2^-28 near the critical
// angle).  Within 2^-30 of the exact values over grazing angles of
// 0.05-3 degrees and beta, delta of 1e-9..1e-2, typically 2^-42; the worst
// case is the numerator of a reflectivity near 1e-7, which cancels in
// cos - root as the double evaluation does.
__device__ __forceinline__ void reflectivity_df(double cos_t, float beta, float delta, F2 &num, F2 &den) {
  const F2 c = df_from(cos_t);
  const F2 nr = two_sum(1.0f, -delta);
  const float b2 = __fmul_rn(beta, beta);
  const F2 bsq = {b2, __fmaf_rn(beta, beta, -b2)};
  const F2 sr = df_sub(df_sqr(nr), bsq);
  const F2 si = df_mul_f(nr, 2.0f * beta);
  // wr = sr - (1 - c^2) as c^2 - (delta (2 - delta) + beta^2): the same
  // value without the cancellation of two numbers near 1
  const F2 k = df_add(df_mul_f(two_sum(2.0f, -delta), delta), bsq);
  const F2 wr = df_sub(df_sqr(c), k), wi = si;
  const F2 r = df_sqrt(df_add(df_sqr(wr), df_sqr(wi)));
  F2 rr, ri;
  const F2 half_wi = {0.5f * wi.h, 0.5f * wi.l};
  if (wr.h >= 0.0f) {
    const F2 h = df_add(r, wr);
    const F2 hh = {0.5f * h.h, 0.5f * h.l}, inv = df_rsqrt(hh);
    rr = df_mul(hh, inv); ri = df_mul(half_wi, inv);
  } else {
    const F2 h = df_sub(r, wr);
    const F2 hh = {0.5f * h.h, 0.5f * h.l}, inv = df_rsqrt(hh);
    rr = df_mul(half_wi, inv); ri = df_mul(hh, inv);
    if (rr.h < 0.0f) { rr = df_neg(rr); ri = df_neg(ri); }
  }
  const F2 ri2 = df_sqr(ri);
  const F2 a1 = df_add(df_sqr(df_sub(c, rr)), ri2), bb1 = df_add(df_sqr(df_add(c, rr)), ri2);
  const F2 pr = df_mul(c, sr), pi_ = df_mul(c, si);
  const F2 a2 = df_add(df_sqr(df_sub(pr, rr)), df_sqr(df_sub(pi_, ri)));
  const F2 bb2 = df_add(df_sqr(df_add(pr, rr)), df_sqr(df_add(pi_, ri)));
  const F2 t = df_add(df_mul(a1, bb2), df_mul(a2, bb1));
  num = {0.5f * t.h, 0.5f * t.l};
  den = df_mul(bb1, bb2);
}
#endif

// sin(pi y) and cos(pi y) within 2^-44 (for angles that set positions and
// directions, whose tolerance is far wider).  y = q/2 + f with q the
// nearest integer to 2y, |f| <= 1/4, both exact; pi f in double-float.
MXD void sincospi_fast(double y, double *s, double *c) {
#ifdef __CUDA_ARCH__
  const double magic = 6755399441055744.0;   // 1.5 2^52: the sum rounds to an integer
  const double t = fma(y, 2.0, magic);
  const int q = __double2loint(t);
  const double f = fma(t - magic, -0.5, y);
  const F2 r = df_mul(F2{0x1.921fb6p+1f, -0x1.777a5cp-24f}, df_from(f));   // pi f
  F2 sr, cr;
  df_sincos(r, sr, cr);
  // sin(q pi/2 + x), cos(q pi/2 + x) from sin x, cos x
  const double a = df_to(sr), b = df_to(cr);
  const int k = q & 3;
  *s = flip_sign((k & 1) ? b : a, (k & 2) != 0);
  *c = flip_sign((k & 1) ? a : b, ((k + 1) & 2) != 0);
#else
  *s = std::sin(PI * y); *c = std::cos(PI * y);
#endif
}

// (float) (amp * sin(arg)) exactly as the double-precision expression
// rounds it (the dither offsets, which Marx_Dither_Type keeps as floats).
// arg is reduced by pi/2 in two Cody-Waite parts of 33 bits (k c1 and k c2
// are exact for |k| < 2^18; the part left out, k 2.3e-21, stays below
// 4e-16), sin in double-float.
// The double-float value is within amp 2^-44 of amp sin(arg), the double
// expression within two of its own ulps; when no float rounding boundary
// lies within twice that distance of the value, both round to the same
// float.  Otherwise (about one value in 10^4), and for |arg| >= 2^18, the
// library sine decides.  amp_exp: an integer with amp <= 2^amp_exp.
MXD float sine_to_float(double amp, int amp_exp, double arg) {
#ifdef __CUDA_ARCH__
  const unsigned long long ab = (unsigned long long) __double_as_longlong(arg);
  if (((ab >> 52) & 0x7ffu) < 1023u + 18u) {
    const double magic = 6755399441055744.0;
    const double t = fma(arg, 0x1.45f306dc9c883p-1, magic);   // arg 2/pi + magic
    const double kd = t - magic;
    double r = fma(-kd, 0x1.921fb544p+0, arg);
    r = fma(-kd, 0x1.0b4611a6p-34, r);
    F2 sr, cr;
    df_sincos(df_from(r), sr, cr);
    const int k = __double2loint(t) & 3;
    const F2 w = (k & 1) ? cr : sr;
    const double v = flip_sign(amp * df_to(w), (k & 2) != 0);
    const unsigned long long vb = (unsigned long long) __double_as_longlong(v);
    const int e = (int) ((vb >> 52) & 0x7ffu);
    const int sh = amp_exp + 1031 - e;   // log2 of amp 2^-44 in ulps of v
    if (e >= 897 && e < 1150 && sh < 26) {
      const uint32_t low = (uint32_t) vb & 0x1FFFFFFFu;   // the 29 bits the float rounding drops
      const uint32_t dist = low > 0x10000000u ? low - 0x10000000u : 0x10000000u - low;
      const uint32_t margin = (2u << (sh > 0 ? sh : 0)) + 8u;
      if (dist > margin) return d2f_rn(v);
    }
  }
  return (float) (amp * sin(arg));
#else
  (void) amp_exp;
  return (float) (amp * std::sin(arg));
#endif
}

// sqrt of a float: in double-float on the FP32 pipe (within 2^-46 of the
// double root; it scales the reflectivity, whose test leaves values within
// 2^-24 of the threshold to a double comparison that a last-bit difference
// of the root cannot reach but with a probability near 1e-16).
MXD double sqrt_of_float(float f) {
#ifdef __CUDA_ARCH__
  if (f > 0.0f && f < 3.0e38f) return df_to(df_sqrt(F2{f, 0.0f}));
#endif
  return sqrt((double) f);
}

// a / b from the correctly rounded reciprocal rb = 1/b by one Markstein
// correction: q = a rb, r = a - q b (exact with a fused multiply-add),
// q + r rb rounds to the correctly rounded quotient, as a division does,
// for finite non-zero operands away from overflow and underflow.
MXD double div_by(double a, double b, double rb) {
#ifdef __CUDA_ARCH__
  const double q = a * rb;
  return fma(fma(-q, b, a), rb, q);
#else
  return a / b;
#endif
}
// fmod(x, y) for x >= 0 and 0 < y from the correctly rounded ry = 1/y.
// fmod's result is exact: with the integer quotient q right, x - q y is the
// remainder itself and one fused multiply-add yields it exactly; a q off by
// one (x ry rounded across an integer) shows as a remainder outside [0, y)
// and is corrected.  Other operands take the library fmod.
MXD double fmod_pos(double x, double y, double ry) {
#ifdef __CUDA_ARCH__
  const double qa = x * ry;
  if (x >= 0.0 && qa < 4.0e15) {
    double q = trunc(qa);
    double r = fma(-q, y, x);
    if (r < 0.0) r = fma(-(q - 1.0), y, x);
    else if (r >= y) r = fma(-(q + 1.0), y, x);
    return r;
  }
  return fmod(x, y);
#else
  (void) ry;
  return std::fmod(x, y);
#endif
}

// JDMbinary_search_f (finterpo.c:37): first index with xp >= x (an equal
// element returns its index), n if all are smaller.
MXD unsigned bsearch_f(float x, const float *xp, unsigned n) {
  unsigned n0 = 0, n1 = n;
  while (n1 > n0 + 1) {
    unsigned n2 = (n0 + n1) >> 1;
    float v = xp[n2];
    if (v >= x) { if (v == x) return n2; n1 = n2; }
    else n0 = n2;
  }
  return (x >= xp[n0]) ? n1 : n0;
}
MXD unsigned bsearch_d(double x, const double *xp, unsigned n) {  // JDMbinary_search_d (dinterpo.c:30)
#ifdef __CUDA_ARCH__
  // Non-negative finite x against a non-negative table: IEEE doubles of
  // one sign order as their bit patterns, so the search runs on the
  // integer pipe.
  const unsigned long long bx = (unsigned long long) __double_as_longlong(x);
  if (bx < 0x7ff0000000000000ull) {
    const unsigned long long *xb = (const unsigned long long *) xp;
    unsigned n0 = 0, n1 = n;
    while (n1 > n0 + 1) {
      unsigned n2 = (n0 + n1) >> 1;
      unsigned long long v = __ldg(xb + n2);
      if (v >= bx) { if (v == bx) return n2; n1 = n2; }
      else n0 = n2;
    }
    return (bx >= __ldg(xb + n0)) ? n1 : n0;
  }
#endif
  unsigned n0 = 0, n1 = n;
  while (n1 > n0 + 1) {
    unsigned n2 = (n0 + n1) >> 1;
    double v = MX_LDG(xp + n2);
    if (v >= x) { if (v == x) return n2; n1 = n2; }
    else n0 = n2;
  }
  return (x >= MX_LDG(xp + n0)) ? n1 : n0;
}
// JDMinterpolate_f (finterpo.c:59-86).  The result is rounded to float, so
// the double expression is evaluated without contraction exactly as the
// reference writes it.
// The interval slopes (float dy over double dx, as the reference divides)
// are precomputed on the host, so the kernel only multiplies; the slope of
// the interval between n0 and n1 is slope[min(n0, n1)] in either order.
MXD float interp_f(float x, const float *xp, const float *yp, const double *slope, unsigned n) {
  if (n == 1) return yp[0];
  unsigned n1 = bsearch_f(x, xp, n), n0 = n1 - 1;
  if (n1 < n && x == xp[n1]) return yp[n1];
  if (n1 == n) { n1--; n0--; }
  if (n1 == 0) n0 = 1;
  const float xf0 = xp[n0], xf1 = xp[n1];
  if (xf1 == xf0) return yp[n1];   // the same test in float: the cast is exact
  double q = slope[n0 < n1 ? n0 : n1];
  return d2f_rn(MX_DADD(f2d(yp[n0]), MX_DMUL(q, MX_DADD(f2d(x), -f2d(xf0)))));
}
// Two tables over the same abscissae (the optical constants beta and
// delta): interp_f of each with one binary search.
MXD void interp2_f(float x, const float *xp, const float *ya, const float *yb, const double *sa, const double *sb,
                   unsigned n, float &a, float &b) {
  if (n == 1) { a = ya[0]; b = yb[0]; return; }
  unsigned n1 = bsearch_f(x, xp, n), n0 = n1 - 1;
  if (n1 < n && x == xp[n1]) { a = ya[n1]; b = yb[n1]; return; }
  if (n1 == n) { n1--; n0--; }
  if (n1 == 0) n0 = 1;
  const float xf0 = xp[n0], xf1 = xp[n1];
  if (xf1 == xf0) { a = ya[n1]; b = yb[n1]; return; }
  const unsigned k = n0 < n1 ? n0 : n1;
  const double dx = MX_DADD(f2d(x), -f2d(xf0));
  a = d2f_rn(MX_DADD(f2d(ya[n0]), MX_DMUL(sa[k], dx)));
  b = d2f_rn(MX_DADD(f2d(yb[n0]), MX_DMUL(sb[k], dx)));
}

// ----------------------------------------------------------- variates --
// Philox4x32-10 (Salmon et al., SC'11).  Uniform slot k of photon `tag`
// carries 53 random bits; normals use single-precision Box-Muller.
MXD void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
    uint64_t p0 = (uint64_t) 0xD2511F53u * c[0], p1 = (uint64_t) 0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0, hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
#endif
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}
// m 2^-53 for a 53-bit integer m, built from its bits on the integer pipe
// (the same value the conversion and the multiplication give, without
// their two FP64-pipe instructions).
MXD double unit_from_bits(uint64_t m) {
#ifdef __CUDA_ARCH__
  if (m == 0) return 0.0;
  const int lz = __clzll((long long) m) - 11;   // shift that brings the leading one to bit 52
  return __longlong_as_double((long long) (((uint64_t) (1022 - lz) << 52) | ((m << lz) & 0xFFFFFFFFFFFFFull)));
#else
  return (double) m * (1.0 / 9007199254740992.0);
#endif
}
MXD double philox_uniform(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0001u, 0u};
  philox(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  uint64_t b = ((uint64_t) c[0] << 32) | c[1];
  return unit_from_bits(b >> 11);
}
// Single-precision natural log and cos(2 pi u) for the normal variates,
// from their series (ln m = 2 atanh((m-1)/(m+1)); Taylor series of sin and
// cos on [0, pi/2)) with every operation explicitly rounded, so the CPU
// oracle reproduces each normal bit for bit.
#ifdef __CUDA_ARCH__
#define FADD(a, b) __fadd_rn(a, b)
#define FSUB(a, b) __fsub_rn(a, b)
#define FMUL(a, b) __fmul_rn(a, b)
#define FDIV(a, b) __fdiv_rn(a, b)
#define FSQRT(a) __fsqrt_rn(a)
MXD uint32_t f2u(float f) { return __float_as_uint(f); }
MXD float u2f(uint32_t u) { return __uint_as_float(u); }
#else
#define FADD(a, b) ((a) + (b))
#define FSUB(a, b) ((a) - (b))
#define FMUL(a, b) ((a) * (b))
#define FDIV(a, b) ((a) / (b))
#define FSQRT(a) std::sqrt(a)
inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
#endif
MXD float series_logf(float u) {   // u in (0, 1], normal (u >= 2^-24)
  uint32_t b = f2u(u);
  int e = (int) ((b >> 23) & 0xffu) - 127;
  float m = u2f((b & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = FMUL(m, 0.5f); e += 1; }
  float s = FDIV(FSUB(m, 1.0f), FADD(m, 1.0f));
  float s2 = FMUL(s, s);
  float poly = FMUL(s2, FADD(0.333333333f, FMUL(s2, FADD(0.2f, FMUL(s2, FADD(0.142857143f,
               FMUL(s2, FADD(0.111111111f, FMUL(s2, 0.0909090909f)))))))));
  float lnm = FMUL(FMUL(2.0f, s), FADD(1.0f, poly));
  float fe = (float) e;
  return FADD(FMUL(fe, 0.693145752f), FADD(FMUL(fe, 1.42860677e-06f), lnm));
}
MXD float series_cos2pi(float u) {   // cos(2 pi u), u in [0, 1)
  float x4 = FMUL(u, 4.0f);
  int q = (int) x4;
  float f = FSUB(x4, (float) q);
  float t = FMUL(f, 1.57079632679f), t2 = FMUL(t, t);
  float c = FADD(1.0f, FMUL(t2, FADD(-0.5f, FMUL(t2, FADD(4.16666667e-02f, FMUL(t2, FADD(-1.38888889e-03f,
            FMUL(t2, FADD(2.48015873e-05f, FMUL(t2, FADD(-2.75573192e-07f, FMUL(t2, 2.08767570e-09f))))))))))));
  float s = FMUL(t, FADD(1.0f, FMUL(t2, FADD(-1.66666667e-01f, FMUL(t2, FADD(8.33333333e-03f, FMUL(t2,
            FADD(-1.98412698e-04f, FMUL(t2, FADD(2.75573192e-06f, FMUL(t2, FADD(-2.50521084e-08f,
            FMUL(t2, 1.60590438e-10f)))))))))))));
  return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}
MXD double philox_normal(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0002u, 0u};
  philox(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  float u1 = (float) ((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
  float u2 = (float) (c[1] >> 8) * (1.0f / 16777216.0f);
  float r = FSQRT(FMUL(-2.0f, series_logf(u1)));
  return f2d(FMUL(r, series_cos2pi(u2)));
}

// Source-level draws (photon generation) use their own Philox domain, so
// they never coincide with a stage's slots: draw k of photon `tag`.
MXD double source_uniform(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0003u, 0u};
  philox(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  uint64_t b = ((uint64_t) c[0] << 32) | c[1];
  return unit_from_bits(b >> 11);
}

// Variate source for one photon: fixed per-stage slot windows.
struct Rng {
  const double *U, *N;   // slot-major pre-drawn arrays, or null for Philox
  uint64_t seed;
  uint32_t n, i, tag;
  int upos, uend, npos, nend;
  bool overrun;
  MXD void window(int ub, int uc, int nb, int nc) { upos = ub; uend = ub + uc; npos = nb; nend = nb + nc; }
  MXD double uniform() {
    if (upos >= uend) { overrun = true; return 0.5; }
    int k = upos++;
    return U ? MX_LDG(U + (size_t) k * n + i) : philox_uniform(seed, tag, (uint32_t) k);
  }
  // Pass over the next uniform slot without drawing it (a test whose
  // outcome is known: a probability of 1).
  MXD void skip_uniform() {
    if (upos >= uend) overrun = true;
    else upos++;
  }
  // Pass over the next normal slot without drawing it (a normal that is
  // multiplied by zero).
  MXD void skip_normal() {
    if (npos >= nend) overrun = true;
    else npos++;
  }
  MXD double normal() {
    if (npos >= nend) { overrun = true; return 0.0; }
    int k = npos++;
    return N ? MX_LDG(N + (size_t) k * n + i) : philox_normal(seed, tag, (uint32_t) k);
  }
};

// Photon state held in registers through the fused trace.
struct Ph {
  double e, t;
  D3 x, p;
  uint32_t flags;
  int shell, order, ccd;
  float ypix, zpix, dith[3];
  // outputs of the LETG and HRC stages, valid where `set` says so
  int8_t sup[4];               // LETG support orders (set bit 1)
  int16_t pha;                 // HRC pulse height    (set bit 2)
  uint8_t region;              // HRC-S shield region (set bit 2)
  uint8_t set;
  float upix, vpix;            // HRC-S u, v pixel    (set bit 4)
  float pi;                    // ACIS PI energy      (set bit 16)
};
#define MX_SET_SUPPORT 1u
#define MX_SET_HRC 2u     // pulse height (HRC, or ACIS with an FEF)
#define MX_SET_UV 4u
#define MX_SET_REGION 8u
#define MX_SET_PI 16u

// ------------------------------------------------------------- mirror --
// JDMquadratic_root (qroot.c:36-70), same cancellation-free form.
MXD int quadratic_root(double a, double b, double c, double &rp, double &rm) {
  if (is_zero(a)) return -1;
  double bsqr = b * b, ac4 = a * c * 4;
  const long long kb = dkey(bsqr), ka = dkey(ac4);
  if (kb > ka) {
    // rp = -2c / (b f), rm = -b f / (2a) from one reciprocal of a b f,
    // with b f = b (1 + sqrt(1 - 4ac/b^2)) = b + sign(b) sqrt(b^2 - 4ac)
    double bf = b + copysign(sqrt_fast(bsqr - ac4), b), inv = rcp_fast(a * bf);
    rp = -2.0 * c * a * inv;
    rm = -0.5 * bf * bf * inv;
    return 1;
  }
  if (kb == ka) { rp = rm = -b / (2.0 * a); return 1; }
  return 0;
}

// compute_conic_intersection (hrma.c:411-478) for x^2+y^2+z^2 = a x^2+b x+c.
MXD int conic_intersection(const MxShellDev &h, int o, D3 &x0, D3 p, D3 &normal) {
  double a = h.a[o], b = h.b[o];
  double t_plus = -x0.x * rcp_fast(p.x), t_minus;
  double x_y = x0.y + t_plus * p.y, x_z = x0.z + t_plus * p.z;
  double alpha = a * p.x * p.x - 1.0;
  double beta = b * p.x - 2.0 * (p.y * x_y + p.z * x_z);
  double gamma = h.c[o] - x_z * x_z - x_y * x_y;
  if (is_zero(alpha)) {
    if (is_zero(beta)) return -1;
    t_plus = t_minus = -gamma / beta;
  } else if (0 >= quadratic_root(alpha, beta, gamma, t_plus, t_minus)) return -1;
  double x_plus = p.x * t_plus, x_minus = p.x * t_minus;
  double xmin = h.xmin[o], xmax = h.xmax[o], t;
  const long long kp = dkey(x_plus), km = dkey(x_minus), kmin = dkey(xmin), kmax = dkey(xmax);
  bool okp = (kp >= kmin) && (kp < kmax), okm = (km >= kmin) && (km < kmax);
  if (okp) t = (okm && km > kp) ? t_minus : t_plus;
  else if (okm) t = t_minus;
  else return -1;
  x0 = mk(p.x * t, x_y + p.y * t, x_z + p.z * t);
  normal = normalized(mk(fma(h.am1[o], x0.x, h.hb[o]), -x0.y, -x0.z));   // ((a - 1) x + b/2, -y, -z)
  return 0;
}

// blur_normal (hrma.c:1054-1093): rotate n by a normal-distributed angle
// about a random axis perpendicular to it.
// With e1 = (0, n.z, -n.y) / len the first perpendicular, e2 = n x e1 and
// perp = cos(phi) e1 + sin(phi) e2 the rotated one, the rotation of unit n
// about unit perp by ang is cos(ang) n + sin(ang) (perp x n), and
// perp x n = sin(phi) e1 - cos(phi) e2, where
// e2 = (-len, n.x n.y / len, n.x n.z / len): the two Rodrigues rotations
// of the reference in closed form, one normalisation.
MXD void blur_normal(D3 &n, double blur_rad, Rng &rng) {
  const double l2 = n.y * n.y + n.z * n.z, inv = mx_rsqrt(l2), len = l2 * inv;
  double s, c;
  sincospi_fast(2.0 * rng.uniform(), &s, &c);   // phi = 2 pi u
  double ang = blur_rad * rng.normal();
  double sa, ca;
  sincos_small(ang, &sa, &ca);
  const double nxy = n.x * n.y, nxz = n.x * n.z;
  const D3 w = mk(c * len, (s * n.z - c * nxy) * inv, (-s * n.y - c * nxz) * inv);   // perp x n
  // a rotation of a unit vector: unit to the last bits without the
  // reference's renormalisation, which moves it by less than 1e-15
  n = ca * n + sa * w;
}

// marx_reflectivity (reflect.c:39-77): polarisation-averaged Fresnel
// |r|^2 for n = 1 - delta + i beta (Jackson 7.39, 7.41), with
// |num/den|^2 = |num|^2 / |den|^2, returned as num / den (den > 0) so that
// the reflectivity test can decide u * den < num without the division.
MXD void reflectivity_parts(double cos_t, double beta, double delta, double &num, double &den) {
  double nr = 1.0 - delta, ni = beta;
  double sin2 = 1.0 - cos_t * cos_t;                     // sin_theta^2
  double sr = nr * nr - ni * ni, si = 2.0 * nr * ni;     // n^2
  double wr = sr - sin2, wi = si;                        // n^2 - sin^2
  // principal square root, branches as JDMc_sqrt (complex.c:201)
  double rr, ri;
  double r = sqrt(wr * wr + wi * wi);
  if (is_zero(r)) { rr = wr; ri = wi; }
  else if (!neg_bit(wr) || is_zero(wr)) {
    double h = 0.5 * (r + wr), inv = mx_rsqrt(h);
    rr = h * inv; ri = 0.5 * wi * inv;
  } else {
    double h = 0.5 * (r - wr), inv = mx_rsqrt(h);
    rr = 0.5 * wi * inv; ri = h * inv;
    if (neg_bit(rr) && !is_zero(rr)) { rr = -rr; ri = -ri; }
  }
  // e_perp = (cos - root) / (cos + root)
  double a1 = (cos_t - rr) * (cos_t - rr) + ri * ri, b1 = (cos_t + rr) * (cos_t + rr) + ri * ri;
  // e_par = (cos n^2 - root) / (cos n^2 + root)
  double pr = cos_t * sr, pi_ = cos_t * si;
  double a2 = (pr - rr) * (pr - rr) + (pi_ - ri) * (pi_ - ri);
  double b2 = (pr + rr) * (pr + rr) + (pi_ + ri) * (pi_ + ri);
  num = 0.5 * (a1 * b2 + a2 * b1);
  den = b1 * b2;
}
MXD double reflectivity(double cos_t, double beta, double delta) {
  double num, den;
  reflectivity_parts(cos_t, beta, delta, num, den);
  return num / den;
}

// interpolate_theta (wfold.c:304-332) on one fold array.
MXD double fold_theta(const MxTables &T, int table, unsigned a, double p) {
  const double *hd = T.fold_hdr + ((size_t) table * MX_FOLD_MAX + a) * 8;
  double p_min = MX_LDG(hd + 1), p_max = MX_LDG(hd + 3);
  if (dkey(p) < dkey(p_min)) return 0.0;
#ifdef __CUDA_ARCH__
  // the power law of the tail as exp(b log(a (1 - p))), a (1 - p) > 0: within
  // about 1e-14 relative of pow, and about half its FP64 instructions
  if (dkey(p_max) < dkey(p)) return exp(MX_LDG(hd + 5) * log(MX_LDG(hd + 4) * (1.0 - p)));
#else
  if (p > p_max) return std::pow(MX_LDG(hd + 4) * (1.0 - p), MX_LDG(hd + 5));
#endif
  double di = (p - p_min) * MX_LDG(hd + 7);
  unsigned i = trunc_to_unsigned(di);
  unsigned num = trunc_to_unsigned(MX_LDG(hd + 6));
  const float *t = T.fold_theta + ((size_t) table * MX_FOLD_MAX + a) * MX_FOLD_THETA;
  if (i + 1 >= num) return (double) MX_LDG(t + num - 1);
  di -= u2d(i);
  return (1.0 - di) * f2d(MX_LDG(t + i)) + di * f2d(MX_LDG(t + i + 1));
}
// marx_wfold_table_interp (wfold.c:334-363).
MXD double wfold_interp(const MxTables &T, int table, double energy, double sin_alpha, double r) {
  unsigned num = T.fold_num[table];
  if (num == 1) return fold_theta(T, table, 0, r);
  double ea = energy * sin_alpha;
  const double *eas = T.fold_ealpha + (size_t) table * MX_FOLD_MAX;
  unsigned i = bsearch_d(ea, eas, num);
  if (i == num) i--;
  if (i == 0) i++;
  double t0 = fold_theta(T, table, i - 1, r), t1 = fold_theta(T, table, i, r);
  double e0 = MX_LDG(eas + i - 1);
  return t0 + (t1 - t0) * (ea - e0) * MX_LDG(T.fold_inv_de + (size_t) table * MX_FOLD_MAX + i - 1);
}

// reflect_from_conic (hrma.c:488-545) after the intersection, in two
// parts so that the wavefront can drop absorbed photons before the rest of
// the reflection.  reflect_test: normal blur and the reflectivity test;
// false if the photon is absorbed (p is left as the reference leaves it).
// pdn receives p.n with the blurred normal n.
MXD bool reflect_test(const MxTables &T, const MxShellDev &h, int o, D3 p, D3 &n, double &pdn, double beta,
                      double delta, double corr, Rng &rng) {
  if (T.use_blur) blur_normal(n, h.blur[o], rng);
  pdn = dot(p, n);
  if (!T.ideal) {
    double r = rng.uniform();
#ifdef __CUDA_ARCH__
    // decided in double-float, unless r * den and num * corr lie within
    // 2^-24 of each other (far wider than the two evaluations' difference):
    // then the double-precision values decide, as below
    {
      F2 fn, fd;
      reflectivity_df(fabs(pdn), d2f_trunc(beta), d2f_trunc(delta), fn, fd);
      const double x = r * df_to(fd), y = df_to(fn) * corr, gap = x - y, ag = fabs(gap);
      if (lt_pos(0x1p-100, y) && lt_pos(0x1p-24 * y, ag) && lt_pos(ag, 0x1p+100)) return neg_bit(gap);
    }
#endif
    double num, den;
    reflectivity_parts(fabs(pdn), beta, delta, num, den);
    // r >= rfl * corr with rfl = num / den, den > 0, decided without the
    // division (the two differ only for r within an ulp of the threshold)
    if (dkey(r * den) >= dkey(num * corr)) return false;
  }
  return true;
}
// reflect_finish: specular reflection and WFold scattering.  Returns -1 if
// the scattering angle exceeds pi/4 (p then holds the specular direction,
// as in the reference), 0 otherwise.
MXD int reflect_finish(const MxTables &T, const MxShellDev &h, int o, int table, D3 &p, D3 n, double pdn,
                       double energy, Rng &rng) {
  p = p + (-2.0 * pdn) * n;
  if (!T.use_wfold) return 0;
  double r = rng.uniform();
  double dg = wfold_interp(T, table, energy, -pdn, r) * h.scat[o];
  if (dkey(dg) > dkey(PI / 4)) return -1;
  if (lt_pos(rng.uniform(), 0.5)) dg = -dg;
  // JDMv_rotate_unit_vector(p, p x n, dg): with a = p x n, p.a = 0 and
  // a x p = n - (p.n) p for unit p, so p becomes cos(dg) p + sin(dg) (n - (p.n) p)
  double sg, cg;
  sincos_small(dg, &sg, &cg);
  const double pn = dot(p, n);
  p = normalized_unit(cg * p + sg * (n + (-pn) * p));
  return 0;
}

// intersects_struts (hrma.c:928-968): three bars rotated by 60 degrees.
MXD bool struts_block_exact(const MxTables &T, int set, D3 x, D3 p) {
  double inv_px = 1.0 / p.x;
  for (int k = 0; k < 2; k++) {
    double hw = T.strut_half_width[set][k];
    double t = (T.strut_xpos[set][k] + T.cap - x.x) * inv_px;
    double y = x.y + p.y * t, z = x.z + p.z * t;
    for (int i = 0; i < 3; i++) {
      if (i != 0) { double tmp = T.cos30 * y - T.sin30 * z; z = T.sin30 * y + T.cos30 * z; y = tmp; }
      if (((-hw < y) && (y < hw)) || ((-hw < z) && (z < hw))) return true;
    }
  }
  return false;
}

// The same test screened in single precision: the bar coordinates of the
// ray in float carry an absolute error far below MX_STRUT_MARGIN (under
// 2e-3 mm for positions of 1e4 mm and directions within a few degrees of
// the axis), so a coordinate more than the margin inside or outside every
// bar edge decides the test as the double-precision one would.  Rays with
// a coordinate within the margin of an edge, or not finite, take the
// double-precision test.
#define MX_STRUT_MARGIN 0.05f
// The screen on float coordinates: 1 blocked, 0 clear, -1 unsure.
MXD int struts_screen(const MxTables &T, int set, float xx, float xy, float xz, float px, float py, float pz) {
  const float inv = 1.0f / px;
  bool unsure = false;
  for (int k = 0; k < 2; k++) {
    const float hw = T.strut_hwf[set][k];
    const float t = (T.strut_xf[set][k] - xx) * inv;
    float y = xy + py * t, z = xz + pz * t;
    for (int i = 0; i < 3; i++) {
      if (i != 0) { float tmp = T.cos30f * y - T.sin30f * z; z = T.sin30f * y + T.cos30f * z; y = tmp; }
      const float dy = fabsf(y) - hw, dz = fabsf(z) - hw;
      if (dy < -MX_STRUT_MARGIN || dz < -MX_STRUT_MARGIN) return 1;
      if (!(dy > MX_STRUT_MARGIN && dz > MX_STRUT_MARGIN)) unsure = true;
    }
  }
  return unsure ? -1 : 0;
}
MXD bool struts_block(const MxTables &T, int set, D3 x, D3 p) {
#ifdef __CUDA_ARCH__
  const int s = struts_screen(T, set, d2f_trunc(x.x), d2f_trunc(x.y), d2f_trunc(x.z), d2f_trunc(p.x),
                              d2f_trunc(p.y), d2f_trunc(p.z));
  if (s >= 0) return s == 1;
#endif
  return struts_block_exact(T, set, x, p);
}
// The photon between the mirrors, from the paraboloid's frame to the MARX
// frame (JDM3m_vector_mul by bwd[0], less to_osac[0]), where the reference
// tests the cap struts and leaves a blocked photon.
MXD void paraboloid_to_marx(const MxShellDev &h, D3 &x, D3 &p) {
  p = mat_mul(h.bwd[0], p);
  x = mat_mul(h.bwd[0], x);
  x = x - mk(h.to_osac[0][0], h.to_osac[0][1], h.to_osac[0][2]);
}
// The cap struts (set 1) for a photon given in the paraboloid's frame: the
// screen runs on its MARX-frame coordinates formed in single precision
// (bwd[0] and to_osac[0] in float).  The frame change adds a few float
// roundings of the 1e4 mm positions, under 4e-3 mm in all with the
// conversions, and under 1e-4 mm at the bars for directions within a few
// degrees of the axis: far inside MX_STRUT_MARGIN.  Near an edge the
// double-precision coordinates decide, as in struts_block.
MXD bool cap_struts_block(const MxTables &T, const MxShellDev &h, D3 x, D3 p) {
#ifdef __CUDA_ARCH__
  const float xx = d2f_trunc(x.x), xy = d2f_trunc(x.y), xz = d2f_trunc(x.z);
  const float px = d2f_trunc(p.x), py = d2f_trunc(p.y), pz = d2f_trunc(p.z);
  const float *m = h.bwd0f;
  const int s = struts_screen(T, 1, fmaf(m[0], xx, fmaf(m[1], xy, m[2] * xz)) - h.osac0f[0],
                              fmaf(m[3], xx, fmaf(m[4], xy, m[5] * xz)) - h.osac0f[1],
                              fmaf(m[6], xx, fmaf(m[7], xy, m[8] * xz)) - h.osac0f[2],
                              fmaf(m[0], px, fmaf(m[1], py, m[2] * pz)), fmaf(m[3], px, fmaf(m[4], py, m[5] * pz)),
                              fmaf(m[6], px, fmaf(m[7], py, m[8] * pz)));
  if (s >= 0) return s == 1;
#endif
  paraboloid_to_marx(h, x, p);
  return struts_block_exact(T, 1, x, p);
}

// Mirror state carried between the three parts of the HRMA trace: the
// photon at a conic intersection (OSAC frame of that optic) that passed
// that optic's reflectivity test, its incoming direction, the blurred
// normal there and p.n, and the optical constants at the photon's energy.
struct MirrorState {
  D3 x, p, n;
  double corr, pdn;
  float beta, delta;
};

// _marx_hrma_mirror_reflect per photon (hrma.c:1183-1339), part 1:
// vignetting, project_photon_to_hrma (hrma.c:984-1050), transform into the
// paraboloid's frame, optical constants, paraboloid intersection.  Returns
// true if the photon reached the paraboloid.
MXD bool mirror_front(const MxTables &T, const MxShellDev *shells, const float *optc, const double *slope, Ph &ph,
                      Rng &rng, MirrorState &m) {
  rng.window(MX_U_MIRROR, 12, MX_N_MIRROR, 2);
  if (!T.ideal) {
    // a uniform in [0, 1) never exceeds a vignetting factor of 1
    if (dkey(T.hrma_vig) >= dkey(1.0)) rng.skip_uniform();
    else if (lt_pos(T.hrma_vig, rng.uniform())) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;
    if (ph.flags & MX_BAD_PHOTON_MASK) return false;
  }
  D3 x = ph.x, p = ph.p;
  int si = -1;
  for (int guard = 0; guard < 64 && si < 0; guard++) {
    double r = rng.uniform();
    if (rng.overrun) return false;
    for (int i = 0; i < 4; i++)
      if (lt_pos(r, shells[i].area_fraction)) { si = i; break; }
  }
  if (si < 0) { rng.overrun = true; return false; }
  const MxShellDev &h = shells[si];
  ph.shell = si;
  double radius;
  if (T.area_uniform) {
    double r0 = h.min_radius, r1 = h.max_radius;
    radius = sqrt_fast(r0 * r0 + (r1 * r1 - r0 * r0) * rng.uniform());
  } else
    radius = h.min_radius + h.dr * rng.uniform();
  double theta;
  for (int guard = 0;; guard++) {
    theta = rng.uniform();
    unsigned quad = quarter_of(theta);
    if (rng.overrun || guard >= 64) { rng.overrun = true; return false; }
    if (h.shutter & (1u << quad)) break;
  }
  double st, ct;
  sincospi_fast(fma(theta, 2.0, -0.25), &st, &ct);   // angle 2 pi (u - 1/8)
  x = mk(h.front_position, radius * st - h.to_osac[0][1], radius * ct - h.to_osac[0][2]);
  if (dkey(T.source_distance) > 0) p = normalized(x + T.source_distance * p);
  if (T.use_struts && struts_block(T, 0, x, p)) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;

  // fwd (x + to_osac): (r sin - t1) + t1 is r sin to within an ulp of t1,
  // and the first column's product with the front plane is a constant
  {
    const double y = radius * st, z = radius * ct;
    const double *f = h.fwd[0];
    x = mk(fma(f[2], z, fma(f[1], y, h.front_fwd[0])), fma(f[5], z, fma(f[4], y, h.front_fwd[1])),
           fma(f[8], z, fma(f[7], y, h.front_fwd[2])));
  }
  p = mat_mul(h.fwd[0], p);
  m.beta = 0.0f; m.delta = 1.0f; m.corr = 1.0;
  if (T.opt_n) {
    float fe = d2f_rn(ph.e);
    interp2_f(fe, optc, optc + T.opt_n, optc + 2 * T.opt_n, slope, slope + (T.opt_n - 1), T.opt_n, m.beta, m.delta);
    if (T.use_scale) {
      const float *ce = optc + 3 * T.opt_n + h.corr_off;
      m.corr = sqrt_of_float(interp_f(fe, ce, ce + h.corr_n, slope + h.corr_slope_off, h.corr_n));
    }
  }
  D3 n;
  if (-1 == conic_intersection(h, 0, x, p, n)) { ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = x; ph.p = p; return false; }
  m.x = x; m.p = p; m.n = n;
  return true;
}

// Part 2: normal blur and reflectivity test at the paraboloid.  Returns
// false if the photon is absorbed there.
MXD bool mirror_ptest(const MxTables &T, const MxShellDev *shells, Ph &ph, Rng &rng, MirrorState &m) {
  if (!reflect_test(T, shells[ph.shell], 0, m.p, m.n, m.pdn, m.beta, m.delta, m.corr, rng)) {
    ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = m.x; ph.p = m.p; return false;
  }
  return true;
}

// Part 3: the rest of the reflection from the paraboloid, back to the MARX
// frame, cap struts, into the hyperboloid's frame, its intersection, normal
// blur and reflectivity test.
MXD bool mirror_middle(const MxTables &T, const MxShellDev *shells, Ph &ph, Rng &rng, MirrorState &m) {
  const MxShellDev &h = shells[ph.shell];
  D3 x = m.x, p = m.p;
  if (0 != reflect_finish(T, h, 0, 2 * ph.shell, p, m.n, m.pdn, ph.e, rng)) {
    ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = x; ph.p = p; return false;
  }
  if (T.use_struts && cap_struts_block(T, h, x, p)) {
    paraboloid_to_marx(h, x, p);   // a blocked photon stays in the MARX frame
    ph.flags |= MX_PHOTON_MIRROR_VBLOCKED; ph.x = x; ph.p = p; return false;
  }
  // into the hyperboloid's frame: bwd[0], less to_osac[0], plus to_osac[1],
  // fwd[1] as one matrix and offset (18 operations instead of 42; within a
  // few ulps of the two steps), with a fixed order of multiply-adds
  {
    const double *M = h.mid, *c = h.mid_off;
    p = mk(fma(M[0], p.x, fma(M[1], p.y, MX_DMUL(M[2], p.z))), fma(M[3], p.x, fma(M[4], p.y, MX_DMUL(M[5], p.z))),
           fma(M[6], p.x, fma(M[7], p.y, MX_DMUL(M[8], p.z))));
    x = mk(fma(M[0], x.x, fma(M[1], x.y, fma(M[2], x.z, c[0]))), fma(M[3], x.x, fma(M[4], x.y, fma(M[5], x.z, c[1]))),
           fma(M[6], x.x, fma(M[7], x.y, fma(M[8], x.z, c[2]))));
  }
  D3 n;
  if (-1 == conic_intersection(h, 1, x, p, n)) { ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = x; ph.p = p; return false; }
  if (!reflect_test(T, h, 1, p, n, m.pdn, m.beta, m.delta, m.corr, rng)) {
    ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = x; ph.p = p; return false;
  }
  m.x = x; m.p = p; m.n = n;
  return true;
}

// Part 4: the rest of the reflection from the hyperboloid, back to the
// MARX frame, post-collimator struts.  Leaves the photon in ph.
MXD void mirror_back(const MxTables &T, const MxShellDev *shells, Ph &ph, Rng &rng, MirrorState &m) {
  const MxShellDev &h = shells[ph.shell];
  D3 x = m.x, p = m.p;
  if (0 != reflect_finish(T, h, 1, 2 * ph.shell + 1, p, m.n, m.pdn, ph.e, rng)) {
    ph.flags |= MX_PHOTON_UNREFLECTED; ph.x = x; ph.p = p; return;
  }
  p = mat_mul(h.bwd[1], p);
  x = mat_mul(h.bwd[1], x);
  x = x - mk(h.to_osac[1][0], h.to_osac[1][1], h.to_osac[1][2]);
  if (T.use_struts && struts_block(T, 2, x, p)) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;
  ph.x = x; ph.p = p;
}

MXD void mirror_stage(const MxTables &T, const MxShellDev *shells, const float *optc, const double *slope, Ph &ph,
                      Rng &rng) {
  MirrorState m;
  if (mirror_front(T, shells, optc, slope, ph, rng, m) && mirror_ptest(T, shells, ph, rng, m) &&
      mirror_middle(T, shells, ph, rng, m))
    mirror_back(T, shells, ph, rng, m);
}

// ------------------------------------------------------------- dither --
// rotate_unit about the x axis: n = (1, 0, 0), n x p = (0, -p.z, p.y).
MXD D3 rotate_x(D3 p, double c, double s) {
  return normalized_unit(mk(c * p.x + p.x * (1.0 - c), c * p.y - s * p.z, c * p.z + s * p.y));
}

// get_aspsol_point + get_aspsol_dither (dither.c:342-371) at time t
// (start_time + arrival time): the rows j - 1, j around t, j the first row
// later than t as the forward reader leaves them, interpolated linearly and
// stored in float as Marx_Dither_Type holds them (ra, dec, roll, dy, dz,
// dtheta).  False when no row is later than t: the reader has run off the
// end of the file.
MXD bool aspsol_state(const MxTables &T, double t, float s[6]) {
  const uint32_t n = T.asp_n;
  if (n == 0 || !(t < T.asp_t[n])) return false;
  uint32_t lo = 1, hi = n;   // asp_t[hi] > t
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (T.asp_t[mid] > t) hi = mid; else lo = mid + 1;
  }
  const double t0 = T.asp_t[lo - 1], t1 = T.asp_t[lo];
  double dt = MX_DADD(t1, -t0);
  if (dt != 0) dt = MX_DDIV(MX_DADD(t, -t0), dt);
  const double *a = T.asp_v + 8 * (size_t) (lo - 1), *b = a + 8;
  for (int k = 0; k < 6; k++) s[k] = (float) MX_DADD(a[k], MX_DMUL(dt, MX_DADD(b[k], -a[k])));
  return true;
}

#ifdef __CUDA_ARCH__
// apply_dither's rotation (below) for offsets ra, dec under 1e-4 rad, as the
// change it makes: p' = p + D with
//   D = -d p + k n + n x p,  n = (0, sin dec, -cos dec sin ra),
//   d = 1 - cos dec cos ra,  k = (p.n) (1/2 + d/4 + d^2/8),
// the terms of D (below 1e-4) in double-float on the FP32 pipe and the sum
// with p in double.  sin and cos go to x^3 and x^2 (the next terms are
// below 1e-18 relative) as in sincos_small, and d is formed as
// (ra^2 + dec^2)/2 - ra^2 dec^2/4, without the cancellation that costs the
// double evaluation seven digits of d.  Eleven FP64 operations (the
// splits, the sums back to double and the additions to p) instead of about
// thirty-five; the result is within an ulp or two of the double evaluation.
__device__ __forceinline__ D3 dither_rotate_df(D3 p, double ra, double dec) {
  const F2 sixth = {0x1.555556p-3f, -0x1.555556p-28f};   // 1/6
  const F2 r = df_from(ra), e = df_from(dec);
  const F2 r2 = df_sqr(r), e2 = df_sqr(e);
  const F2 sr = df_sub(r, df_mul(df_mul(r, r2), sixth)), sd = df_sub(e, df_mul(df_mul(e, e2), sixth));
  const F2 cd = df_add(F2{1.0f, 0.0f}, F2{-0.5f * e2.h, -0.5f * e2.l});
  const F2 ny = sd, nz = df_neg(df_mul(cd, sr));
  const F2 h = df_add(r2, e2), q = df_mul(r2, e2);
  const F2 d = df_sub(F2{0.5f * h.h, 0.5f * h.l}, F2{0.25f * q.h, 0.25f * q.l});
  const F2 px = df_from(p.x), py = df_from(p.y), pz = df_from(p.z);
  const F2 pn = df_add(df_mul(py, ny), df_mul(pz, nz));
  const F2 k = df_mul(pn, df_add(F2{0.5f, 0.0f}, df_mul(d, df_add(F2{0.25f, 0.0f}, df_mul_f(d, 0.125f)))));
  const F2 md = df_neg(d);
  const F2 dx = df_add(df_mul(md, px), df_sub(df_mul(ny, pz), df_mul(nz, py)));
  const F2 dy = df_add(df_add(df_mul(md, py), df_mul(k, ny)), df_mul(nz, px));
  const F2 dz = df_sub(df_add(df_mul(md, pz), df_mul(k, nz)), df_mul(ny, px));
  return mk(p.x + df_to(dx), p.y + df_to(dy), p.z + df_to(dz));
}
#endif

// get_internal_dither / get_aspsol_dither + dither_ray + apply_dither
// (dither.c:167-182, 350-389, 551-581, 609-628).  The dither angles pass
// through float as they do in Marx_Dither_Type.
MXD void dither_stage(const MxTables &T, Ph &ph, Rng &rng) {
  rng.window(0, 0, MX_N_DITHER, 2);
  float fra, fdec, froll;
  if (T.dither_file) {
    float s[6];
    if (!aspsol_state(T, T.start_time + ph.t, s)) { ph.flags |= MX_PHOTON_ASPECT_END; return; }
    ph.dith[0] = s[0]; ph.dith[1] = s[1]; ph.dith[2] = s[2];
    // record only (get_aspsol_dither_record_only, :404-418): the rays are
    // already dithered; the aspect blur still applies
    fra = T.asp_record_only ? 0.0f : s[0];
    fdec = T.asp_record_only ? 0.0f : s[1];
    froll = T.asp_record_only ? 0.0f : s[2];
  } else {
    // (a zero start time or phase is added exactly: skipped)
    double t = (2.0 * PI) * (is_zero(T.start_time) ? ph.t : T.start_time + ph.t);
    // amp * sin(2 pi t / period + phase) rounded to float as the reference
    // stores it; a zero amplitude makes it zero whatever the sine
    float f[2];
    for (int k = 0; k < 2; k++)
      f[k] = !is_zero(T.dith_amp[k])
                 ? sine_to_float(T.dith_amp[k], T.dith_amp_exp[k],
                                 is_zero(T.dith_phase[k]) ? div_by(t, T.dith_period[k], T.dith_inv_period[k])
                                                          : div_by(t, T.dith_period[k], T.dith_inv_period[k]) +
                                                                T.dith_phase[k])
                 : 0.0f;
    fra = f[0];
    fdec = f[1];
    if (T.roll_fixed) froll = T.roll_f;
    else froll = (float) (T.nominal_roll + T.dith_amp[2] * sin(div_by(t, T.dith_period[2], T.dith_inv_period[2]) +
                                                                T.dith_phase[2]));
    ph.dith[0] = fra; ph.dith[1] = fdec; ph.dith[2] = froll;
  }
  double ra = f2d(fra) + T.aspect_blur * rng.normal();
  double dec = f2d(fdec) + T.aspect_blur * rng.normal();
  // roll about the x axis (JDMv_rotate_unit_vector with n = x); a fixed
  // roll of zero leaves p as it is
  D3 p = ph.p;
  if (!T.roll_fixed) {
    double sr, cr;
    sincos_small(-f2d(froll), &sr, &cr);
    p = rotate_x(p, cr, sr);
  } else if (!T.roll_zero)
    p = rotate_x(p, T.roll_cos, T.roll_sin);
#ifdef __CUDA_ARCH__
  // arcsecond offsets (the usual case): the same rotation in double-float
  const double ara = fabs(ra), adec = fabs(dec);
  if (lt_pos(ara, 1e-4) && lt_pos(adec, 1e-4) && (lt_pos(1e-19, ara) || lt_pos(1e-19, adec))) {
    ph.p = dither_rotate_df(p, ra, dec);
    return;
  }
#endif
  double sr, cr, sd, cd;
  sincos_small(ra, &sr, &cr);
  sincos_small(dec, &sd, &cd);
  double cos_theta = cd * cr;
  D3 n = mk(0, sd, -cd * sr);
  double s2 = n.y * n.y + n.z * n.z;
  if (!lt_pos(1e-40, s2)) { ph.p = p; return; }
  // rotate_unit(p, n / s, cos_theta, s) with s = |n| written without the
  // unit axis: cos p + ((p.n)(1 - cos) / s^2) n + n x p, n.x = 0.  With
  // s^2 = sin^2 the factor (1 - cos) / s^2 is 1 / (1 + cos) = 1 / (2 - d),
  // d = 1 - cos; for arcsecond offsets (d < 1e-6) its series
  // 1/2 + d/4 + d^2/8 is exact to 1e-19 and saves the division.
  const double pn = p.y * n.y + p.z * n.z;
  const double d = 1.0 - cos_theta;
  const double k = lt_pos(d, 1e-6) ? pn * (0.5 + d * (0.25 + d * 0.125)) : pn * d / s2;
  // a rotation of a unit vector: unit to the last bits without the
  // reference's renormalisation, which moves it by less than 1e-15
  ph.p = mk(cos_theta * p.x + (n.y * p.z - n.z * p.y), cos_theta * p.y + k * n.y + n.z * p.x,
            cos_theta * p.z + k * n.z - n.y * p.x);
}

// ------------------------------------------------------------ grating --
MXD D3 rot_x(D3 a, double c, double s) { return mk(a.x, c * a.y - s * a.z, s * a.y + c * a.z); }

// a l + b d + c n with a fixed order of fused multiply-adds, so that every
// kernel that inlines it rounds it alike (left to the compiler, the
// contraction of a sum of products may differ from one kernel to another).
MXD D3 comb3(double a, D3 l, double b, D3 d, double c, D3 n) {
  return mk(fma(a, l.x, fma(b, d.x, MX_DMUL(c, n.x))), fma(a, l.y, fma(b, d.y, MX_DMUL(c, n.y))),
            fma(a, l.z, fma(b, d.z, MX_DMUL(c, n.z))));
}
// intersect + newtons_quartic (diffract.c:622-687): Rowland torus.
MXD int rowland_intersect(D3 &x0, D3 p, double rowland) {
  double t = -x0.x * rcp_fast(p.x);
  x0 = mk(0.0, x0.y + p.y * t, x0.z + p.z * t);
  double pxpz = p.x * p.x + p.z * p.z;
  double x2 = x0.z * x0.z + x0.y * x0.y;
  double r2 = rowland * rowland;
  double pdotx = p.y * x0.y + p.z * x0.z;
  double a = 4.0 * pdotx;
  double b = 2.0 * x2 + a * pdotx - r2 * pxpz;
  double c = a * x2 - 2.0 * r2 * p.z * x0.z;
  double d = x2 * x2 - r2 * x0.z * x0.z;
  double t0 = -rowland * sqrt_fast(pxpz);
  double a2 = 2.0 * a, a3 = 3.0 * a, b2 = 2.0 * b;
  for (int it = 0; it < 10; it++) {
    double tt = t0 * t0;
    double num = tt * (3.0 * tt + a2 * t0 + b) - d;
    double den = tt * (4.0 * t0 + a3) + b2 * t0 + c;
    t = num * rcp_fast(den);
    if (lt_pos(fabs(t - t0), 1.0e-4)) { x0 = x0 + t * p; return 0; }
    t0 = t;
  }
  return -1;
}

// diffract_photon (diffract.c:706-823) for a primary grating (theta = 0)
// with facet sectors when the grating has them.
MXD int diffract_photon(const MxTables &T, const MxGratingDev &g, int order_idx, double energy,
                        D3 x, D3 &P, Rng &rng) {
  double nlod = MX_LDG(T.order_k + g.order_off + order_idx) * rcp_fast(energy);
  const double xx = dot(x, x);
  const D3 n = is_zero(xx) ? -1.0 * x : (-mx_rsqrt(xx)) * x;   // -x / |x|
  D3 l = normalized(mk(n.z, 0.0, -n.x));
  D3 d = cross(n, l);
  double dtheta, dpp;
  if (g.nsec > 0) {
    const double *smin = T.sectors + g.sec_off;          // [6][nsec]: min max dth dthb dpp dppb
    const unsigned ns = (unsigned) g.nsec;
    unsigned sn = ns;   // ns: not settled by the screen
#ifdef __CUDA_ARCH__
    {
      // single-precision screen: the azimuth from atan2f is within 2e-6 rad
      // of the double one; a photon more than 1e-5 rad inside a sector
      // (from its two edges and the next sector's start) is in that sector
      // in double precision too.  Others take the double-precision search.
      float af = atan2f(d2f_trunc(x.y), d2f_trunc(x.z));
      if (af < 0.0f) af += 6.28318531f;
      const double a = f2d(af);
      const unsigned k = bsearch_d(a, smin, ns);
      if (k > 0 && lt_pos(MX_LDG(smin + k - 1) + 1e-5, a) && lt_pos(a + 1e-5, MX_LDG(smin + ns + k - 1)) &&
          (k == ns || lt_pos(a + 1e-5, MX_LDG(smin + k))))
        sn = k - 1;
    }
#endif
    if (sn == ns) {
      double sector = atan2(x.y, x.z);
      if (sector < 0) sector = 2 * PI + sector;
      sn = bsearch_d(sector, smin, ns);
      if (sn == 0) return -1;
      sn -= 1;
      if ((MX_LDG(smin + g.nsec + sn) <= sector) || (MX_LDG(smin + sn) > sector)) return -1;
    }
    dtheta = MX_LDG(smin + 2 * g.nsec + sn) + MX_LDG(smin + 3 * g.nsec + sn) * rng.normal();
    dpp = MX_LDG(smin + 4 * g.nsec + sn) + MX_LDG(smin + 5 * g.nsec + sn) * rng.normal();
  } else {
    dtheta = g.theta_blur * rng.normal();
    dpp = g.dp_over_p * rng.normal();
  }
  double theta = 0.0 - dtheta;
  // the facet basis turned by theta, l' = c l + s d and d' = c d - s l,
  // enters through its components only: p.l', p.d' from p.l, p.d, and the
  // new direction p_d d' + p_n n + p_l l' (and the dP/P term -f d') as
  // coefficients of l, d and n
  double sn = 0.0, cs = 1.0;
  if (!is_zero(theta)) sincos_small(theta, &sn, &cs);
  const double pl0 = dot(P, l), pd0 = dot(P, d);
  const double p_l = fma(cs, pl0, MX_DMUL(sn, pd0)), p_d = nlod + fma(cs, pd0, -MX_DMUL(sn, pl0));
  const double pn2 = fma(-p_d, p_d, fma(-p_l, p_l, 1.0));
  if (neg_bit(pn2) && !is_zero(pn2)) return -1;
  double p_n, inv_pn;
  sqrt_rsqrt(pn2, p_n, inv_pn);
  double cl = fma(p_l, cs, -MX_DMUL(p_d, sn)), cd = fma(p_l, sn, MX_DMUL(p_d, cs)), cn = p_n;
  if (is_zero(dpp)) {
    P = comb3(cl, l, cd, d, cn, n);
    return 0;
  }
  const double f = MX_DMUL(nlod, dpp);
  cl = fma(f, sn, cl); cd = fma(-f, cs, cd); cn = fma(f, MX_DMUL(p_d, inv_pn), cn);
  P = normalized(comb3(cl, l, cd, d, cn, n));
  return 0;
}

// Cumulative order efficiencies at energy fe (JDMinterpolate_n_fvector,
// finterpo.c:134-190: first bracket index >= 1 with E <= energies[idx],
// capped at n-1; each order's value rounded to float) and the order choice
// of diffract_photon_from_grating (diffract.c:828-849): the first index
// whose cumulative efficiency reaches r, or -1.  cum is [energy][order].
// Whether the cumulative efficiency of order index k, interpolated at w
// into the energy bin of width dx (rdx = 1/dx) and rounded to float,
// reaches r (r <= c; r and c are not negative).
MXD bool order_reaches(const float *c0, int norders, int k, bool flat, double w, double dx, double rdx, double r) {
  float c;
  if (flat) c = MX_LDG(c0 + k);
  else {
    const double y0 = f2d(MX_LDG(c0 + k)), y1 = f2d(MX_LDG(c0 + norders + k));
    c = d2f_rn(MX_DADD(y0, div_by(MX_DMUL(MX_DADD(y1, -y0), w), dx, rdx)));
  }
  return !lt_pos(f2d(c), r);
}
MXD int choose_order(const float *ge, unsigned n, const float *cum, int norders, bool monotone, float fe, double r) {
  unsigned lo = 1, hi = n - 1;
  while (lo < hi) {
    unsigned mid = (lo + hi) >> 1;
    if (fe > MX_LDG(ge + mid)) lo = mid + 1; else hi = mid;   // floats compare as their doubles do
  }
  unsigned idx = lo;
  double x0 = f2d(MX_LDG(ge + idx - 1)), x1 = f2d(MX_LDG(ge + idx)), dx = MX_DADD(x1, -x0);
  double w = MX_DADD(f2d(fe), -x0);
  const float *c0 = cum + (size_t) (idx - 1) * norders;
  const bool flat = is_zero(dx);
  // the quotient by dx from one correctly rounded reciprocal: a Markstein
  // division (div_by) rounds as the division does
  const double rdx = flat ? 0.0 : MX_DDIV(1.0, dx);
  if (monotone && (flat || (!neg_bit(w) && dkey(w) <= dkey(dx)))) {
    // Between two rows that are non-decreasing in the order index the
    // interpolated row is too (rounding to float keeps the order), so the
    // first index reaching r is found by bisection over the same values.
    int a = 0, b = norders;
    while (a < b) {
      int m = (a + b) >> 1;
      if (order_reaches(c0, norders, m, flat, w, dx, rdx, r)) b = m; else a = m + 1;
    }
    return a < norders ? a : -1;
  }
  for (int k = 0; k < norders; k++)
    if (order_reaches(c0, norders, k, flat, w, dx, rdx, r)) return k;
  return -1;
}

// diffract_photon for an LETG support grating (diffract_from_support_grating,
// diffract.c:917-970): no facet sectors, no alignment blur and no dP/P
// (both zero for the support gratings, though their normals are still
// drawn), the facet basis rotated about n by the support's fixed angle.
MXD int diffract_support(const MxTables &T, const MxSupportDev &g, int order_idx, double energy, D3 x, D3 &P,
                         Rng &rng) {
  double nlod = MX_LDG(T.support_k + g.order_off + order_idx) * rcp_fast(energy);
  const double xx = dot(x, x);
  const D3 n = is_zero(xx) ? -1.0 * x : (-mx_rsqrt(xx)) * x;   // -x / |x|
  D3 l = normalized(mk(n.z, 0.0, -n.x));
  D3 d = cross(n, l);
  rng.skip_normal();   // dtheta = 0 x N
  rng.skip_normal();   // dP/P = 0 x N
  // the basis turned by the support's angle enters through its components,
  // as in diffract_photon
  const double cs = g.rotate ? g.cos_t : 1.0, sn = g.rotate ? g.sin_t : 0.0;
  const double pl0 = dot(P, l), pd0 = dot(P, d);
  const double p_l = fma(cs, pl0, MX_DMUL(sn, pd0)), p_d = nlod + fma(cs, pd0, -MX_DMUL(sn, pl0));
  const double pn2 = fma(-p_d, p_d, fma(-p_l, p_l, 1.0));
  if (neg_bit(pn2) && !is_zero(pn2)) return -1;
  const double p_n = sqrt_fast(pn2);
  P = comb3(fma(p_l, cs, -MX_DMUL(p_d, sn)), l, fma(p_l, sn, MX_DMUL(p_d, cs)), d, p_n, n);
  return 0;
}

// diffract (diffract.c:974-1130) for one photon, in two parts: vignetting,
// rotation into the grating frame, Rowland torus, the primary grating's
// order; then its diffraction, for the LETG the four support gratings, and
// the rotation back.
// grating_front: the grating's vignetting, the Rowland torus and the order
// choice.  Returns the chosen order index, with the photon at the torus in
// the grating's frame in x, p, or -1 when the photon's grating stage ends
// here (vignetted: ph unchanged; no order chosen: ph.x, ph.p rotated back
// from the torus).  Most photons that reach the gratings end here (no
// order), so the wavefront diffracts the others in a phase of their own.
MXD int grating_front(const MxTables &T, const MxGratingDev *grs, int kind, Ph &ph, Rng &rng, D3 &x, D3 &p) {
  const bool letg = kind == MX_GRATING_LETG;
  if (letg) rng.window(MX_U_LETG, 6, MX_N_LETG, 10);
  else rng.window(MX_U_GRATING, 2, MX_N_GRATING, 2);
  const MxGratingDev &g = grs[(letg ? 4 : 0) + ph.shell];
  if (lt_pos(g.vig, rng.uniform())) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;
  if (ph.flags & MX_BAD_PHOTON_MASK) return -1;
  x = rot_x(ph.x, g.cos_m, g.sin_m);
  p = rot_x(ph.p, g.cos_m, g.sin_m);
  if (-1 == rowland_intersect(x, p, g.rowland)) ph.flags |= MX_PHOTON_UNDIFFRACTED;
  const int chosen = choose_order(T.geff_energy + g.geff_off, (unsigned) g.nenergy, T.geff_cum + g.cum_off, g.norders,
                                  g.monotone != 0, d2f_rn(ph.e), rng.uniform());
  if (chosen < 0) {
    // no order: the LETG's supports are skipped (the photon is flagged)
    ph.flags |= MX_PHOTON_UNDIFFRACTED;
    ph.x = rot_x(x, g.cos_p, g.sin_p);
    ph.p = rot_x(p, g.cos_p, g.sin_p);
    return -1;
  }
  ph.order = chosen - g.max_order;
  return chosen;
}
// grating_back: the diffraction into the chosen order, for the LETG its
// four support gratings (fine, then coarse at 60, 120 and 0 degrees), and
// the rotation back; the rng window is grating_front's.
MXD void grating_back(const MxTables &T, const MxGratingDev *grs, int kind, Ph &ph, Rng &rng, D3 x, D3 p, int chosen) {
  const bool letg = kind == MX_GRATING_LETG;
  const MxGratingDev &g = grs[(letg ? 4 : 0) + ph.shell];
  if (-1 == diffract_photon(T, g, chosen, ph.e, x, p, rng)) ph.flags |= MX_PHOTON_UNDIFFRACTED;
  if (letg) {
    const float fe = d2f_rn(ph.e);
    for (int s = 0; s < 4; s++) {
      const MxSupportDev &sg = T.supports[s];
      if (!sg.norders) continue;
      if (ph.flags & MX_BAD_PHOTON_MASK) continue;
      int k = choose_order(T.support_energy, (unsigned) T.support_nenergy, T.support_cum + sg.cum_off, sg.norders,
                           sg.monotone != 0, fe, rng.uniform());
      if (k < 0) { ph.flags |= MX_PHOTON_UNDIFFRACTED; continue; }
      // order list 0, +1, -1, +2, -2, ... (init_one_grating, diffract.c:392-405)
      ph.sup[s] = (int8_t) ((k & 1) ? (k + 1) / 2 : -(k / 2));
      ph.set |= MX_SET_SUPPORT;
      if (-1 == diffract_support(T, sg, k, ph.e, x, p, rng)) ph.flags |= MX_PHOTON_UNDIFFRACTED;
    }
  }
  ph.x = rot_x(x, g.cos_p, g.sin_p);
  ph.p = rot_x(p, g.cos_p, g.sin_p);
}
// diffract (diffract.c:974-1130) for one photon, both parts.
MXD void grating_stage(const MxTables &T, const MxGratingDev *grs, int kind, Ph &ph, Rng &rng) {
  D3 x, p;
  const int chosen = grating_front(T, grs, kind, ph, rng, x, p);
  if (chosen >= 0) grating_back(T, grs, kind, ph, rng, x, p, chosen);
}

// ----------------------------------------------------------- detector --
// intersect_with_detector_plane (detector.c:56-109).
MXD int chip_plane(const MxChipDev &g, D3 x0, D3 p, D3 &x, double &dx, double &dy, bool must_hit) {
  D3 nrm = mk(g.normal[0], g.normal[1], g.normal[2]), ll = mk(g.x_ll[0], g.x_ll[1], g.x_ll[2]);
  double pdn = dot(p, nrm);
  if (is_zero(pdn)) return -1;
  D3 r = x0 - ll;
  r = r + (-dot(r, nrm) * rcp_fast(pdn)) * p;
  int hit = 1;
  double rx = r.x * g.xhat[0] + r.y * g.xhat[1] + r.z * g.xhat[2];
  if ((dkey(rx) < 0) || (dkey(rx) >= dkey(g.xlen))) { if (must_hit) return 0; hit = 0; }
  double ry = r.x * g.yhat[0] + r.y * g.yhat[1] + r.z * g.yhat[2];
  if ((dkey(ry) < 0) || (dkey(ry) >= dkey(g.ylen))) { if (must_hit) return 0; hit = 0; }
  x = r + ll; dx = rx; dy = ry;
  return hit;
}

// Single-precision screen of chip_plane's must-hit test: 0 when the ray
// certainly misses the chip (its chip coordinates lie more than
// MX_CHIP_MARGIN outside an edge), 1 otherwise.  The float coordinates
// carry an absolute error below 1e-2 mm for positions of up to 1e4 mm from
// the chip, far inside the margin; a ray that is not certainly outside
// takes the double-precision test, which alone decides a hit.
#define MX_CHIP_MARGIN 0.1f
MXD int chip_screen(const MxChipDev &g, float x0, float x1, float x2, float p0, float p1, float p2) {
  const float r0 = x0 - g.f_ll[0], r1 = x1 - g.f_ll[1], r2 = x2 - g.f_ll[2];
  const float pdn = p0 * g.f_normal[0] + p1 * g.f_normal[1] + p2 * g.f_normal[2];
  const float s = -(r0 * g.f_normal[0] + r1 * g.f_normal[1] + r2 * g.f_normal[2]) / pdn;
  const float q0 = r0 + s * p0, q1 = r1 + s * p1, q2 = r2 + s * p2;
  const float rx = q0 * g.f_xhat[0] + q1 * g.f_xhat[1] + q2 * g.f_xhat[2];
  const float ry = q0 * g.f_yhat[0] + q1 * g.f_yhat[1] + q2 * g.f_yhat[2];
  if (rx < -MX_CHIP_MARGIN || rx > g.f_xlen + MX_CHIP_MARGIN || ry < -MX_CHIP_MARGIN ||
      ry > g.f_ylen + MX_CHIP_MARGIN)
    return 0;
  return 1;
}
// The first chip from k on that the screen does not rule out (nchips if
// none).  Stepping from one candidate to the next keeps a warp's lanes
// together: each runs the double-precision test once, on its own candidate
// chip, in the same iteration, instead of at the loop index where its chip
// happens to come.
MXD int next_chip(const MxChipDev *chips, int nchips, int k, float x0, float x1, float x2, float p0, float p1,
                  float p2) {
  for (; k < nchips; k++)
    if (chip_screen(chips[k], x0, x1, x2, p0, p1, p2)) break;
  return k;
}

// The detector frame of a photon: _marx_dither_detector then
// _marx_transform_ray (detector.c:244-284, trans.c:40-77).  DetOffset plus,
// with DitherModel FILE, the aspect solution's dy, dz at the photon's time,
// and a rotation by its dtheta about x (rotate_matrix of the identity: rows
// (1,0,0), (0,c,s), (0,-s,c)).  The reference moves one global matrix there
// and back per photon; here each photon has its own.
struct DetFrame { D3 off; double c, s; };
MXD DetFrame det_frame(const MxTables &T, double t) {
  DetFrame f;
  f.off = mk(T.det_offset[0], T.det_offset[1], T.det_offset[2]);
  f.c = 1.0; f.s = 0.0;
  float s[6];
  if (T.dither_file && aspsol_state(T, T.start_time + t, s)) {
    f.off.y = T.det_offset[1] + f2d(s[3]);
    f.off.z = T.det_offset[2] + f2d(s[4]);
    const double th = f2d(s[5]);
    if (th != 0.0) sincos_small(th, &f.s, &f.c);
  }
  return f;
}
// rotate_vector and rotate_vector_inv (trans.c:40-66) with that matrix;
// the x row is the identity's.
MXD D3 det_rotate(const DetFrame &f, D3 v) {
  return mk(v.x, MX_DADD(MX_DMUL(f.c, v.y), MX_DMUL(f.s, v.z)), MX_DADD(MX_DMUL(-f.s, v.y), MX_DMUL(f.c, v.z)));
}
MXD D3 det_rotate_inv(const DetFrame &f, D3 v) {
  return mk(v.x, MX_DADD(MX_DMUL(f.c, v.y), MX_DMUL(-f.s, v.z)), MX_DADD(MX_DMUL(f.s, v.y), MX_DMUL(f.c, v.z)));
}
// into the frame: x - offset, then rotated (T.dither_file only)
MXD void det_enter(const MxTables &T, const DetFrame &f, D3 &x, D3 &p) {
  x = x - f.off;
  if (T.dither_file) { x = det_rotate(f, x); p = det_rotate(f, p); }
}
MXD void det_leave(const MxTables &T, const DetFrame &f, D3 &x, D3 &p) {
  if (T.dither_file) { p = det_rotate_inv(f, p); x = det_rotate_inv(f, x); }
  x = x + f.off;
}

// _marx_acis_i_detect / _marx_acis_s_detect per photon (acis-i.c:124-157,
// acis-s.c:203-239), _marx_intersect_with_detector (detector.c:112-168),
// _marx_acis_apply_streak (acis-i.c:60-93).  QE and pulse height are not
// modelled (DetIdeal); the detector frame is the identity rotation plus the
// DetOffset translation (INTERNAL dither has no detector motion).
// _marx_acis_apply_streak (acis-i.c:60-100): a photon arriving during the
// frame transfer lands on a random row of its column.  x, p in the
// detector frame.
MXD void acis_streak(const MxTables &T, const MxChipDev &d, Ph &ph, D3 &x, D3 &p, Rng &rng) {
  if (!(dkey(T.frame_transfer) > 0)) return;
  double t = fmod_pos(T.start_time + ph.t, T.frame_time, T.inv_frame_time);
  if (t > T.exposure) {
    ph.zpix = (float) (1.0 + 1022.0 * rng.uniform());
    double xp = ((double) ph.ypix - d.xoff) * d.xpix, yp = ((double) ph.zpix - d.yoff) * d.ypix;
    x = mk(d.x_ll[0] + (xp * d.xhat[0] + yp * d.yhat[0]), d.x_ll[1] + (xp * d.xhat[1] + yp * d.yhat[1]),
           d.x_ll[2] + (xp * d.xhat[2] + yp * d.yhat[2]));
    p = normalized(x - mk(T.focal_length, 0, 0));
    ph.flags |= MX_PHOTON_ACIS_STREAKED;
  }
}

// ------------------------------------------------------- ACIS QE, FEF --
// compute_contamination (aciscontam.c:93-135) at chip pixel (cx, cy).
MXD double acis_contam(const MxTables &T, const MxContamDev &c, double en, double cx, double cy) {
  const float fe = (float) en;
  double fxy = 0.0, v = 0.0;
  if (c.mode != 2) {
    if (c.mode == 0) {   // fxy_acis_i (aciscontam.c:140-155)
      const double dx = cx - c.x0, dy = cy - c.y0;
      double r = (8.0 / 1024.0) * sqrt(dx * dx + dy * dy);
      r /= 8.07;
      fxy = 1.29 * r * r;
    } else {             // fxy_acis456789 (aciscontam.c:177-189)
      const double y0 = 512.0;
      fxy = cy <= 512.0 ? pow(fabs((cy - y0) / (64.0 - y0)), 5.5) : pow(fabs((cy - y0) / (964.0 - y0)), 4.5);
    }
    for (int i = 0; i < c.nl; i++) {
      const MxTabDev &t = c.mu[i];
      const double mu = f2d(interp_f(fe, T.fef_f + t.x_off, T.fef_f + t.y_off, T.fef_slope + t.s_off, (unsigned) t.n));
      v += mu * (c.tau0[i] + c.tau1[i] * fxy);
    }
  } else {
    if ((cx < 0) || (cx >= 1024) || (cy < 0) || (cy >= 1024)) return 0.0;
    cx /= c.blk;
    cy /= c.blk;
    const unsigned ofs = (1024u / (unsigned) c.blk) * (unsigned) cy + (unsigned) cx;
    for (int i = 0; i < c.nl; i++) {
      const MxTabDev &t = c.mu[i];
      const double mu = f2d(interp_f(fe, T.fef_f + t.x_off, T.fef_f + t.y_off, T.fef_slope + t.s_off, (unsigned) t.n));
      fxy = f2d(T.fef_f[c.fxy_off[i] + ofs]);
      v += mu * (c.tau0[i] + c.tau1[i] * fxy);
    }
  }
  return exp(-v);
}

// The acceptance of _marx_acis_apply_qe_and_pha (acis-s.c:145-163): the
// CALDB QE (no filter table: the CALDB build reads none) times the
// contamination against one uniform.
MXD bool acis_qe_accept(const MxTables &T, int ccd, const Ph &ph, Rng &rng) {
  const double r = rng.uniform();
  const MxContamDev &c = T.contam[ccd];
  const double qe = f2d(interp_f((float) ph.e, T.fef_f + c.qe.x_off, T.fef_f + c.qe.y_off, T.fef_slope + c.qe.s_off,
                                 (unsigned) c.qe.n));
  const double qe_filter = 1.0;
  const double qe_contam = acis_contam(T, c, ph.e, (double) ph.ypix, (double) ph.zpix);
  return !(r >= qe * qe_filter * qe_contam);
}

constexpr int MX_FEF_MAX_GAUSS = MX_FEF_GAUSSIANS;

// gaussian_integral (acis_fef.c:380-392) over [0, inf) and (-inf, 0]: the
// erf of the upper (lower) infinite bound is 1 (-1).
MXD void fef_areas(float amp, float center, float sigma, double &above, double &below) {
  const double s = (double) sigma * 1.4142135623730951;
  if (s == 0.0) { above = below = 0.0; return; }
  const double e0 = erf((0 - (double) center) / s), w = 2.5066282746310002 * (double) sigma;
  above = 0.5 * amp * (1.0 - e0) * w;
  below = 0.5 * amp * (e0 - -1.0) * w;
}

// marx_apply_acis_rmf (acis_fef.c:910-1079) for a photon at chip pixel
// (x, y): the region's gaussians interpolated in energy and normalised
// (normalize_gaussians, :509-579), a pulse height drawn from them
// (compute_pha_with_pos_amps, :407-469; compute_pha_with_neg_amps,
// :471-507), and its PI energy.  False where the reference returns -1.
// Draws come from the FEF window; the reference's unbounded loops stop at
// its end (the photon is then flagged as a variate overrun).
MXD bool acis_fef(const MxTables &T, int ccd, float x, float y, double energy, Rng &rng, int16_t &pha_out,
                  float &pi_out) {
  // find_fef
  if (x < 0) { if (!T.det_extend) return false; x = 0; }
  else if (x >= 1024.0f) { if (!T.det_extend) return false; x = 1023.0f; }
  if (y < 0) { if (!T.det_extend) return false; y = 0; }
  else if (y >= 1024.0f) { if (!T.det_extend) return false; y = 1023.0f; }
  const unsigned ci = (unsigned) (x / 32.0f), cj = (unsigned) (y / 32.0f);
  if (ci >= 32 || cj >= 32 || ccd < 0 || ccd >= 10) return false;
  const int idx = T.fef_map[((unsigned) ccd * 32 + ci) * 32 + cj];
  if (idx < 0) return false;
  const MxFefDev f = T.fef[idx];
  const float *E = T.fef_f + f.e_off, *CH = E + f.n_e, *G = T.fef_f + f.g_off;
  const unsigned n = (unsigned) f.n_e;
  const int ng = f.n_g;
  unsigned k = bsearch_f((float) energy, E, n);
  if (k == 0) k++;
  if (k == n) k--;
  const double t = (energy - (double) E[k - 1]) / (double) (E[k] - E[k - 1]);
  const float *g0 = G + 3 * (size_t) (k - 1) * ng, *g1 = g0 + 3 * ng;
  float amp[MX_FEF_MAX_GAUSS], cen[MX_FEF_MAX_GAUSS], sig[MX_FEF_MAX_GAUSS], cum[MX_FEF_MAX_GAUSS];
  bool tail[MX_FEF_MAX_GAUSS];
  double pos = 0.0, neg = 0.0;
#pragma unroll
  for (int g = 0; g < MX_FEF_MAX_GAUSS; g++) {
    amp[g] = cen[g] = sig[g] = cum[g] = 0.0f;
    tail[g] = false;
    if (g >= ng) continue;
    const float a0 = g0[3 * g], c0 = g0[3 * g + 1], s0 = g0[3 * g + 2];
    const float a1 = g1[3 * g], c1 = g1[3 * g + 1], s1 = g1[3 * g + 2];
    cen[g] = (float) ((double) c0 + t * (double) (c1 - c0));
    double v = (double) s0 + t * (double) (s1 - s0);
    if (v > 0.0) {
      sig[g] = (float) v;
      v = (double) a0 + t * (double) (a1 - a0);
      if ((v < 0.0) && ((a1 > 0.0f) || (a0 > 0.0f))) v = 0.0;
      amp[g] = (float) v;
    }
    double above, below;
    fef_areas(amp[g], cen[g], sig[g], above, below);
    if (below > above) tail[g] = above / below < 0.1;
    if (above >= 0) pos += above;
    else neg -= above;
    cum[g] = (float) pos;
  }
  if (pos <= neg) return false;               // HAS_TOTAL_NEG_AREA
  if (pos > 0) {
#pragma unroll
    for (int g = 0; g < MX_FEF_MAX_GAUSS; g++) cum[g] = (float) ((double) cum[g] / pos);
  }
  double pha = -1.0;
  for (int tries = 0; tries < 100; tries++) {   // compute_pha_with_neg_amps (one pass when no amplitude is negative)
    // compute_pha_with_pos_amps
    for (;;) {
      const double r = rng.uniform();
      if (rng.overrun) return false;
      pha = -1.0;
      bool drawn = false;
#pragma unroll
      for (int g = 0; g < MX_FEF_MAX_GAUSS; g++) {
        if (drawn || g >= ng || (double) cum[g] <= r) continue;
        drawn = true;
        if (!tail[g]) {
          int count = 0;
          do {
            pha = (double) cen[g] + (double) sig[g] * rng.normal();
            count++;
          } while ((pha < 0) && (count < 100) && !rng.overrun);
        } else {
          const double s = (double) ((0.0f - cen[g]) / sig[g]);
          double u, xx;
          do {
            u = rng.uniform();
            double vv;
            do { vv = rng.uniform(); } while (vv == 0.0 && !rng.overrun);
            xx = sqrt(s * s - 2 * log(vv));
          } while ((xx * u > s) && !rng.overrun);
          pha = (double) cen[g] + xx * (double) sig[g];
        }
      }
      if (rng.overrun) return false;
      if (drawn && !(pha < 0)) break;           // else: a new choice of gaussian
    }
    if (neg == 0.0) break;
    double psum = 0.0, sum = 0.0;
#pragma unroll
    for (int g = 0; g < MX_FEF_MAX_GAUSS; g++) {
      if (g >= ng || sig[g] == 0.0f) continue;   // evaluate_gaussian
      const double xx = (pha - (double) cen[g]) / (double) sig[g];
      const double d = amp[g] * exp(-0.5 * xx * xx);
      sum += d;
      if (d > 0) psum += d;
    }
    const double u = rng.uniform();
    if (rng.overrun) return false;
    if (u * psum < sum) break;
    if (tries == 99) return false;
  }
  const int16_t ipha = (int16_t) pha;
  const double ph2 = (double) ipha - rng.uniform();
  if (rng.overrun) return false;
  const float pi = interp_f((float) ph2, CH, E, T.fef_slope + f.s_off, n);
  if (pi < 0) return false;
  pha_out = ipha;
  pi_out = pi;
  return true;
}

MXD void detect_stage(const MxTables &T, const MxChipDev *chips, int nchips, Ph &ph, Rng &rng) {
  rng.window(MX_U_DETECT, 2, MX_N_DETECT, 2);
  const DetFrame fr = det_frame(T, ph.t);
  D3 x = ph.x, p = ph.p;
  det_enter(T, fr, x, p);
  int hit = -1;
  D3 xh = x;
  double dx = 0, dy = 0;
#ifdef __CUDA_ARCH__
  const float fx0 = d2f_trunc(x.x), fx1 = d2f_trunc(x.y), fx2 = d2f_trunc(x.z);
  const float fp0 = d2f_trunc(p.x), fp1 = d2f_trunc(p.y), fp2 = d2f_trunc(p.z);
  for (int k = next_chip(chips, nchips, 0, fx0, fx1, fx2, fp0, fp1, fp2); k < nchips;
       k = next_chip(chips, nchips, k + 1, fx0, fx1, fx2, fp0, fp1, fp2))
    if (1 == chip_plane(chips[k], x, p, xh, dx, dy, true)) { hit = k; break; }
#else
  for (int k = 0; k < nchips; k++)
    if (1 == chip_plane(chips[k], x, p, xh, dx, dy, true)) { hit = k; break; }
#endif
  if (hit < 0 && T.det_extend) {
    double best = -1;
    for (int k = 0; k < nchips; k++) {
      D3 xx; double ddx, ddy;
      if (-1 == chip_plane(chips[k], x, p, xx, ddx, ddy, false)) continue;
      double ex = ddx - 0.5 * chips[k].xlen, ey = ddy - 0.5 * chips[k].ylen, r2 = ex * ex + ey * ey;
      if (r2 < best || hit < 0) { hit = k; xh = xx; dx = ddx; dy = ddy; best = r2; }
    }
  }
  if (hit < 0) {
    ph.flags |= MX_PHOTON_MISSED_DETECTOR;
    ph.ccd = -1;
  } else {
    const MxChipDev &d = chips[hit];
    x = xh;
    ph.ccd = d.id;
    ph.ypix = d2f_rn(div_by(dx, d.xpix, d.inv_xpix));
    ph.zpix = d2f_rn(div_by(dy, d.ypix, d.inv_ypix));
    // with an FEF or the QE acceptance the response and the streak are a
    // pass of their own over the photons on a chip (mx_acis_fef_kernel)
    if (!T.acis_fef && !T.acis_qe) acis_streak(T, d, ph, x, p, rng);
  }
  det_leave(T, fr, x, p);
  ph.x = x;
  ph.p = p;
}

// ---------------------------------------------------------------- HRC --
MXD float hrc_interp(const MxTables &T, const MxTabDev &t, float x) {   // JDMinterpolate_f
  return interp_f(x, T.hrc_tab + t.x_off, T.hrc_tab + t.y_off, T.hrc_slope + t.s_off, (unsigned) t.n);
}

// _marx_hrc_compute_pha (hrc-i.c:71-91): delta E / E = 1 (FWHM).
MXD int16_t hrc_pha(double energy, Rng &rng) {
  if (energy <= 0.5) energy = 141.582 * sqrt(energy);
  else if (energy < 2.0) energy = 107.299 * pow(energy, 0.1);
  else energy = 115.0;
  energy = energy * (1.0 + 0.424661 * rng.normal());
  if (energy < 0.0) energy = 0.0;
  return (int16_t) energy;
}

// get_filter_region (hrc-s.c:119-185): UV/ion shield region 0..3 at (y, z)
// in the MARX frame, or -1 in a gap.
MXD int hrc_filter_region(const MxHrcDev &h, double y, double z) {
  y -= h.shield_yc;
  z -= h.shield_zc;
  if (y < 0) {
    y = -y;
    if (y < h.shield_l) return 0;
    if (y < h.shield_sl) return z >= h.shield_t ? 0 : 1;
    if (y >= h.shield_sl_gap) return z >= h.shield_t ? 2 : 3;
    return -1;
  }
  if (y < h.shield_r) return 0;
  if (y < h.shield_sr) return z >= h.shield_t ? 0 : 1;
  if (y >= h.shield_sr_gap) return z >= h.shield_t ? 2 : 3;
  return -1;
}

// rand_gauss2d_radius (hrcblur.c:233-245): a draw of exactly 0 is redrawn.
MXD double gauss2d_radius(double sigma, Rng &rng) {
  double c;
  int guard = 0;
  do { c = rng.uniform(); } while (c == 0.0 && !rng.overrun && ++guard < 8);
  return sigma * sqrt(-2 * log(c));
}

// _marx_hrc_blur_position (hrcblur.c:258-298).
MXD void hrc_blur(const MxHrcDev &h, bool extend, double &dx, double &dy, Rng &rng) {
  double r = rng.uniform(), x0, y0;
  if (r < h.g1_w) { r = gauss2d_radius(h.g1_sigma, rng); x0 = 0.0; y0 = 0.0; }
  else if (r < h.g1_w + h.g2_w) { r = gauss2d_radius(h.g2_sigma, rng); x0 = h.g2_x; y0 = h.g2_y; }
  else {
    double c = rng.uniform(), rmax = h.l1_rmax / h.l1_hwhm;
    r = h.l1_hwhm * sqrt(expm1(c * log1p(rmax * rmax)));
    x0 = h.l1_x; y0 = h.l1_y;
  }
  double theta = (2.0 * PI) * rng.uniform();
  dx += x0 + r * cos(theta);
  dy += y0 + r * sin(theta);
  if (!extend) {
    if (dx < 0.0) dx = 0.0;
    if (dy < 0.0) dy = 0.0;
  }
}

// drake_intersection + the reflection of _marx_drake_reflect (drake.c:250-351)
// for one photon, in the MARX frame.
MXD void drake_reflect(const MxTables &T, const MxHrcDev &h, Ph &ph, Rng &rng) {
  const D3 x0 = ph.x, p = ph.p;
  for (int i = 0; i < h.drake_n; i++) {
    const MxPlateDev &r = h.plates[i];
    const D3 nrm = mk(r.normal[0], r.normal[1], r.normal[2]), a = mk(r.a[0], r.a[1], r.a[2]);
    double pdn = dot(p, nrm);
    if (pdn == 0.0) continue;
    double t = dot(a - x0, nrm) / pdn;
    D3 nx = x0 + t * p;
    D3 xp = nx - a;
    double xx = dot(xp, mk(r.e1[0], r.e1[1], r.e1[2]));
    if ((xx < 0.0) || (xx >= r.len1)) continue;
    double yy = dot(xp, mk(r.e2[0], r.e2[1], r.e2[2]));
    if ((yy < 0.0) || (yy >= r.len2)) continue;
    const bool cr = xx < h.drake_cr_width;
    ph.x = nx;
    float fe = d2f_rn(ph.e);
    float beta = hrc_interp(T, cr ? h.cr_beta : h.c_beta, fe), delta = hrc_interp(T, cr ? h.cr_delta : h.c_delta, fe);
    const double u = rng.uniform();
    int blocked = -1;   // -1: left to the double-precision test
#ifdef __CUDA_ARCH__
    {
      // the double-float reflectivity decides unless u den and num lie
      // within 2^-24 of each other, as in reflect_test
      F2 fn, fd;
      reflectivity_df(fabs(pdn), beta, delta, fn, fd);
      const double y = df_to(fn), gap = y - u * df_to(fd), ag = fabs(gap);
      if (lt_pos(0x1p-100, y) && lt_pos(0x1p-24 * y, ag) && lt_pos(ag, 0x1p+100)) blocked = neg_bit(gap) ? 1 : 0;
    }
#endif
    if (blocked < 0) blocked = reflectivity(fabs(pdn), f2d(beta), f2d(delta)) < u ? 1 : 0;
    if (blocked) { ph.flags |= MX_PHOTON_DRAKE_BLOCKED; return; }
    ph.p = p + (-2.0 * pdn) * nrm;
    ph.flags |= MX_PHOTON_DRAKE_REFLECTED;
    return;
  }
}

// _marx_hrc_i_detect / _marx_hrc_s_detect per photon (hrc-i.c:116-176,
// hrc-s.c:254-319) with apply_hrc_qe (hrc-i.c:93-114, hrc-s.c:188-230).
MXD void hrc_detect_stage(const MxTables &T, const MxChipDev *chips, int nchips, Ph &ph, Rng &rng) {
  const MxHrcDev &h = T.hrc;
  rng.window(MX_U_HRC, 6, MX_N_HRC, 2);
  const bool hrcs = h.kind == MX_DETECTOR_HRC_S;
  if (hrcs && h.drake_n) {
    drake_reflect(T, h, ph, rng);
    if (ph.flags & MX_BAD_PHOTON_MASK) return;
  }
  const DetFrame fr = det_frame(T, ph.t);
  D3 x = ph.x, p = ph.p;
  det_enter(T, fr, x, p);
  int hit = -1;
  D3 xh = x;
  double dx = 0, dy = 0;
#ifdef __CUDA_ARCH__
  {
    const float fx0 = d2f_trunc(x.x), fx1 = d2f_trunc(x.y), fx2 = d2f_trunc(x.z);
    const float fp0 = d2f_trunc(p.x), fp1 = d2f_trunc(p.y), fp2 = d2f_trunc(p.z);
    for (int k = next_chip(chips, nchips, 0, fx0, fx1, fx2, fp0, fp1, fp2); k < nchips;
         k = next_chip(chips, nchips, k + 1, fx0, fx1, fx2, fp0, fp1, fp2))
      if (1 == chip_plane(chips[k], x, p, xh, dx, dy, true)) { hit = k; break; }
  }
#else
  for (int k = 0; k < nchips; k++)
    if (1 == chip_plane(chips[k], x, p, xh, dx, dy, true)) { hit = k; break; }
#endif
  if (hit < 0 && T.det_extend) {
    double best = -1;
    for (int k = 0; k < nchips; k++) {
      D3 xx; double ddx, ddy;
      if (-1 == chip_plane(chips[k], x, p, xx, ddx, ddy, false)) continue;
      double ex = ddx - 0.5 * chips[k].xlen, ey = ddy - 0.5 * chips[k].ylen, r2 = ex * ex + ey * ey;
      if (r2 < best || hit < 0) { hit = k; xh = xx; dx = ddx; dy = ddy; best = r2; }
    }
  }
  if (hit < 0) {
    ph.flags |= MX_PHOTON_MISSED_DETECTOR;
    ph.ccd = -1;
    det_leave(T, fr, x, p);
    ph.x = x; ph.p = p;
    return;
  }
  x = xh;
  const MxChipDev &d = chips[hit];
  const float fe = d2f_rn(ph.e);
  bool ok = true;
  const int m = hrcs ? d.id - 1 : 0;                     // facet index 0..2
  const MxTabDev &mcp = h.mcp[hrcs ? 2 - m : 0];         // HRC-S MCP ids 1, 2, 3 use QE files 2, 1, 0
  if (mcp.n && rng.uniform() >= (double) hrc_interp(T, mcp, fe)) ok = false;
  int region = 0;
  if (ok && hrcs) {
    double t = (h.shield_x - x.x) / p.x;
    region = hrc_filter_region(h, x.y + t * p.y, x.z + t * p.z);
    if (region < 0) ok = false;
  }
  if (ok) {
    const MxTabDev &f = h.filt[region];
    if (f.n && rng.uniform() >= (double) hrc_interp(T, f, fe)) ok = false;
  }
  if (!ok) {
    ph.flags |= MX_PHOTON_UNDETECTED;
    ph.ccd = -1;
  } else {
    if (hrcs) { ph.region = (uint8_t) region; ph.set |= MX_SET_REGION; }
    ph.pha = hrc_pha(ph.e, rng);
    ph.set |= MX_SET_HRC;
    if (h.blur && !T.det_ideal) hrc_blur(h, T.det_extend != 0, dx, dy, rng);
    ph.ccd = d.id;
    if (hrcs) {   // _marx_hrc_s_compute_pixel (hrc_s_geom.c:289-340)
      double u = h.u_active0 + div_by(dx, h.pix[0], h.inv_pix[0]);
      double v = h.v_active0[m] + div_by(dy, h.pix[1], h.inv_pix[1]);
      ph.upix = (float) u; ph.vpix = (float) v;
      ph.set |= MX_SET_UV;
      ph.ypix = (float) (h.cxcy0[m][0] + (u - h.uv0[m][0]));
      ph.zpix = (float) (h.cxcy0[m][1] + (v - h.uv0[m][1]));
    } else {      // _marx_hrc_i_compute_pixel (hrc_i_geom.c:134-143)
      ph.ypix = (float) (h.ll_cxcy[0] + div_by(dx, h.pix[0], h.inv_pix[0]));
      ph.zpix = (float) (h.ll_cxcy[1] + div_by(dy, h.pix[1], h.inv_pix[1]));
    }
  }
  det_leave(T, fr, x, p);
  ph.x = x;
  ph.p = p;
}

MXD void any_detect_stage(const MxTables &T, const MxChipDev *chips, int nchips, Ph &ph, Rng &rng) {
  if (T.det_kind == MX_DETECTOR_HRC_I || T.det_kind == MX_DETECTOR_HRC_S) hrc_detect_stage(T, chips, nchips, ph, rng);
  else detect_stage(T, chips, nchips, ph, rng);
}

// The fused per-photon trace: dither at creation (source.c:357), then the
// stages of process_photons (marx.c:240-273); a photon with a bad flag is
// skipped by later stages as marx_prune_photons drops it, and a photon
// whose stage ran out of pre-drawn variates is not traced further.
MXD void trace_photon(const MxTables &T, const MxShellDev *shells, const float *optc, const double *slope,
                      const MxGratingDev *grs, const MxChipDev *chips, uint32_t stages, Ph &ph, Rng &rng) {
  if ((stages & MX_STAGE_DITHER) && T.dither) dither_stage(T, ph, rng);
  if ((stages & MX_STAGE_MIRROR) && !(ph.flags & MX_BAD_PHOTON_MASK)) mirror_stage(T, shells, optc, slope, ph, rng);
  if (rng.overrun) return;
  if ((stages & MX_STAGE_GRATING) && T.grating && !(ph.flags & MX_BAD_PHOTON_MASK))
    grating_stage(T, grs, T.grating, ph, rng);
  if (rng.overrun) return;
  if ((stages & MX_STAGE_DETECT) && T.nchips && !(ph.flags & MX_BAD_PHOTON_MASK))
    any_detect_stage(T, chips + T.chip_off, T.nchips, ph, rng);
}

}  // namespace mx
