// Float-float arithmetic and elementary functions for the GCMC path.
//
// On GB300 a warp issues one FP64 instruction per ~64 clocks however many
// of its lanes are active (an FP64 exp costs ~1100 clocks of one warp), so
// the short serial chains of GRAND -- one pair law, one map interpolation,
// one acceptance -- take microseconds in FP64.  Here a value is carried as
// the unevaluated sum h + l of two floats with |l| <= ulp(h)/2 (about 48
// significant bits, relative error ~2^-47 per operation) and every step runs
// on the FP32 pipe.  Exponent range is float's, and values below 2^-102
// lose low bits (their low part is a float subnormal): callers keep
// arguments in range (or fall back to FP64 for the rare pair that is not).
//
// Methods (all published, none taken from a vendor library):
//   - two_sum, fast_two_sum (Knuth, TAOCP vol. 2, 4.2.2; Dekker 1971) and
//     two_prod by fused multiply-add, composed into addition, product,
//     division and square root as in Hida, Li and Bailey's double-double
//     library ("accurate" addition; quotient by three reciprocal-scaled
//     corrections; square root by Karp and Markstein's single correction of
//     a float estimate refined by one float Newton step; reciprocal square
//     root by one Newton correction of the same estimate).
//   - exp: x = k ln2 + r, |r| <= ln2/2, with ln 2 split over three floats so
//     that k times the two leading parts is exact (Cody and Waite), exp(r) by
//     its Taylor series to degree 13 (remainder < 2^-57) evaluated by
//     Estrin's scheme (four dependent levels), then scaled by 2^k.
//   - cos: x = k pi/2 + r, |r| <= pi/4, with pi/2 split the same way, then
//     +-cos r or +-sin r by quadrant, by their Taylor series to r^18 and r^19
//     (remainders < 2^-63).
// The constants are the float splits of ln 2, pi/2, 2/pi, log2 e and 1/n!,
// rounded from 80-digit decimal values (Machin's formula for pi): a leading
// part of 16 significant bits, the next 16 bits, the rest rounded to float
// (reduction constants); nearest float and nearest float of the remainder
// (the others).
#pragma once
#include "ff.cuh"

namespace bgpu {

struct f2 {
  float h, l;
};

__device__ __forceinline__ f2 f2_f(float h) { return {h, 0.0f}; }
__device__ __forceinline__ f2 f2_neg(f2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ double f2_dbl(f2 a) { return (double)a.h + (double)a.l; }
// nearest float-float of a double (exact when x has at most 48 significant
// bits spread over the float range)
__device__ __forceinline__ f2 f2_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

// p + e == a * b exactly
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  float s, e, t, f;
  two_sum(a.h, b.h, s, e);
  two_sum(a.l, b.l, t, f);
  e = __fadd_rn(e, t);
  fast_two_sum(s, e, s, e);
  e = __fadd_rn(e, f);
  fast_two_sum(s, e, s, e);
  return {s, e};
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) { return f2_add(a, f2_neg(b)); }

__device__ __forceinline__ f2 f2_addf(f2 a, float b) {
  float s, e;
  two_sum(a.h, b, s, e);
  e = __fadd_rn(e, a.l);
  fast_two_sum(s, e, s, e);
  return {s, e};
}

__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  float p, e;
  two_prod(a.h, b.h, p, e);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}

__device__ __forceinline__ f2 f2_mulf(f2 a, float b) {
  float p, e;
  two_prod(a.h, b, p, e);
  e = __fmaf_rn(a.l, b, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}

__device__ __forceinline__ f2 f2_sqr(f2 a) {
  float p, e;
  two_prod(a.h, a.h, p, e);
  e = __fmaf_rn(__fmul_rn(2.0f, a.h), a.l, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}

// a * b + c
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) { return f2_add(f2_mul(a, b), c); }

// a / b: three quotient digits, each the remainder times 1/b.h
__device__ __forceinline__ f2 f2_div(f2 a, f2 b) {
  const float rb = __frcp_rn(b.h);
  const float q1 = __fmul_rn(a.h, rb);
  f2 r = f2_sub(a, f2_mulf(b, q1));
  const float q2 = __fmul_rn(r.h, rb);
  r = f2_sub(r, f2_mulf(b, q2));
  const float q3 = __fmul_rn(r.h, rb);
  float s, e;
  fast_two_sum(q1, q2, s, e);
  return f2_addf({s, e}, q3);
}

__device__ __forceinline__ f2 f2_rcp(f2 b) { return f2_div(f2_f(1.0f), b); }

// sqrt(a) for a >= 0 (0 for a <= 0)
__device__ __forceinline__ f2 f2_sqrt(f2 a) {
  if (!(a.h > 0.0f)) return f2_f(0.0f);
  const float x = rsqrtf(a.h);
  float y = __fmul_rn(a.h, x);
  y = __fmaf_rn(__fmul_rn(0.5f, x), __fmaf_rn(-y, y, a.h), y);  // float Newton step
  float p, e;
  two_prod(y, y, p, e);
  // a - y^2 (a.h - p is exact: they agree to ~2^-23)
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.h, p), e), a.l);
  float s, t;
  fast_two_sum(y, __fmul_rn(__fmul_rn(0.5f, x), d), s, t);
  return {s, t};
}

// 1/sqrt(a) for a > 0: a float estimate refined by one float Newton step,
// then the correction y (1 - r)^(-1/2) ~ y (1 + r/2 + 3 r^2/8) with
// r = 1 - a y^2 formed from exact products (|r| ~ 2^-23, so float holds it
// to the bits that matter and the series' next term is below 2^-68)
__device__ __forceinline__ f2 f2_rsqrt(f2 a) {
  float y = rsqrtf(a.h);
  y = __fmaf_rn(__fmul_rn(0.5f, y), __fmaf_rn(-a.h, __fmul_rn(y, y), 1.0f), y);
  float p, e1, q, e2;
  two_prod(y, y, p, e1);    // y^2 = p + e1
  two_prod(a.h, p, q, e2);  // a.h p = q + e2
  const float r = __fsub_rn(__fsub_rn(__fsub_rn(__fsub_rn(1.0f, q), e2), __fmul_rn(a.h, e1)),
                            __fmul_rn(a.l, p));
  float s, t;
  fast_two_sum(y, __fmul_rn(y, __fmul_rn(r, __fmaf_rn(0.375f, r, 0.5f))), s, t);
  return {s, t};
}

// ---- constants -------------------------------------------------------------
// ln 2 = kLn2a + kLn2b + kLn2c (16 + 16 significant bits + float)
constexpr float kLn2a = 0x1.62e4p-1f, kLn2b = 0x1.7f7ep-20f, kLn2c = -0x1.c610cap-37f;
// pi/2 = kPio2a + kPio2b + kPio2c
constexpr float kPio2a = 0x1.922p+0f, kPio2b = -0x1.2aeep-18f, kPio2c = -0x1.e973dcp-35f;
constexpr float kLog2e = 0x1.715476p+0f;  // log2 e, nearest float
constexpr float kTwoOPi = 0x1.45f306p-1f; // 2/pi, nearest float
constexpr float kPiH = 0x1.921fb6p+1f, kPiL = -0x1.777a5cp-24f;  // pi
// 1/n!, n = 0..19: nearest float and nearest float of the remainder
__device__ __constant__ const float kInvFact[20][2] = {
    {0x1p+0f, 0.0f},
    {0x1p+0f, 0.0f},
    {0x1p-1f, 0.0f},
    {0x1.555556p-3f, -0x1.555556p-28f},
    {0x1.555556p-5f, -0x1.555556p-30f},
    {0x1.111112p-7f, -0x1.dddddep-32f},
    {0x1.6c16c2p-10f, -0x1.27d27ep-35f},
    {0x1.a01a02p-13f, -0x1.7f97fap-39f},
    {0x1.a01a02p-16f, -0x1.7f97fap-42f},
    {0x1.71de3ap-19f, 0x1.55b1ccp-45f},
    {0x1.27e4fcp-22f, -0x1.10ec14p-47f},
    {0x1.ae6456p-26f, 0x1.fd5138p-52f},
    {0x1.1eed8ep-29f, 0x1.ff1b12p-54f},
    {0x1.612462p-33f, -0x1.8af25ep-58f},
    {0x1.93974ap-37f, 0x1.180f94p-62f},
    {0x1.ae7f3ep-41f, 0x1.ccee08p-67f},
    {0x1.ae7f3ep-45f, 0x1.ccee08p-71f},
    {0x1.952c78p-49f, -0x1.f9ea56p-74f},
    {0x1.682786p-53f, 0x1.dcbeccp-80f},
    {0x1.2f49b4p-57f, 0x1.a05056p-83f}};

__device__ __forceinline__ f2 inv_fact(int n) { return {kInvFact[n][0], kInvFact[n][1]}; }

// a - k (c1 + c2 + c3), k an integer-valued float with |k| < 2^8: k c1 and
// k c2 are exact (16-bit constants), k c3 is formed exactly by two_prod
__device__ __forceinline__ f2 f2_reduce(f2 a, float k, float c1, float c2, float c3) {
  f2 r = f2_addf(a, -__fmul_rn(k, c1));
  r = f2_addf(r, -__fmul_rn(k, c2));
  float p, e;
  two_prod(k, c3, p, e);
  return f2_sub(r, {p, e});
}

// sum_{n<N} coef(n) x^n by Estrin's scheme: the pairs coef(2k) +
// coef(2k+1) x, then pairs of those with x^2, with x^4, with x^8 -- four
// levels of dependent multiply-adds (N <= 16) instead of Horner's N - 1.
template <int N, class Coef>
__device__ __forceinline__ f2 f2_estrin(f2 x, Coef coef) {
  static_assert(N >= 2 && N <= 16, "Estrin: 2..16 coefficients");
  f2 v[(N + 1) / 2];
#pragma unroll
  for (int k = 0; k < (N + 1) / 2; ++k)
    v[k] = 2 * k + 1 < N ? f2_fma(coef(2 * k + 1), x, coef(2 * k)) : coef(2 * k);
  f2 xp = f2_sqr(x);
#pragma unroll
  for (int m = (N + 1) / 2; m > 1; m = (m + 1) / 2) {
#pragma unroll
    for (int k = 0; k < (m + 1) / 2; ++k)
      v[k] = 2 * k + 1 < m ? f2_fma(v[2 * k + 1], xp, v[2 * k]) : v[2 * k];
    xp = f2_sqr(xp);
  }
  return v[0];
}

// exp(a) for |a.h| <= 87 (the caller keeps the argument there)
__device__ __forceinline__ f2 f2_exp(f2 a) {
  const float k = rintf(__fmul_rn(a.h, kLog2e));
  const f2 r = f2_reduce(a, k, kLn2a, kLn2b, kLn2c);
  const f2 s = f2_estrin<14>(r, [](int n) { return inv_fact(n); });
  const int ki = (int)k;
  return {ldexpf(s.h, ki), ldexpf(s.l, ki)};
}

// cos(a) for |a.h| < 256 pi/2 (the caller keeps the argument there)
__device__ __forceinline__ f2 f2_cos(f2 a) {
  const float k = rintf(__fmul_rn(a.h, kTwoOPi));
  const f2 r = f2_reduce(a, k, kPio2a, kPio2b, kPio2c);
  const f2 s = f2_sqr(r);
  const int q = ((int)k) & 3;
  f2 v;
  if (q & 1)  // sin r = r (1 - r^2/3! + r^4/5! ...)
    v = f2_mul(f2_estrin<10>(s, [](int n) {
                 const f2 c = inv_fact(2 * n + 1);
                 return (n & 1) ? f2_neg(c) : c;
               }),
               r);
  else  // cos r = 1 - r^2/2! + r^4/4! ...
    v = f2_estrin<10>(s, [](int n) {
      const f2 c = inv_fact(2 * n);
      return (n & 1) ? f2_neg(c) : c;
    });
  // cos(r + k pi/2) = cos r, -sin r, -cos r, sin r for k = 0, 1, 2, 3 mod 4
  return (q == 1 || q == 2) ? f2_neg(v) : v;
}

}  // namespace bgpu
