// Shared device helpers for the GB300 exterior Helmholtz BEM kernels.
//
// Complex numbers are interleaved (re, im) float2 / double2.  "df" is
// double-float arithmetic: a value carried as an unevaluated sum hi + lo of two
// floats, built from the error-free transformations two-sum (Knuth) and
// two-product (via fmaf).  It carries ~44 bits of significand at a handful of
// FP32 instructions per operation, which matters on this part: FP64 issues at a
// small fraction of the FP32 rate.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#define BEM_HD __host__ __device__ __forceinline__
#define BEM_D __device__ __forceinline__

// -------------------------------------------------------------- complex ----
BEM_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
BEM_HD double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
BEM_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
BEM_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
BEM_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
BEM_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
BEM_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
BEM_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

template <typename R> struct cplx;
template <> struct cplx<float> {
  typedef float2 type;
  static BEM_HD float2 make(float a, float b) { return make_float2(a, b); }
};
template <> struct cplx<double> {
  typedef double2 type;
  static BEM_HD double2 make(double a, double b) { return make_double2(a, b); }
};

// ------------------------------------------------------------ double-float --
struct df {
  float hi, lo;
};

BEM_D df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
BEM_D df quick_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
BEM_D df two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}
BEM_D df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
BEM_D df df_neg(df a) { return {-a.hi, -a.lo}; }
BEM_D df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
BEM_D df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
BEM_D df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// sqrt of a positive df: one Newton step on an FP32 root taken from the
// approximate reciprocal root.  The step removes the root's error to second
// order (relative error about 2^-44); a.hi <= 0 gives 0.
BEM_D float rsqrt_ftz(float x);
BEM_D df df_sqrt(df a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  const float y = rsqrt_ftz(a.hi);
  const float s = a.hi * y;
  df s2 = two_prod(s, s);
  float r = ((a.hi - s2.hi) - s2.lo + a.lo) * (0.5f * y);
  return quick_two_sum(s, r);
}

// 2*pi as a three-term float expansion (hi + mid + lo), for argument reduction.
#define BEM_TWO_PI_HI 6.28318548202514648f
#define BEM_TWO_PI_MID -1.7484555314695172e-07f
#define BEM_TWO_PI_LO -6.8604980400235275e-15f
#define BEM_INV_TWO_PI 0.159154943091895336f
#define BEM_INV_FOUR_PI 0.0795774715459476678f

// Single-instruction approximations (PTX .approx.ftz: subnormal inputs and
// results flush to zero).  The library is built without -ftz, and the non-ftz
// forms of these PTX instructions carry subnormal handling around each one; the
// hot loops only apply them to arguments clamped well away from the subnormal
// range (r^2 >= 1e-30, |angle| <= pi + 1e-6).  Documented accuracy (PTX ISA):
// rsqrt/rcp about 2^-22 relative (rcp: 1 ulp), sin/cos 2^-20.5 absolute on [-pi, pi].
BEM_D float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
BEM_D float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
BEM_D void sincos_ftz(float x, float* s, float* c) {
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(*s) : "f"(x));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(*c) : "f"(x));
}
// Nearest integer of |x| < 2^22 on the FMA pipe: adding 1.5 * 2^23 rounds away
// every fraction bit (round to nearest even); subtracting it back is exact.
// __fadd_rn / __fsub_rn are never contracted with a multiply that produced x, so
// the result is that of the rounded x in every inlined context.
BEM_D float round_nearest_small(float x) {
  const float kMagic = 12582912.0f;
  return __fsub_rn(__fadd_rn(x, kMagic), kMagic);
}

// sin x and cos x with RELATIVE accuracy for small |x| (sin(z/2) feeds
// 1 - cos z = 2 sin^2(z/2), where an absolute-accuracy approximation loses all
// relative accuracy as z -> 0).  x is reduced by the nearest multiple n*pi (pi
// split in two floats; each multiple flips both signs), then the Taylor series
// in x^2: sin to x^13, cos to x^12, coefficients (-1)^j / (2j+1)! and
// (-1)^j / (2j)!; the truncation error is below 7e-9 on |x| <= pi/2.
// For |x| < 2^20.
BEM_D void sincos_taylor(float x, float* s, float* c) {
  const float n = round_nearest_small(x * 0.318309873342514f);
  float r = fmaf(-n, 3.14159274101257324f, x);
  r = fmaf(-n, -8.742278012618954e-08f, r);
  const float r2 = r * r;
  float ps = 1.6059043836821613e-10f;
  ps = fmaf(ps, r2, -2.505210838544172e-08f);
  ps = fmaf(ps, r2, 2.7557319223985893e-06f);
  ps = fmaf(ps, r2, -1.984126984126984e-04f);
  ps = fmaf(ps, r2, 8.333333333333333e-03f);
  ps = fmaf(ps, r2, -1.6666666666666666e-01f);
  float sv = fmaf(ps * r2, r, r);
  float pc = 2.08767569878681e-09f;
  pc = fmaf(pc, r2, -2.755731922398589e-07f);
  pc = fmaf(pc, r2, 2.48015873015873e-05f);
  pc = fmaf(pc, r2, -1.388888888888889e-03f);
  pc = fmaf(pc, r2, 4.1666666666666664e-02f);
  pc = fmaf(pc, r2, -0.5f);
  float cv = fmaf(pc, r2, 1.0f);
  // (-1)^n from the parity of n (|n| < 2^20, exact in float)
  const bool odd = (((int)n) & 1) != 0;
  *s = odd ? -sv : sv;
  *c = odd ? -cv : cv;
}

// theta = a - 2*pi*rint(a / 2pi) for a df angle; the result lies in [-pi, pi]
// and is accurate to about 2^-44 * |a| + 2^-24.
BEM_D float df_reduce_two_pi(df a) {
  float n = rintf(a.hi * BEM_INV_TWO_PI);
  df t = two_prod(-n, BEM_TWO_PI_HI);  // exact -n*2pi_hi
  df r = df_add(a, t);
  r = df_add(r, two_prod(-n, BEM_TWO_PI_MID));
  return r.hi + (r.lo - n * BEM_TWO_PI_LO);
}

// Reduce an FP32 angle of moderate size (|t| < 2^20) into [-pi, pi].
BEM_D float reduce_two_pi(float t) {
  float n = round_nearest_small(t * BEM_INV_TWO_PI);
  t = fmaf(-n, BEM_TWO_PI_HI, t);
  return fmaf(-n, BEM_TWO_PI_MID, t);
}

// -------------------------------------------------------- status / limits --
// Device status word written by kernels that can detect bad input; the host
// reads it after the launch.  No kernel traps or spins without a bound.
enum BemDeviceStatus : int {
  BEM_DEV_OK = 0,
  BEM_DEV_ZERO_PIVOT = 1,
  BEM_DEV_NONFINITE = 2,
};
