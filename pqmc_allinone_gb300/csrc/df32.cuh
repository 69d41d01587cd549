// df32.cuh -- double-float arithmetic: a value is hi + lo with two FP32
// words (48-bit significand, FP32 exponent range).  Error-free
// transformations after Dekker (1971) and Knuth's two-sum; products use the
// FMA two-product.  On GB300 the FP32 pipe is ~67x the FP64 pipe, so FP64-
// class accuracy for the bulk linear algebra of the batched form is cheaper
// here than native FP64.
#pragma once
#include <cuda_runtime.h>

struct df {
  float hi, lo;
};
struct dfc {
  df re, im;
};

__device__ __forceinline__ df df_make(double v) {
  float h = __double2float_rn(v);
  float l = __double2float_rn(v - (double)h);
  return df{h, l};
}
__device__ __forceinline__ double df_to_d(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df{s, e};
}
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df df_mulf(df a, float b) {
  float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df df_div(df a, df b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  df r = df_sub(a, df_mulf(b, q1));
  float q2 = __fdiv_rn(r.hi, b.hi);
  r = df_sub(r, df_mulf(b, q2));
  float q3 = __fdiv_rn(r.hi, b.hi);
  df q = quick_two_sum(q1, q2);
  return df_add(q, df{q3, 0.0f});
}
__device__ __forceinline__ df df_sqrt(df a) {
  if (a.hi <= 0.0f) return df{0.0f, 0.0f};
  float x = rsqrtf(a.hi);
  float y = __fmul_rn(a.hi, x);
  df yy = df_mul(df{y, 0.0f}, df{y, 0.0f});
  float d = __fmul_rn(df_sub(a, yy).hi, __fmul_rn(x, 0.5f));
  return two_sum(y, d);
}

// complex
__device__ __forceinline__ dfc dfc_make(double2 v) { return dfc{df_make(v.x), df_make(v.y)}; }
__device__ __forceinline__ double2 dfc_to_d(dfc a) { return make_double2(df_to_d(a.re), df_to_d(a.im)); }
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfc{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfc{df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return dfc{df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
// conj(a) * b
__device__ __forceinline__ dfc dfc_mulc(dfc a, dfc b) {
  return dfc{df_add(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_sub(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfc_zero() { return dfc{{0.0f, 0.0f}, {0.0f, 0.0f}}; }

// A complex double-float held in 16 bytes as float4 {re_hi, im_hi, re_lo,
// im_lo}: the storage of G inside a mixed-precision batched sweep (the same
// footprint as an FP64 complex, converted in place at the sweep boundary).
__device__ __forceinline__ float4 dg_make(double2 v) {
  const df r = df_make(v.x), i = df_make(v.y);
  return make_float4(r.hi, i.hi, r.lo, i.lo);
}
__device__ __forceinline__ double2 dg_to_d(float4 g) {
  return make_double2((double)g.x + (double)g.z, (double)g.y + (double)g.w);
}
// rounded to a single FP32 complex
__device__ __forceinline__ float2 dg_f2(float4 g) { return make_float2(__fadd_rn(g.x, g.z), __fadd_rn(g.y, g.w)); }
// (hi, lo) += a, a an FP32 value (two-sum, then renormalise)
__device__ __forceinline__ void df_accf(float& hi, float& lo, float a) {
  df s = two_sum(hi, a);
  s.lo = __fadd_rn(s.lo, lo);
  s = quick_two_sum(s.hi, s.lo);
  hi = s.hi;
  lo = s.lo;
}
__device__ __forceinline__ float4 dg_addf(float4 g, float2 a) {
  df_accf(g.x, g.z, a.x);
  df_accf(g.y, g.w, a.y);
  return g;
}
__device__ __forceinline__ float4 dg_from_dfc(dfc a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }
__device__ __forceinline__ dfc dfc_from_dg(float4 g) { return dfc{df{g.x, g.z}, df{g.y, g.w}}; }

// (h, l) -= x*y for double-float reals: the product formed error-free
// (FMA two-product plus the hi*lo cross terms), its high part subtracted by a
// two-sum, the low-order parts gathered in l (not renormalised)
__device__ __forceinline__ void df_msub_acc(float& h, float& l, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = __fmaf_rn(xh, yh, -p);
  const float c = __fmaf_rn(xh, yl, __fmul_rn(xl, yh));
  const df s = two_sum(h, -p);
  h = s.hi;
  l = __fsub_rn(__fadd_rn(l, s.lo), __fadd_rn(e, c));
}
// a - f*b for double-float complex values, one renormalisation per component
// (about half the instructions of dfc_sub(a, dfc_mul(f, b)))
__device__ __forceinline__ dfc dfc_fms(dfc a, dfc f, dfc b) {
  float rh = a.re.hi, rl = a.re.lo, ih = a.im.hi, il = a.im.lo;
  df_msub_acc(rh, rl, f.re.hi, f.re.lo, b.re.hi, b.re.lo);     // re -= fr br
  df_msub_acc(rh, rl, -f.im.hi, -f.im.lo, b.im.hi, b.im.lo);   // re += fi bi
  df_msub_acc(ih, il, f.re.hi, f.re.lo, b.im.hi, b.im.lo);     // im -= fr bi
  df_msub_acc(ih, il, f.im.hi, f.im.lo, b.re.hi, b.re.lo);     // im -= fi br
  return dfc{quick_two_sum(rh, rl), quick_two_sum(ih, il)};
}
