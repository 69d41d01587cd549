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

// single FP32 complex values (float2 {re, im})
__device__ __forceinline__ float2 f2(double2 a) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ float2 fm(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 fa(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsb(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// the high words of a double-float complex (the FP32 rounding of its value)
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.x, v.y); }
// acc + a*b in four FMAs
__device__ __forceinline__ float2 fcfma(float2 a, float2 b, float2 acc) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y)));
}

__device__ __forceinline__ float2 fdiv1(float2 a) {   // 1/a
  float n = a.x * a.x + a.y * a.y;
  return make_float2(a.x / n, -a.y / n);
}

// small complex inverse in FP32 by Gauss-Jordan with partial pivoting on one
// thread (sizes below 4)
__device__ inline void finv_small(int n, float2* a) {
  float2 inv[16];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) inv[i + n * j] = make_float2(i == j ? 1.f : 0.f, 0.f);
  for (int j = 0; j < n; ++j) {
    int jp = j;
    float best = -1.f;
    for (int i = j; i < n; ++i) {
      float v = fabsf(a[i + n * j].x) + fabsf(a[i + n * j].y);
      if (v > best) { best = v; jp = i; }
    }
    if (jp != j)
      for (int k = 0; k < n; ++k) {
        float2 t = a[j + n * k]; a[j + n * k] = a[jp + n * k]; a[jp + n * k] = t;
        t = inv[j + n * k]; inv[j + n * k] = inv[jp + n * k]; inv[jp + n * k] = t;
      }
    float2 r = fdiv1(a[j + n * j]);
    for (int k = 0; k < n; ++k) { a[j + n * k] = fm(a[j + n * k], r); inv[j + n * k] = fm(inv[j + n * k], r); }
    for (int i = 0; i < n; ++i) {
      if (i == j) continue;
      float2 f = a[i + n * j];
      for (int k = 0; k < n; ++k) {
        a[i + n * k] = fsb(a[i + n * k], fm(f, a[j + n * k]));
        inv[i + n * k] = fsb(inv[i + n * k], fm(f, inv[j + n * k]));
      }
    }
  }
  for (int k = 0; k < n * n; ++k) a[k] = inv[k];
}

__device__ inline float2 fdet_small(int n, const float2* a) {
  if (n == 1) return a[0];
  if (n == 2) return fsb(fm(a[0], a[3]), fm(a[2], a[1]));
  float2 b[16];
  for (int k = 0; k < n * n; ++k) b[k] = a[k];
  float2 det = make_float2(1.f, 0.f);
  for (int j = 0; j < n; ++j) {
    int jp = j;
    float best = -1.f;
    for (int i = j; i < n; ++i) {
      float v = fabsf(b[i + n * j].x) + fabsf(b[i + n * j].y);
      if (v > best) { best = v; jp = i; }
    }
    if (jp != j) {
      for (int k = 0; k < n; ++k) { float2 t = b[j + n * k]; b[j + n * k] = b[jp + n * k]; b[jp + n * k] = t; }
      det = make_float2(-det.x, -det.y);
    }
    det = fm(det, b[j + n * j]);
    float2 r = fdiv1(b[j + n * j]);
    for (int i = j + 1; i < n; ++i) {
      float2 f = fm(b[i + n * j], r);
      for (int k = j; k < n; ++k) b[i + n * k] = fsb(b[i + n * k], fm(f, b[j + n * k]));
    }
  }
  return det;
}

// determinant of the dim x dim FP32 matrix R (shared, column-major) returned
// to every lane: Laplace expansion along rows 0,1 over six lanes for dim 4,
// lane 0 otherwise
__device__ __forceinline__ float2 wf_det(int dim, const float2* R, int lane) {
  float2 v = make_float2(0.f, 0.f);
  if (dim == 4) {
    if (lane < 6) {
      // column pair (j,k) of rows 0,1 and the complementary pair (l,m) of
      // rows 2,3, packed one hex digit per lane (no local-memory tables)
      const int sh = 4 * lane;
      const int j = (0x211000 >> sh) & 15, k = (0x332321 >> sh) & 15;
      const int l = (0x000112 >> sh) & 15, m = (0x123233 >> sh) & 15;
      const float sg = ((0x12 >> lane) & 1) ? -1.f : 1.f;
      float2 mi = fsb(fm(R[0 + 4 * j], R[1 + 4 * k]), fm(R[0 + 4 * k], R[1 + 4 * j]));
      float2 co = fsb(fm(R[2 + 4 * l], R[3 + 4 * m]), fm(R[2 + 4 * m], R[3 + 4 * l]));
      float2 t = fm(mi, co);
      v = make_float2(sg * t.x, sg * t.y);
    }
    for (int o = 4; o > 0; o >>= 1) {
      float vx = __shfl_down_sync(0xffffffffu, v.x, o), vy = __shfl_down_sync(0xffffffffu, v.y, o);
      if (lane + o < 8) { v.x += vx; v.y += vy; }
    }
  } else if (lane == 0) {
    v = fdet_small(dim, R);
  }
  return make_float2(__shfl_sync(0xffffffffu, v.x, 0), __shfl_sync(0xffffffffu, v.y, 0));
}

// R <- R^-1 in place (shared, column-major): adjugate over 16 lanes for dim 4
// (the complementary row/column triples formed branch-free, one reciprocal
// of |det|^2 per lane), lane-0 Gauss-Jordan otherwise
__device__ __forceinline__ void wf_inverse(int dim, float2* R, float2 det, int lane) {
  if (dim == 4) {
    float2 cof = make_float2(0.f, 0.f);
    const int i = lane & 3, j = lane >> 2;
    if (lane < 16) {
      // rows other than i and columns other than j, ascending
      const int r0 = i == 0 ? 1 : 0, r1 = i <= 1 ? 2 : 1, r2 = i <= 2 ? 3 : 2;
      const int c0 = j == 0 ? 1 : 0, c1 = j <= 1 ? 2 : 1, c2 = j <= 2 ? 3 : 2;
      const float2 a00 = R[r0 + 4 * c0], a01 = R[r0 + 4 * c1], a02 = R[r0 + 4 * c2];
      const float2 a10 = R[r1 + 4 * c0], a11 = R[r1 + 4 * c1], a12 = R[r1 + 4 * c2];
      const float2 a20 = R[r2 + 4 * c0], a21 = R[r2 + 4 * c1], a22 = R[r2 + 4 * c2];
      cof = fa(fsb(fm(a00, fsb(fm(a11, a22), fm(a12, a21))), fm(a01, fsb(fm(a10, a22), fm(a12, a20)))),
               fm(a02, fsb(fm(a10, a21), fm(a11, a20))));
      if ((i + j) & 1) cof = make_float2(-cof.x, -cof.y);
      const float rn = __frcp_rn(det.x * det.x + det.y * det.y);   // 1/det = conj(det)/|det|^2
      cof = fm(cof, make_float2(det.x * rn, -det.y * rn));
    }
    __syncwarp();
    if (lane < 16) R[j + 4 * i] = cof;
    __syncwarp();
    return;
  }
  if (lane == 0) finv_small(dim, R);
  __syncwarp();
}
