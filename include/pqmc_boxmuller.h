/*
 * pqmc_boxmuller.h -- the Gaussian phonon-field proposal (jump_distance *
 * N(0,1) by Box-Muller on two ran2 draws, PQMC_PROPOSAL_GAUSSIAN) evaluated
 * with IEEE double additions, multiplications, one division and one square
 * root in a fixed order, so that the CUDA kernels and a C++ host build
 * produce the same bits: no library logarithm or cosine (whose last bit may
 * differ between the device and host libraries) and no fused multiply-add
 * (device operations are the explicitly rounded __dmul_rn / __dadd_rn; host
 * code is compiled with -ffp-contract=off).
 *
 *   log u    u = m 2^e with m in (1/sqrt2, sqrt2] split from the bits;
 *            log m = 2 atanh s, s = (m - 1)/(m + 1), by the odd series of
 *            atanh to s^23 (|s| <= 0.172, truncation below 2^-60); e ln 2
 *            with ln 2 split into a high part with trailing zero bits and a
 *            low part (the Cody-Waite reduction, Cody and Waite, "Software
 *            Manual for the Elementary Functions", 1980).
 *   cos 2pi t  t reduced in turns exactly (t - floor(t + 1/2), symmetries
 *            about 1/4 and 1/8), then the Taylor series of cos or sin at
 *            |z| <= pi/4 to z^18 / z^19 (truncation below 2^-60).
 * Both are accurate to a few units in the last place; what matters for the
 * accept/reject sequence is that device and host agree bit for bit.
 */
#ifndef PQMC_BOXMULLER_H
#define PQMC_BOXMULLER_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PQMC_BM_FN __host__ __device__ __forceinline__
#else
#define PQMC_BM_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define PQMC_BM_MUL(a, b) __dmul_rn((a), (b))
#define PQMC_BM_ADD(a, b) __dadd_rn((a), (b))
#define PQMC_BM_DIV(a, b) __ddiv_rn((a), (b))
#define PQMC_BM_SQRT(a) __dsqrt_rn(a)
#else
#define PQMC_BM_MUL(a, b) ((a) * (b))
#define PQMC_BM_ADD(a, b) ((a) + (b))
#define PQMC_BM_DIV(a, b) ((a) / (b))
#define PQMC_BM_SQRT(a) sqrt(a)
#endif

PQMC_BM_FN int64_t pqmc_bm_bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
PQMC_BM_FN double pqmc_bm_from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

/* natural logarithm of a positive normal double */
PQMC_BM_FN double pqmc_bm_log(double u) {
  const int64_t bits = pqmc_bm_bits(u);
  int e = (int)((bits >> 52) & 0x7ff) - 1023;
  double m = pqmc_bm_from_bits((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);   /* [1, 2) */
  if (m > 1.4142135623730951) {   /* sqrt 2 */
    m = PQMC_BM_MUL(m, 0.5);
    e += 1;
  }
  const double s = PQMC_BM_DIV(PQMC_BM_ADD(m, -1.0), PQMC_BM_ADD(m, 1.0));
  const double z = PQMC_BM_MUL(s, s);
  double q = 1.0 / 23.0;
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 21.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 19.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 17.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 15.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 13.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 11.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 9.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 7.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 5.0);
  q = PQMC_BM_ADD(PQMC_BM_MUL(q, z), 1.0 / 3.0);
  /* log m = 2 s (1 + z q) */
  const double lm = PQMC_BM_MUL(PQMC_BM_MUL(2.0, s), PQMC_BM_ADD(1.0, PQMC_BM_MUL(z, q)));
  const double ln2_hi = 6.93147180369123816490e-01; /* ln 2 rounded to 32 significant bits */
  const double ln2_lo = 1.90821492927058770002e-10; /* ln 2 - ln2_hi */
  const double de = (double)e;
  return PQMC_BM_ADD(PQMC_BM_MUL(de, ln2_hi), PQMC_BM_ADD(lm, PQMC_BM_MUL(de, ln2_lo)));
}

/* cos(2 pi t) for a double t whose 2t + 1 is exact (any value of a ran2 draw) */
PQMC_BM_FN double pqmc_bm_cos2pi(double t) {
  double fl = (double)(int64_t)PQMC_BM_ADD(t, 0.5);   /* floor for t > -1/2 */
  if (fl > PQMC_BM_ADD(t, 0.5)) fl = PQMC_BM_ADD(fl, -1.0);
  double a = PQMC_BM_ADD(t, -fl);   /* in [-1/2, 1/2) */
  if (a < 0.0) a = -a;
  double sign = 1.0;
  if (a > 0.25) { /* cos 2pi a = -cos 2pi (1/2 - a) */
    a = PQMC_BM_ADD(0.5, -a);
    sign = -1.0;
  }
  const bool use_sin = a > 0.125; /* cos 2pi a = sin 2pi (1/4 - a) */
  if (use_sin) a = PQMC_BM_ADD(0.25, -a);
  const double zz = PQMC_BM_MUL(6.283185307179586, a);   /* in [0, pi/4] */
  const double w = PQMC_BM_MUL(zz, zz);
  double r;
  if (use_sin) {
    double p = -1.0 / 121645100408832000.0;   /* -1/19! */
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 355687428096000.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 1307674368000.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 6227020800.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 39916800.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 362880.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 5040.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 120.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 6.0);
    r = PQMC_BM_ADD(zz, PQMC_BM_MUL(PQMC_BM_MUL(zz, w), p));   /* z + z^3 p(w) */
  } else {
    double p = 1.0 / 6402373705728000.0;   /* 1/18! */
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 20922789888000.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 87178291200.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 479001600.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 3628800.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 40320.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 1.0 / 720.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), -1.0 / 24.0);
    p = PQMC_BM_ADD(PQMC_BM_MUL(p, w), 0.5);
    r = PQMC_BM_ADD(1.0, -PQMC_BM_MUL(w, p));   /* 1 - w (1/2 - w/24 + ...) */
  }
  return PQMC_BM_MUL(sign, r);
}

/* the Gaussian jump jump_distance * sqrt(-2 log u1) cos(2 pi u2) */
PQMC_BM_FN double pqmc_bm_gauss_jump(double jump_distance, double u1, double u2) {
  const double rad = PQMC_BM_SQRT(PQMC_BM_MUL(-2.0, pqmc_bm_log(u1)));
  return PQMC_BM_MUL(jump_distance, PQMC_BM_MUL(rad, pqmc_bm_cos2pi(u2)));
}

#endif /* PQMC_BOXMULLER_H */
