// rng.cuh -- device copy of ran2_s (src/mod_ranstate.f90:171-191).
//
// Integer recurrence in 32-bit wrap-around arithmetic; the REAL(SP) result
// amm*merge(rans, not(rans), rans<0) with amm = nearest(1.0_sp,-1.0_sp)/
// hgng (:59) is formed with round-to-nearest single-precision intrinsics so
// the compiler cannot fuse or widen it.  ran_sysm (:233-236) = r*2-1 in
// single precision.
#pragma once
#include <stdint.h>

struct Ran2Dev {
  int32_t iran, jran, kran, mran, nran;

  __device__ __forceinline__ float next() {
    int32_t rans = (int32_t)((uint32_t)iran - (uint32_t)kran);
    if (rans < 0) rans = (int32_t)((uint32_t)rans + 2147483579u);
    iran = jran;
    jran = kran;
    kran = rans;
    uint32_t n = (uint32_t)nran;
    n ^= n << 13;
    n ^= n >> 17;
    n ^= n << 5;
    nran = (int32_t)n;
    uint32_t m = (uint32_t)mran;
    uint32_t lo = m & 65535u;
    m = ((3533u * (m >> 16) + lo) << 16) + 3533u * lo + 820265819u;
    mran = (int32_t)m;
    int32_t r = (int32_t)(((uint32_t)nran ^ (uint32_t)kran) + (uint32_t)mran);
    int32_t v = r < 0 ? r : ~r;
    const float amm = __fdiv_rn(0.99999994039535522461f, -2147483648.0f);
    return __fmul_rn(amm, __int2float_rn(v));
  }
  __device__ __forceinline__ float ran_sysm() {
    float r = next();
    return __fsub_rn(__fmul_rn(r, 2.0f), 1.0f);
  }
};
