// ozaki.cuh -- error-free splitting of double-float values into BF16 slices
// (the Ozaki scheme: Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication", Numer. Algorithms 59 (2012)), shared by the exact round
// update (exact.cu, 5 slices) and the recompute's GEMMs (ozgemm.cu, 6).
//
// A row (column) whose entries have magnitude below 2^e is cut into NS
// pieces on the grids 2^(e-8), 2^(e-16), ...: piece s is an integer of at
// most 256 (129 after the first) times 2^(e-8(s+1)), exact in BF16.  Two
// pieces multiply exactly, and the products of one level (i + j) share a
// grid, so up to 128 of them sum exactly in an FP32 accumulator for levels
// 0, 1 and 2 (|sum| < 2^24 grid units).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include "df32.cuh"

namespace pqmc {

// the exponent e of a row with largest |entry| vmax (vmax < 2^e), at least
// FLOOR; with NS pieces FLOOR >= 8 NS - 126 keeps the deepest grid
// 2^(e - 8 NS) a normal FP32 power of two
template <int FLOOR>
__device__ __forceinline__ int oz_exp_f(float vmax) {
  const int b = (__float_as_int(vmax) >> 23) & 0xff;   // vmax >= 0
  return vmax > 0.f ? max(b - 126, FLOOR) : FLOOR;     // vmax < 2^(b-126)
}
__device__ __forceinline__ float oz_pow2(int k) { return __int_as_float((127 + k) << 23); }   // |k| <= 126

// the NS pieces of the double-float value (h, l) for the exponent e
template <int NS>
__device__ __forceinline__ void oz_split_n(float h, float l, int e, float* q) {
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const int sh = 8 * (s + 1) - e;
    const float v = rintf(__fmul_rn(h, oz_pow2(sh)));
    const float qs = __fmul_rn(v, oz_pow2(-sh));
    q[s] = qs;
    h = __fsub_rn(h, qs);   // exact: h and qs lie within half a grid step
    const df n = two_sum(h, l);
    h = n.hi;
    l = n.lo;
  }
}
__device__ __forceinline__ uint32_t oz_pack2(float a, float b) {
  __nv_bfloat162 t = __floats2bfloat162_rn(a, b);   // a at the lower address
  return *reinterpret_cast<uint32_t*>(&t);
}
__device__ __forceinline__ uint4 oz_pack8(const float* v) {
  return make_uint4(oz_pack2(v[0], v[1]), oz_pack2(v[2], v[3]), oz_pack2(v[4], v[5]), oz_pack2(v[6], v[7]));
}

}  // namespace pqmc
