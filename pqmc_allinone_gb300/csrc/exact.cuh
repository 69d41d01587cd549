// exact.cuh -- the exact round update of the batched mixed-precision sweep.
//
// A scan round decides its moves from FP32 ratios and records the accepted
// plaquettes (sites S in acceptance order, their Delta blocks).  The round's
// accepted rank-dim updates of src/mod_update.f90:146-192 compose, because
// the plaquettes of a family are disjoint, into one Woodbury update of the G
// the round started from:
//
//   G <- G + G(:,S) M (E_S - G(S,:)),   M = Delta_S W^-1,  W = I + G(S,S) Delta_S,
//
// with Delta_S block diagonal.  (The block pivots of W in acceptance order
// are the sequential ratio matrices R_j = I + Geff_j(S_j,S_j) Delta_j of the
// reference.)  The update is evaluated from the double-float G, never from
// the scan's FP32 panels:
//   k_xslice  the Ozaki slices of G(:,S) and of Z = E_S - G(S,:);
//   k_xinv    W in double-float and the FP32 inverse V0 of its rounding;
//   k_xres    one Newton step V1 = V0 + V0 (I - W V0) with a double-float
//             residual, M = Delta_S V1 and the Ozaki slices of M;
//   k_xgemm   X = G(:,S) M, then G += X Z, on the tensor cores: every
//             operand is cut into OZ_S BF16 slices on a per-row (per-column)
//             power-of-two grid, so that the products of one slice level
//             sum exactly in an FP32 accumulator (Ozaki, Ogita, Oishi and
//             Rump, "Error-free transformations of matrix multiplication",
//             Numer. Algorithms 59 (2012)); the levels are combined in
//             double-float.
#pragma once
#include "chain.cuh"
#include "tc.cuh"

namespace pqmc {

constexpr int OZ_S = 5;   // BF16 slices per operand (8 bits each)

// one chain of the exact update (device array, one entry per chain)
struct XDesc {
  float4* g;               // double-float G, parity 0
  float4* g_alt;           // parity 1
  int ns, ncopy, tr_weight, kmax;
  const int* kcount;       // panel columns of the round (written by the scan)
  int* acc_site;           // (kmax) accepted sites, dim per move, in acceptance order
  float4* acc_delta;       // (kmax) 16 entries per accepted move: its Delta (double-float)
  float4* wdf;             // (kmax x kmax) W in double-float, column j at wdf + j*kmax
  float2* v0;              // (kmax x kmax) FP32 inverse of W
  unsigned char* img;      // slice images (oz_chain_bytes)
  DevScalars* sc;
  int* err;
  unsigned long long* nflush;   // flushes with columns (roofline accounting)
};

// image slots of one chain: A of G(:,S) and of X (row tiles), B of M, B of Z
// (column tiles), OZ_S slices each, UM_IMG bytes per slot
__host__ __device__ __forceinline__ int oz_slot_a1(int ns, int t, int s) { (void)ns; return t * OZ_S + s; }
__host__ __device__ __forceinline__ int oz_slot_a2(int ns, int t, int s) { return (um_rtiles(ns) + t) * OZ_S + s; }
__host__ __device__ __forceinline__ int oz_slot_b1(int ns, int s) { return 2 * um_rtiles(ns) * OZ_S + s; }
__host__ __device__ __forceinline__ int oz_slot_b2(int ns, int t, int s) {
  return (2 * um_rtiles(ns) + 1 + t) * OZ_S + s;
}
// Z's column tiles: 64 columns for k_xgemm<1>, 32 for k_xflush2; slots for
// the narrower ones, which are more
__host__ __device__ __forceinline__ int oz_ztiles(int ns) { return (ns + 31) / 32; }
__host__ __device__ __forceinline__ size_t oz_chain_bytes(int ns) {
  return (size_t)(2 * um_rtiles(ns) + 1 + oz_ztiles(ns)) * OZ_S * UM_IMG;
}

// The exact update of one round for C chains: exact_core (three launches:
// the operand slices, W^-1, M) and exact_products (two launches: the
// tensor-core products).  `prio` marks the launches with priority
// `prio_hi` (kept as node priorities when the stream is being captured).
// ct: the flush tile's width, 64 (k_xgemm<1>, one CTA per SM) or 32
// (k_xflush2, two CTAs per SM); exact_core cuts Z into tiles of that width
int exact_core(const XDesc* d_x, int C, int ns, int dim, int parity, int ct, cudaStream_t st, bool prio,
               int prio_hi);
int exact_products(const XDesc* d_x, int C, int ns, int parity, int ct, cudaStream_t st, bool prio, int prio_hi);
int exact_setup();   // raises the kernels' dynamic shared-memory limits

}  // namespace pqmc
