// recompute_b.cu -- stabilised Green's-function recompute for a batch of
// chains (get_g_scratch_T0 / cal_g_and_det_T0, src/mod_evolution.f90:113-195,
// 330-357) in double-float (df32) arithmetic on the FP32 pipe, with the
// log-weight accumulated in FP64.
//
// Per chain:  propagate the block (df32) -> CholeskyQR2 of the Ns x nelec
// factor (Gram, Cholesky and triangular inverse in df32) -> P^H B P ->
// Gauss-Jordan inverse with partial pivoting (log det from the pivots, FP64)
// -> G = R (P^H B P)^-1 L.  All products are batched complex GEMMs over the
// chains.  CholeskyQR gives the Householder Q up to column phases and
// |diag R| for D; G and Re ln_cw do not depend on those phases.
#include <cooperative_groups.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "chain.cuh"
#include "df32.cuh"
#include "ozgemm.cuh"
#include "recompute_b.cuh"

namespace pqmc {

// ---------------------------------------------------------------------------
// Batched complex GEMM, FP64 storage, df32 arithmetic:
//   C_c = op(A_c) op(B_c)  (+ C_c when accumulate)
struct GemmArgs {
  const cplx* A;
  const cplx* B;
  cplx* C;
  int lda, ldb, ldc;
  int out_df;   // C is written in the double-float float4 form (not accumulated)
  int shape;    // 0 general; 1 only the lower triangle of C is needed (Gram
                // matrix for a Cholesky factor); 2 B is upper triangular
  // A and B already split into double-float (re.hi, re.lo, im.hi, im.lo),
  // same layout and leading dimension (set by BatchRecompute::gemm)
  const float4* Adf = nullptr;
  const float4* Bdf = nullptr;
};

// one operand of one chain split into double-float once per GEMM, so that
// the k-tiles of every CTA that reads it stage it without FP64 instructions
// (a double -> float pair conversion issues on the FP64 pipe, 1/64 of the
// FP32 rate on this GPU, and each element is staged by every CTA of its
// row or column of tiles)
struct ConvArgs {
  const cplx* src;
  float4* dst;
  long n;
};
__global__ void k_gemm_split(const ConvArgs* args) {
  const ConvArgs a = args[blockIdx.y];
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < a.n; e += (long)gridDim.x * blockDim.x) {
    const cplx v = a.src[e];
    const df vr = df_make(v.x), vi = df_make(v.y);
    a.dst[e] = make_float4(vr.hi, vr.lo, vi.hi, vi.lo);
  }
}

// Batched complex GEMM with FP64-class accuracy on the FP32 pipe: the
// operands are split into double-float (hi + lo), every real product is
// formed error-free (hi*hi by FMA two-product plus the hi*lo cross terms),
// its high part enters the running sum through a two-sum and all low-order
// parts are summed in plain FP32 (the compensated dot product "Dot2" of
// Ogita, Rump and Oishi, 2005).  About 12 FP32 instructions per real
// multiply-add instead of ~27 for full double-float arithmetic.
// CTA tile 64 x 64, 4 x 4 outputs per thread, k-tiles of 16.
constexpr int DG_BM = 64, DG_BN = 64, DG_BK = 16;

struct d2acc {
  float h, l;
};
// acc += x*y, x = (xh, xl), y = (yh, yl)
__device__ __forceinline__ void dot2_mac(d2acc& acc, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = __fmaf_rn(xh, yh, -p);
  const float c = __fmaf_rn(xh, yl, __fmul_rn(xl, yh));
  const float s = __fadd_rn(acc.h, p);
  const float bb = __fsub_rn(s, acc.h);
  const float err = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.h = s;
  acc.l = __fadd_rn(acc.l, __fadd_rn(err, __fadd_rn(e, c)));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_dfgemm2(const GemmArgs* args, int m, int n, int k, int accumulate) {
  const GemmArgs g = args[blockIdx.z];
  // (re.hi, re.lo, im.hi, im.lo); one float4 of padding per row, so that the
  // staging of a conjugate-transposed operand (consecutive threads on
  // consecutive rows q) does not put a quarter-warp on one bank group
  __shared__ float4 sA[DG_BK][DG_BM + 1];
  __shared__ float4 sB[DG_BK][DG_BN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int row0 = blockIdx.x * DG_BM, col0 = blockIdx.y * DG_BN;
  if (g.shape == 1 && row0 + DG_BM <= col0) return;   // tile strictly above the diagonal
  if (g.shape == 2) k = min(k, col0 + DG_BN);          // B(q, c) = 0 for q > c
  d2acc cr[4][4], ci[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cr[i][j] = d2acc{0.f, 0.f};
      ci[i][j] = d2acc{0.f, 0.f};
    }
  for (int kk = 0; kk < k; kk += DG_BK) {
    // stage A(row0:+64, kk:+16) and B(kk:+16, col0:+64) as double-float, reading
    // memory in its contiguous direction
    for (int e = tid; e < DG_BM * DG_BK; e += 256) {
      int r, q;
      if (TA) { q = e % DG_BK; r = e / DG_BK; } else { r = e % DG_BM; q = e / DG_BM; }
      const int gr = row0 + r, gk = kk + q;
      if (g.Adf) {   // the split of df_make, bit for bit (conj negates both parts)
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gr < m && gk < k) {
          v = TA ? g.Adf[gk + (size_t)g.lda * gr] : g.Adf[gr + (size_t)g.lda * gk];
          if (TA) v = make_float4(v.x, v.y, -v.z, -v.w);
        }
        sA[q][r] = v;
        continue;
      }
      cplx v = mk(0.0);
      if (gr < m && gk < k) v = TA ? cconj(g.A[gk + (size_t)g.lda * gr]) : g.A[gr + (size_t)g.lda * gk];
      const df vr = df_make(v.x), vi = df_make(v.y);
      sA[q][r] = make_float4(vr.hi, vr.lo, vi.hi, vi.lo);
    }
    for (int e = tid; e < DG_BK * DG_BN; e += 256) {
      int q, c;
      if (TB) { c = e % DG_BN; q = e / DG_BN; } else { q = e % DG_BK; c = e / DG_BK; }
      const int gc = col0 + c, gk = kk + q;
      if (g.Bdf) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gc < n && gk < k) {
          v = TB ? g.Bdf[gc + (size_t)g.ldb * gk] : g.Bdf[gk + (size_t)g.ldb * gc];
          if (TB) v = make_float4(v.x, v.y, -v.z, -v.w);
        }
        sB[q][c] = v;
        continue;
      }
      cplx v = mk(0.0);
      if (gc < n && gk < k) v = TB ? cconj(g.B[gc + (size_t)g.ldb * gk]) : g.B[gk + (size_t)g.ldb * gc];
      const df vr = df_make(v.x), vi = df_make(v.y);
      sB[q][c] = make_float4(vr.hi, vr.lo, vi.hi, vi.lo);
    }
    __syncthreads();
#pragma unroll 2
    for (int q = 0; q < DG_BK; ++q) {
      float4 av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = sA[q][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = sB[q][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float4 x = av[i], y = bv[j];
          // re += xr yr - xi yi ; im += xr yi + xi yr
          dot2_mac(cr[i][j], x.x, x.y, y.x, y.y);
          dot2_mac(cr[i][j], -x.z, -x.w, y.z, y.w);
          dot2_mac(ci[i][j], x.x, x.y, y.z, y.w);
          dot2_mac(ci[i][j], x.z, x.w, y.x, y.y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = row0 + tx + 16 * i, c = col0 + ty + 16 * j;
      if (r >= m || c >= n) continue;
      df re = quick_two_sum(cr[i][j].h, cr[i][j].l), im = quick_two_sum(ci[i][j].h, ci[i][j].l);
      cplx* p = g.C + r + (size_t)g.ldc * c;
      if (g.out_df) {
        *reinterpret_cast<float4*>(p) = make_float4(re.hi, im.hi, re.lo, im.lo);
      } else if (accumulate) {
        const dfc v = dfc_add(dfc{re, im}, dfc_make(*p));
        *p = dfc_to_d(v);
      } else {
        *p = make_double2(df_to_d(re), df_to_d(im));
      }
    }
}

int dfgemm_batched(cudaStream_t s, char ta, char tb, int m, int n, int k, const GemmArgs* d_args, int count,
                   int accumulate) {
  dim3 grid((m + DG_BM - 1) / DG_BM, (n + DG_BN - 1) / DG_BN, count);
  bool TA = ta == 'C', TB = tb == 'C';
  if (!TA && !TB) k_dfgemm2<false, false><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else if (TA && !TB) k_dfgemm2<true, false><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else if (!TA && TB) k_dfgemm2<false, true><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else k_dfgemm2<true, true><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// block-wide helpers
__device__ __forceinline__ float blk_sum_f(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  float t = threadIdx.x < nw ? red[threadIdx.x] : 0.f;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) red[32] = t;
  __syncthreads();
  float r = red[32];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// Cholesky W = L L^H (lower, in place, df32 kept in a scratch copy), then
// Rinv = (L^H)^-1 = (L^-1)^H written as FP64 to `rinv` (n x n, upper), and
// d_j = L_jj (real).  One CTA per chain.
struct CholArgs {
  cplx* W;        // n x n Hermitian (input, FP64), destroyed
  dfc* work;      // n x n df32 scratch
  cplx* rinv;     // n x n output
  cplx* d;        // n output (multiplied into when accumulate)
  int* status;
};

__global__ void __launch_bounds__(512) k_chol_inv(const CholArgs* args, int n, int accumulate_d) {
  const CholArgs a = args[blockIdx.x];
  dfc* L = a.work;
  __shared__ float red[34];
  __shared__ dfc s_piv;
  __shared__ int s_bad;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) L[e] = dfc_make(a.W[e]);
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  // right-looking Cholesky on the lower triangle
  for (int j = 0; j < n; ++j) {
    if (threadIdx.x == 0) {
      df ajj = L[j + (size_t)n * j].re;
      if (!(ajj.hi > 0.0f)) {
        s_bad = 1;
        ajj = df{1.0f, 0.0f};
      }
      df lj = df_sqrt(ajj);
      L[j + (size_t)n * j] = dfc{lj, {0.f, 0.f}};
      s_piv = dfc{lj, {0.f, 0.f}};
    }
    __syncthreads();
    const df inv = df_div(df{1.0f, 0.0f}, s_piv.re);
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
      dfc v = L[i + (size_t)n * j];
      L[i + (size_t)n * j] = dfc{df_mul(v.re, inv), df_mul(v.im, inv)};
    }
    __syncthreads();
    // trailing update: L(i,k) -= L(i,j) conj(L(k,j)) for j < k <= i; threads run
    // down the columns (consecutive rows i) so the accesses coalesce
    const int m = n - j - 1;
    for (long e = threadIdx.x; e < (long)m * m; e += blockDim.x) {
      const int ii = (int)(e % m), kk = (int)(e / m);
      if (ii < kk) continue;
      const int i = j + 1 + ii, k = j + 1 + kk;
      const dfc lij = L[i + (size_t)n * j], lkj = L[k + (size_t)n * j];
      L[i + (size_t)n * k] = dfc_sub(L[i + (size_t)n * k], dfc_mul(lij, dfc{lkj.re, df_neg(lkj.im)}));
    }
    __syncthreads();
  }
  // d_j = L_jj
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double v = df_to_d(L[j + (size_t)n * j].re);
    if (accumulate_d) a.d[j] = mk(a.d[j].x * v, 0.0);
    else a.d[j] = mk(v, 0.0);
  }
  // the factor stays in `work`; k_tri_inv forms (L^H)^-1
  if (threadIdx.x == 0 && s_bad) *a.status = 1;
}

// R^-1 for R = L^H (upper triangular) from the double-float Cholesky factor L
// (lower, column-major) left in `work`: one warp per column j solves
// R x = e_j by back substitution, x_i = -(sum_{k=i+1..j} conj(L_ki) x_k) / L_ii,
// reading column i of L (contiguous).  Written to `rinv` in FP64.
constexpr int TRI_WARPS = 8;
__global__ void __launch_bounds__(TRI_WARPS * 32) k_tri_inv(const CholArgs* args, int n) {
  extern __shared__ __align__(16) unsigned char tri_dyn[];
  const CholArgs a = args[blockIdx.y];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * TRI_WARPS + warp;
  if (j >= n) return;
  dfc* x = reinterpret_cast<dfc*>(tri_dyn) + (size_t)warp * n;
  const dfc* L = a.work;
  if (lane == 0) {
    const df d = L[j + (size_t)n * j].re;
    x[j] = dfc{df_div(df{1.f, 0.f}, d), {0.f, 0.f}};
  }
  __syncwarp();
  for (int i = j - 1; i >= 0; --i) {
    const dfc* Li = L + (size_t)n * i;
    dfc acc = dfc_zero();
    for (int k = i + 1 + lane; k <= j; k += 32) acc = dfc_add(acc, dfc_mulc(Li[k], x[k]));
    for (int o = 16; o > 0; o >>= 1) {
      dfc t;
      t.re.hi = __shfl_xor_sync(0xffffffffu, acc.re.hi, o);
      t.re.lo = __shfl_xor_sync(0xffffffffu, acc.re.lo, o);
      t.im.hi = __shfl_xor_sync(0xffffffffu, acc.im.hi, o);
      t.im.lo = __shfl_xor_sync(0xffffffffu, acc.im.lo, o);
      acc = dfc_add(acc, t);
    }
    if (lane == 0) {
      const df d = Li[i].re;   // L_ii, real and positive
      x[i] = dfc{df_neg(df_div(acc.re, d)), df_neg(df_div(acc.im, d))};
    }
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) a.rinv[i + (size_t)n * j] = i <= j ? dfc_to_d(x[i]) : mk(0.0);
}

// The same R^-1 = L^-H, column j per warp, by column-oriented substitution:
// x_k = (delta_kj - s_k) / L_kk for k = j .. 0, then s_m += conj(L_km) x_k
// for every m < k.  Lane l owns the rows m = l (mod 32) (their s_m and x_m
// in registers); row k of L is loaded one step ahead, so the chain of
// dependent steps waits on the arithmetic and one shuffle, not on memory.
// Rows up to 32 * TRI_SLOTS (nelec <= 256).
constexpr int TRI_SLOTS = 8;
__global__ void __launch_bounds__(TRI_WARPS * 32) k_tri_inv_rows(const CholArgs* args, int n) {
  const CholArgs a = args[blockIdx.y];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * TRI_WARPS + warp;
  if (j >= n) return;
  const dfc* L = a.work;
  dfc cur[TRI_SLOTS], nxt[TRI_SLOTS], sx[TRI_SLOTS];
  df dcur = {1.f, 0.f}, dnxt = {1.f, 0.f};
#pragma unroll
  for (int t = 0; t < TRI_SLOTS; ++t) {
    const int m = lane + 32 * t;
    sx[t] = dfc_zero();
    cur[t] = m < j ? L[j + (size_t)n * m] : dfc_zero();
  }
  if (lane == (j & 31)) dcur = L[j + (size_t)n * j].re;
  for (int k = j; k >= 0; --k) {
    // row k-1 and its diagonal entry, ahead of need
#pragma unroll
    for (int t = 0; t < TRI_SLOTS; ++t) {
      const int m = lane + 32 * t;
      nxt[t] = m < k - 1 ? L[(k - 1) + (size_t)n * m] : dfc_zero();
    }
    if (k >= 1 && lane == ((k - 1) & 31)) dnxt = L[(k - 1) + (size_t)n * (k - 1)].re;
    // x_k by its owner lane (the others compute a discarded value), broadcast
    dfc sk = dfc_zero();
#pragma unroll
    for (int t = 0; t < TRI_SLOTS; ++t) sk = (lane + 32 * t == k) ? sx[t] : sk;
    const df inv = df_div(df{1.f, 0.f}, dcur);
    const dfc v = dfc_sub(k == j ? dfc{{1.f, 0.f}, {0.f, 0.f}} : dfc_zero(), sk);
    dfc xk = dfc{df_mul(v.re, inv), df_mul(v.im, inv)};
#pragma unroll
    for (int t = 0; t < TRI_SLOTS; ++t) sx[t] = (lane + 32 * t == k) ? xk : sx[t];
    const int src = k & 31;
    xk.re.hi = __shfl_sync(0xffffffffu, xk.re.hi, src);
    xk.re.lo = __shfl_sync(0xffffffffu, xk.re.lo, src);
    xk.im.hi = __shfl_sync(0xffffffffu, xk.im.hi, src);
    xk.im.lo = __shfl_sync(0xffffffffu, xk.im.lo, src);
    // s_m += conj(L_km) x_k for the rows m < k this lane owns
#pragma unroll
    for (int t = 0; t < TRI_SLOTS; ++t)
      if (lane + 32 * t < k) sx[t] = dfc_add(sx[t], dfc_mulc(cur[t], xk));
#pragma unroll
    for (int t = 0; t < TRI_SLOTS; ++t) cur[t] = nxt[t];
    dcur = dnxt;
  }
#pragma unroll
  for (int t = 0; t < TRI_SLOTS; ++t) {
    const int m = lane + 32 * t;
    if (m < n) a.rinv[m + (size_t)n * j] = m <= j ? dfc_to_d(sx[t]) : mk(0.0);
  }
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inverse in place with partial pivoting (df32 scratch), FP64
// log det from the pivots (zgetrf/zdet conventions: product of pivots, sign
// of the row interchanges).  One CTA per chain.
struct GJArgs {
  cplx* M;        // n x n in/out (FP64)
  dfc* work;      // n x n df32 scratch
  cplx* logdet;   // out
  cplx* piv;      // n scratch (FP64 pivots)
  int* perm;      // n scratch
  int* status;
};

__global__ void __launch_bounds__(512) k_gj_inverse(const GJArgs* args, int n) {
  const GJArgs a = args[blockIdx.x];
  dfc* A = a.work;
  __shared__ float sv[512];
  __shared__ int si[512];
  __shared__ int s_p;
  __shared__ dfc s_rec;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = dfc_make(a.M[e]);
  __syncthreads();
  int nswap = 0;
  for (int k = 0; k < n; ++k) {
    float best = -1.f;
    int bi = k;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      dfc v = A[i + (size_t)n * k];
      float m = fabsf(v.re.hi) + fabsf(v.im.hi);
      if (m > best) { best = m; bi = i; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        float ov = sv[threadIdx.x + s];
        int oi = si[threadIdx.x + s];
        if (ov > sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x])) {
          sv[threadIdx.x] = ov;
          si[threadIdx.x] = oi;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) s_p = si[0];
    __syncthreads();
    const int p = s_p;
    if (p != k) {
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        dfc t = A[k + (size_t)n * j];
        A[k + (size_t)n * j] = A[p + (size_t)n * j];
        A[p + (size_t)n * j] = t;
      }
      ++nswap;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      dfc pv = A[k + (size_t)n * k];
      a.piv[k] = dfc_to_d(pv);
      a.perm[k] = p;
      // 1/pv = conj(pv)/|pv|^2
      df nrm = df_add(df_mul(pv.re, pv.re), df_mul(pv.im, pv.im));
      if (nrm.hi == 0.0f) *a.status = 1;
      df inv = df_div(df{1.f, 0.f}, nrm.hi == 0.0f ? df{1.f, 0.f} : nrm);
      s_rec = dfc{df_mul(pv.re, inv), df_neg(df_mul(pv.im, inv))};
      A[k + (size_t)n * k] = dfc{{1.f, 0.f}, {0.f, 0.f}};
    }
    __syncthreads();
    const dfc rec = s_rec;
    for (int j = threadIdx.x; j < n; j += blockDim.x) A[k + (size_t)n * j] = dfc_mul(A[k + (size_t)n * j], rec);
    __syncthreads();
    // eliminate column k from every other row
    for (long e = threadIdx.x; e < (long)n * n; e += blockDim.x) {
      int i = (int)(e % n), j = (int)(e / n);
      if (i == k) continue;
      dfc f = A[i + (size_t)n * k];
      if (j == k) continue;
      A[i + (size_t)n * j] = dfc_sub(A[i + (size_t)n * j], dfc_mul(f, A[k + (size_t)n * j]));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      if (i == k) continue;
      dfc f = A[i + (size_t)n * k];
      A[i + (size_t)n * k] = dfc_sub(dfc_zero(), dfc_mul(f, A[k + (size_t)n * k]));
    }
    __syncthreads();
  }
  // undo the column interchanges in reverse order
  for (int k = n - 1; k >= 0; --k) {
    int p = a.perm[k];
    if (p != k)
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        dfc t = A[i + (size_t)n * k];
        A[i + (size_t)n * k] = A[i + (size_t)n * p];
        A[i + (size_t)n * p] = t;
      }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) a.M[e] = dfc_to_d(A[e]);
  // log det = sum log(piv) + i pi (#swaps odd)
  __shared__ double rre[512], rim[512];
  double sr = 0.0, sim = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    cplx l = clog_(a.piv[i]);
    sr += l.x;
    sim += l.y;
  }
  rre[threadIdx.x] = sr;
  rim[threadIdx.x] = sim;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rre[threadIdx.x] += rre[threadIdx.x + s];
      rim[threadIdx.x] += rim[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *a.logdet = mk(rre[0], rim[0] + ((nswap & 1) ? 3.14159265358979323846 : 0.0));
}

// ---------------------------------------------------------------------------
// One-way propagation in df32 (the columns of X live in shared memory as
// df32); forward: X(S,:) <- E X(S,:), backward (adjoint): X(S,:) <- E^H X(S,:)
struct PropArgs {
  DevModel M;
  cplx* X;
  const cplx* expkv;
};

// expKV of the nt slices of one propagation converted once to double-float,
// in application order and already transposed-conjugated for the backward
// direction: ekv[((it * n_pf + f) * max_pla + p) * 16 + r + 4 k] = M(r, k)
// with M = expKV (forward) or expKV^H (backward).
__global__ void k_ekv_df(const PropArgs* args, dfc* ekv_all, size_t stride, int t_from, int nt, int forward) {
  __shared__ PropArgs sa;
  if (threadIdx.x == 0) sa = args[blockIdx.y];
  __syncthreads();
  const DevModel& M = sa.M;
  dfc* out = ekv_all + stride * blockIdx.y;
  const long total = (long)nt * M.n_pf * M.max_pla * 16;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int k16 = (int)(e % 16);
    long rest = e / 16;
    const int p = (int)(rest % M.max_pla);
    rest /= M.max_pla;
    const int f = (int)(rest % M.n_pf);
    const int it = (int)(rest / M.n_pf);
    const int pf = forward ? f : M.n_pf - 1 - f;
    const int t = (forward ? t_from + it : t_from - it) - 1;
    const int dim = M.pf_dim[pf], r = k16 % 4, k = k16 / 4;
    dfc v = dfc_zero();
    if (p < M.pf_npla[pf] && r < dim && k < dim) {
      const cplx* E = sa.expkv + M.kv_base(p, pf, t);
      v = dfc_make(forward ? E[r + M.pdim * k] : cconj(E[k + M.pdim * r]));
    }
    out[e] = v;
  }
}

// One-way propagation of PROP_NC columns of X through nt slices (all
// families, application order) in double-float, the columns held in shared
// memory.  Work items are (plaquette, column group): the plaquette's matrix
// stays in registers across the group's columns.
constexpr int PROP_NC = 8, PROP_NCG = 2;

template <int DIM>
__global__ void __launch_bounds__(256) k_bprop_df(const PropArgs* args, const dfc* ekv_all, size_t stride, int n,
                                                  int nt, int forward) {
  __shared__ PropArgs sa;
  extern __shared__ __align__(16) unsigned char dyn[];
  if (threadIdx.x == 0) sa = args[blockIdx.y];
  __syncthreads();
  const DevModel& M = sa.M;
  const int ns = M.ns, pd = M.pdim, npf = M.n_pf, mp = M.max_pla;
  dfc* col = reinterpret_cast<dfc*>(dyn);                               // [PROP_NC][ns]
  int* s_site = reinterpret_cast<int*>(col + (size_t)PROP_NC * ns);     // [n_pf][max_pla][4]
  const int c0 = blockIdx.x * PROP_NC, ncol = min(PROP_NC, n - c0);
  cplx* X = sa.X + (size_t)ns * c0;
  for (int e = threadIdx.x; e < ncol * ns; e += blockDim.x) col[e] = dfc_make(X[e]);
  for (int e = threadIdx.x; e < npf * mp * 4; e += blockDim.x) {
    const int k = e % 4, p = (e / 4) % mp, pf = e / (4 * mp);
    s_site[e] = (p < M.pf_npla[pf] && k < M.pf_dim[pf]) ? M.site[k + pd * (p + mp * pf)] : 0;
  }
  __syncthreads();
  const dfc* ekv = ekv_all + stride * blockIdx.y;
  constexpr int CPG = PROP_NC / PROP_NCG;
  for (int it = 0; it < nt; ++it) {
    for (int f = 0; f < npf; ++f) {
      const int pf = forward ? f : npf - 1 - f;
      const int npla = M.pf_npla[pf], dim = M.pf_dim[pf];
      const dfc* Ef = ekv + ((size_t)it * npf + f) * mp * 16;
      for (int item = threadIdx.x; item < npla * PROP_NCG; item += blockDim.x) {
        const int p = item % npla, cg = item / npla;
        dfc e[DIM][DIM];
        int S[DIM];
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
          S[r] = s_site[(pf * mp + p) * 4 + r];
#pragma unroll
          for (int k = 0; k < DIM; ++k) e[r][k] = Ef[(size_t)p * 16 + r + 4 * k];
        }
#pragma unroll
        for (int j = 0; j < CPG; ++j) {
          const int c = cg * CPG + j;
          if (c >= ncol) break;
          dfc* x = col + (size_t)c * ns;
          dfc v[DIM];
#pragma unroll
          for (int k = 0; k < DIM; ++k) v[k] = k < dim ? x[S[k]] : dfc_zero();
#pragma unroll
          for (int r = 0; r < DIM; ++r) {
            if (r >= dim) break;
            // compensated dot product of the plaquette row with the column (Dot2)
            d2acc ar{0.f, 0.f}, ai{0.f, 0.f};
#pragma unroll
            for (int k = 0; k < DIM; ++k) {
              const dfc& ek = e[r][k];
              dot2_mac(ar, ek.re.hi, ek.re.lo, v[k].re.hi, v[k].re.lo);
              dot2_mac(ar, -ek.im.hi, -ek.im.lo, v[k].im.hi, v[k].im.lo);
              dot2_mac(ai, ek.re.hi, ek.re.lo, v[k].im.hi, v[k].im.lo);
              dot2_mac(ai, ek.im.hi, ek.im.lo, v[k].re.hi, v[k].re.lo);
            }
            x[S[r]] = dfc{quick_two_sum(ar.h, ar.l), quick_two_sum(ai.h, ai.l)};
          }
        }
      }
      __syncthreads();
    }
  }
  for (int e = threadIdx.x; e < ncol * ns; e += blockDim.x) X[e] = dfc_to_d(col[e]);
}

__host__ __forceinline__ size_t prop_smem(int ns, int n_pf, int max_pla) {
  return sizeof(dfc) * (size_t)PROP_NC * ns + sizeof(int) * 4 * (size_t)n_pf * max_pla;
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inverse with partial pivoting in double-float on a cluster of
// GJ_CL thread blocks per matrix: each block keeps a slab of columns in its
// shared memory; at pivot step k the block owning column k picks the pivot,
// and writes the pivot row index, 1/pivot and the multiplier column into
// every block of the cluster through distributed shared memory.  Same
// result layout as k_gj_inverse (inverse in place in M, log det, pivots).
constexpr int GJ_CL = 4;
constexpr int GJ_MAXN = 512;
namespace cgx = cooperative_groups;

__global__ void __cluster_dims__(GJ_CL, 1, 1) __launch_bounds__(256) k_gj_cluster(const GJArgs* args, int n) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char gj_dyn[];
  // multipliers, pivot row and reciprocal pivot of step k in buffer k&1
  // (written by the owner block into every block; double-buffered so that
  // one cluster barrier per step suffices)
  __shared__ dfc s_f[2][GJ_MAXN];
  __shared__ int s_p[2];
  __shared__ dfc s_rec[2];
  __shared__ int s_perm[GJ_MAXN];
  __shared__ float s_bv[32];
  __shared__ int s_bi[32];
  const int rank = (int)cl.block_rank();
  const GJArgs a = args[blockIdx.x / GJ_CL];
  const int w = (n + GJ_CL - 1) / GJ_CL, c_lo = rank * w, c_hi = min(n, c_lo + w), nc = max(0, c_hi - c_lo);
  dfc* A = reinterpret_cast<dfc*>(gj_dyn);   // [nc][n] local slab, A[i + n*(j - c_lo)]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int jl = warp; jl < nc; jl += nw)
    for (int i = lane; i < n; i += 32) A[(size_t)n * jl + i] = dfc_make(a.M[(size_t)(c_lo + jl) * n + i]);
  __syncthreads();
  cl.sync();   // every block of the cluster runs before its shared memory is written
  int nswap = 0;
  for (int k = 0; k < n; ++k) {
    const int buf = k & 1;
    if (k / w == rank) {
      // column k is current: this block finished its elimination of step k-1
      const dfc* col = A + (size_t)n * (k - c_lo);
      float best = -1.f;
      int bi = k;
      for (int i = k + tid; i < n; i += blockDim.x) {
        const float m = fabsf(col[i].re.hi) + fabsf(col[i].im.hi);
        if (m > best) { best = m; bi = i; }
      }
      // largest magnitude, smallest row on ties: within each warp, then over warps
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) {
        s_bv[warp] = best;
        s_bi[warp] = bi;
      }
      __syncthreads();
      if (warp == 0) {
        best = lane < nw ? s_bv[lane] : -2.f;
        bi = lane < nw ? s_bi[lane] : n;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) s_bi[0] = bi;
      }
      __syncthreads();
      const int p = s_bi[0];
      const dfc pv = col[p];
      df nrm = df_add(df_mul(pv.re, pv.re), df_mul(pv.im, pv.im));
      if (tid == 0) {
        if (nrm.hi == 0.0f) *a.status = 1;
        a.piv[k] = dfc_to_d(pv);
      }
      const df inv = df_div(df{1.f, 0.f}, nrm.hi == 0.0f ? df{1.f, 0.f} : nrm);
      const dfc rec = dfc{df_mul(pv.re, inv), df_neg(df_mul(pv.im, inv))};
      // multipliers f_i = A(sigma(i), k) with rows k and p exchanged
      for (int i = tid; i < n; i += blockDim.x) {
        const dfc v = col[(i == k) ? p : ((i == p) ? k : i)];
#pragma unroll
        for (int r = 0; r < GJ_CL; ++r) cl.map_shared_rank(&s_f[buf][0], r)[i] = v;
      }
      if (tid < GJ_CL) {
        *cl.map_shared_rank(&s_p[buf], tid) = p;
        *cl.map_shared_rank(&s_rec[buf], tid) = rec;
      }
    }
    cl.sync();
    const int p = s_p[buf];
    const dfc rec = s_rec[buf];
    const dfc* f = s_f[buf];
    if (tid == 0) s_perm[k] = p;
    if (p != k) ++nswap;
    // exchange rows k and p, scale row k, eliminate, in this block's columns
    for (int jl = tid; jl < nc; jl += blockDim.x) {
      dfc* cj = A + (size_t)n * jl;
      if (p != k) {
        const dfc t = cj[k];
        cj[k] = cj[p];
        cj[p] = t;
      }
      cj[k] = (c_lo + jl == k) ? rec : dfc_mul(cj[k], rec);
    }
    __syncthreads();
    for (int jl = warp; jl < nc; jl += nw) {
      dfc* cj = A + (size_t)n * jl;
      const dfc ck = cj[k];
      if (c_lo + jl == k) {
        for (int i = lane; i < n; i += 32)
          if (i != k) cj[i] = dfc_sub(dfc_zero(), dfc_mul(f[i], rec));
      } else {
        for (int i = lane; i < n; i += 32)
          if (i != k) cj[i] = dfc_fms(cj[i], f[i], ck);
      }
    }
    __syncthreads();   // this block's next pivot column is current
  }
  // undo the row exchanges as column exchanges: computed column c ends at pos(c)
  __shared__ int s_at[GJ_MAXN];
  if (tid == 0) {
    for (int q = 0; q < n; ++q) s_at[q] = q;
    for (int k = n - 1; k >= 0; --k) {
      const int p = s_perm[k];
      const int t = s_at[k];
      s_at[k] = s_at[p];
      s_at[p] = t;
    }
  }
  __syncthreads();
  // s_at[q] = computed column found at final position q; write this block's columns there
  for (int q = 0; q < n; ++q) {
    const int c = s_at[q];
    if (c < c_lo || c >= c_hi) continue;
    const dfc* cj = A + (size_t)n * (c - c_lo);
    for (int i = tid; i < n; i += blockDim.x) a.M[(size_t)q * n + i] = dfc_to_d(cj[i]);
  }
  if (rank == 0) {
    // log det = sum log(piv) + i pi (odd number of exchanges)
    __shared__ double rre[256], rim[256];
    double sr = 0.0, sim = 0.0;
    for (int i = tid; i < n; i += blockDim.x) {
      const cplx l = clog_(a.piv[i]);
      sr += l.x;
      sim += l.y;
    }
    rre[tid] = sr;
    rim[tid] = sim;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (tid < st) {
        rre[tid] += rre[tid + st];
        rim[tid] += rim[tid + st];
      }
      __syncthreads();
    }
    if (tid == 0) *a.logdet = mk(rre[0], rim[0] + ((nswap & 1) ? 3.14159265358979323846 : 0.0));
  }
}

// Cholesky W = L L^H in double-float on a cluster of GJ_CL blocks.  Column
// k lives in block k % GJ_CL (cyclic, so every block has about the same
// share of each trailing update), local slot k / GJ_CL, in shared memory.
// Right-looking, one cluster barrier per column: the block owning column j
// forms L(:,j) (its column is final once its own update by column j-1 has
// finished) and writes it into buffer j&1 of every block; after the barrier
// each block updates its own trailing columns, a warp per column and a lane
// per row.  The writer of buffer (j+1)&1 can only have passed barrier j, by
// which every block has finished reading that buffer for column j-1.  The
// factor goes to `work` for k_tri_inv and d_j = L_jj to `d` (multiplied in
// when accumulate_d).
__global__ void __cluster_dims__(GJ_CL, 1, 1) __launch_bounds__(256) k_chol_cluster(const CholArgs* args, int n,
                                                                                      int accumulate_d) {
  cgx::cluster_group cl = cgx::this_cluster();
  extern __shared__ __align__(16) unsigned char ch_dyn[];
  __shared__ dfc s_f[2][GJ_MAXN];   // L(:,j) of the current column, double-buffered
  __shared__ int s_bad;
  __shared__ df s_l;
  const int rank = (int)cl.block_rank();
  const CholArgs a = args[blockIdx.x / GJ_CL];
  const int nc = (n - rank + GJ_CL - 1) / GJ_CL;   // columns rank, rank + GJ_CL, ...
  dfc* A = reinterpret_cast<dfc*>(ch_dyn);         // [nc][n]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int kl = warp; kl < nc; kl += nw) {
    const cplx* src = a.W + (size_t)(rank + GJ_CL * kl) * n;
    for (int i = lane; i < n; i += 32) A[(size_t)n * kl + i] = dfc_make(src[i]);
  }
  if (tid == 0) s_bad = 0;
  cl.sync();   // every block of the cluster runs before its shared memory is written
  for (int j = 0; j < n; ++j) {
    const int buf = j & 1;
    if (j % GJ_CL == rank) {
      dfc* col = A + (size_t)n * (j / GJ_CL);
      if (tid == 0) {
        df ajj = col[j].re;
        if (!(ajj.hi > 0.0f)) {
          s_bad = 1;
          ajj = df{1.0f, 0.0f};
        }
        s_l = df_sqrt(ajj);
        col[j] = dfc{s_l, {0.f, 0.f}};
      }
      __syncthreads();
      const df inv = df_div(df{1.0f, 0.0f}, s_l);
      for (int i = j + 1 + tid; i < n; i += blockDim.x) {
        const dfc v = dfc{df_mul(col[i].re, inv), df_mul(col[i].im, inv)};
        col[i] = v;
#pragma unroll
        for (int r = 0; r < GJ_CL; ++r) cl.map_shared_rank(&s_f[buf][0], r)[i] = v;
      }
    }
    cl.sync();
    // L(i,k) -= L(i,j) conj(L(k,j)) for j < k <= i, k in this block's columns
    const int kl0 = j < rank ? 0 : (j - rank) / GJ_CL + 1;
    const dfc* f = s_f[buf];
    for (int kl = kl0 + warp; kl < nc; kl += nw) {
      const int k = rank + GJ_CL * kl;
      const dfc lkj = f[k];
      const dfc ckj = dfc{lkj.re, df_neg(lkj.im)};
      dfc* col = A + (size_t)n * kl;
      for (int i = k + lane; i < n; i += 32) col[i] = dfc_fms(col[i], f[i], ckj);
    }
    __syncthreads();   // this block's next pivot column is final
  }
  for (int kl = tid; kl < nc; kl += blockDim.x) {
    const int j = rank + GJ_CL * kl;
    const double v = df_to_d(A[(size_t)n * kl + j].re);
    a.d[j] = accumulate_d ? mk(a.d[j].x * v, 0.0) : mk(v, 0.0);
  }
  for (int kl = warp; kl < nc; kl += nw) {
    dfc* dst = a.work + (size_t)(rank + GJ_CL * kl) * n;
    for (int i = lane; i < n; i += 32) dst[i] = A[(size_t)n * kl + i];
  }
  if (tid == 0 && s_bad) *a.status = 1;
}

// ---------------------------------------------------------------------------
// Final weight and error per chain: ln_cw = branch((logdet + sum log D) TR ncopy)
struct WeightArgs {
  DevScalars* sc;
  const cplx* d_block;    // the D block rewritten by this recompute (nelec)
  cplx* d_logsum;         // (nblock) per-block sum of log D
  int blk0;               // its 0-based index
  int nblock;
  const cplx* logdet;
  const cplx* gold;
  const cplx* gnew;
  int tr_weight, ncopy;
  int gdf;   // gold and gnew are in the double-float float4 form
};

__global__ void k_bweight(const WeightArgs* args, int ndcount, long ng, int compare) {
  const WeightArgs a = args[blockIdx.x];
  __shared__ double rre[256], rim[256], rmx[256], rdf[256], rgn[256];
  double sr = 0.0, sim = 0.0, mx = 0.0, df = 0.0, gn = 0.0;
  for (int i = threadIdx.x; i < ndcount; i += blockDim.x) {
    cplx l = clog_(a.d_block[i]);
    sr += l.x;
    sim += l.y;
  }
  if (compare && a.gdf) {
    // differences of double-float values in FP32: hi and lo parts separately
    const float4* go = reinterpret_cast<const float4*>(a.gold);
    const float4* gw = reinterpret_cast<const float4*>(a.gnew);
    float mxf = 0.f, dff = 0.f, gnf = 0.f;
    for (long e = threadIdx.x; e < ng; e += blockDim.x) {
      const float4 o = go[e], w = gw[e];
      const float dr = (o.x - w.x) + (o.z - w.z), di = (o.y - w.y) + (o.w - w.w);
      const float nr = w.x + w.z, ni = w.y + w.w;
      const float d2 = dr * dr + di * di;
      mxf = fmaxf(mxf, d2);
      dff += d2;
      gnf += nr * nr + ni * ni;
    }
    mx = sqrt((double)mxf);
    df = dff;
    gn = gnf;
  } else if (compare) {
    for (long e = threadIdx.x; e < ng; e += blockDim.x) {
      const cplx gnew = a.gnew[e], dg = csub(a.gold[e], gnew);
      mx = fmax(mx, cabsd(dg));
      df += cabs2(dg);
      gn += cabs2(gnew);
    }
  }
  rre[threadIdx.x] = sr;
  rim[threadIdx.x] = sim;
  rmx[threadIdx.x] = mx;
  rdf[threadIdx.x] = df;
  rgn[threadIdx.x] = gn;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rre[threadIdx.x] += rre[threadIdx.x + s];
      rim[threadIdx.x] += rim[threadIdx.x + s];
      rmx[threadIdx.x] = fmax(rmx[threadIdx.x], rmx[threadIdx.x + s]);
      rdf[threadIdx.x] += rdf[threadIdx.x + s];
      rgn[threadIdx.x] += rgn[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.d_logsum[a.blk0] = mk(rre[0], rim[0]);
    cplx sumd = mk(0.0);
    for (int b = 0; b < a.nblock; ++b) sumd = cadd(sumd, a.d_logsum[b]);
    cplx l = cadd(*a.logdet, sumd);
    if (a.tr_weight) l = cadd(l, cconj(l));
    l = cscale(l, (double)a.ncopy);
    const double two_pi_sp = (double)(2.0f * 3.14159265358979323846f);
    cplx nw = mk(l.x, fmod(l.y, two_pi_sp));
    if (compare) {
      double ew = fabs(nw.x - a.sc->ln_cw.x);
      a.sc->err_g = rmx[0];
      const double rel = rgn[0] > 0.0 ? sqrt(rdf[0] / rgn[0]) : 0.0;
      a.sc->err_g_rel = rel;
      if (rel > a.sc->err_g_rel_max) a.sc->err_g_rel_max = rel;
      a.sc->err_w = ew;
      a.sc->err_fast = ew;
      double m = fmax(rmx[0], ew);
      if (m > a.sc->err_fast_max) a.sc->err_fast_max = m;
    }
    a.sc->ln_cw = nw;
  }
}

// ---------------------------------------------------------------------------
BatchRecompute::~BatchRecompute() {
  void* ps[] = {d_gemm, d_chol, d_gj, d_prop, d_weight, work_df, tmpX, gram, rinv, pbp, wmat, logdet, piv, perm,
                status, ekv_df, d_conv, split_a, split_b, d_og, og_img};
  for (void* p : ps)
    if (p) cudaFree(p);
}

int BatchRecompute::setup(const std::vector<pqmc_chain*>& chains, cudaStream_t s) {
  stream = s;
  C = (int)chains.size();
  pqmc_chain* c0 = chains[0];
  ns = c0->ns;
  ne = c0->nelec;
  cs = chains;
  auto al = [](void** p, size_t b) -> int {
    PQMC_CUDA(cudaMalloc(p, b));
    return PQMC_OK;
  };
  PQMC_TRY(al((void**)&d_gemm, sizeof(GemmArgs) * C * 8));
  PQMC_TRY(al((void**)&d_conv, sizeof(ConvArgs) * C * 2 * 8));
  PQMC_TRY(al((void**)&split_a, sizeof(float4) * (size_t)C * ns * ne));   // every operand fits in ns x ne
  PQMC_TRY(al((void**)&split_b, sizeof(float4) * (size_t)C * ns * ne));
  PQMC_TRY(al((void**)&d_chol, sizeof(CholArgs) * C));
  PQMC_TRY(al((void**)&d_gj, sizeof(GJArgs) * C * 2));
  PQMC_TRY(al((void**)&d_prop, sizeof(PropArgs) * C * 2));
  PQMC_TRY(al((void**)&d_weight, sizeof(WeightArgs) * C));
  PQMC_TRY(al((void**)&work_df, sizeof(dfc) * (size_t)C * ne * ne));
  PQMC_TRY(al((void**)&tmpX, sizeof(cplx) * (size_t)C * ns * ne));
  PQMC_TRY(al((void**)&gram, sizeof(cplx) * (size_t)C * ne * ne));
  PQMC_TRY(al((void**)&rinv, sizeof(cplx) * (size_t)C * ne * ne));
  PQMC_TRY(al((void**)&pbp, sizeof(cplx) * (size_t)C * ne * ne));
  PQMC_TRY(al((void**)&wmat, sizeof(cplx) * (size_t)C * ns * ne));
  PQMC_TRY(al((void**)&logdet, sizeof(cplx) * C));
  PQMC_TRY(al((void**)&piv, sizeof(cplx) * (size_t)C * ne));
  PQMC_TRY(al((void**)&perm, sizeof(int) * (size_t)C * ne));
  PQMC_TRY(al((void**)&status, sizeof(int) * C));
  PQMC_CUDA(cudaMemset(status, 0, sizeof(int) * C));
  ekv_slices = c0->ngroup;
  ekv_stride = (size_t)ekv_slices * c0->n_pf * c0->max_pla * 16;
  PQMC_TRY(al((void**)&ekv_df, sizeof(dfc) * ekv_stride * C));
  {
    const size_t smem = prop_smem(ns, c0->n_pf, c0->max_pla);
    int dev = 0, optin = 0;
    PQMC_CUDA(cudaGetDevice(&dev));
    PQMC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem + 1024 > (size_t)optin) {
      set_error("batch recompute: %zu bytes of shared memory needed for the propagation", smem);
      return PQMC_ERR_ARG;
    }
    PQMC_CUDA(raise_dyn_smem(k_bprop_df<1>, (int)smem));
    PQMC_CUDA(raise_dyn_smem(k_bprop_df<2>, (int)smem));
    PQMC_CUDA(raise_dyn_smem(k_bprop_df<3>, (int)smem));
    PQMC_CUDA(raise_dyn_smem(k_bprop_df<4>, (int)smem));
    const size_t tsm = sizeof(dfc) * TRI_WARPS * (size_t)ne;
    if (tsm + 1024 > (size_t)optin) {
      set_error("batch recompute: nelec %d too large for the triangular inverse", ne);
      return PQMC_ERR_ARG;
    }
    PQMC_CUDA(raise_dyn_smem(k_tri_inv, (int)tsm));
    // the cluster Gauss-Jordan needs a quarter of the matrix per block in shared memory
    const size_t gsm = sizeof(dfc) * (size_t)((ne + GJ_CL - 1) / GJ_CL) * ne;
    gj_cluster = ne <= GJ_MAXN && gsm + 32768 <= (size_t)optin;   // plus the static shared memory
    if (gj_cluster) {
      PQMC_CUDA(raise_dyn_smem(k_gj_cluster, (int)gsm));
      PQMC_CUDA(raise_dyn_smem(k_chol_cluster, (int)gsm));
    }
  }
  // the GEMM engine: the tensor cores unless PQMC_RECOMPUTE_GEMM=0
  const char* ev = getenv("PQMC_RECOMPUTE_GEMM");
  return set_engine(ev && ev[0] == '0' ? 0 : 1);
}

static inline cplx* qblk(pqmc_chain* c, int b1) { return c->q_string + (size_t)c->ns * c->nelec * (b1 - 1); }
static inline cplx* dblk(pqmc_chain* c, int b1) { return c->d_string + (size_t)c->nelec * (b1 - 1); }

int BatchRecompute::set_engine(int e) {
  if (e != 0 && e != 1) {
    set_error("recompute GEMM engine: 0 (double-float, FP32 pipe) or 1 (Ozaki, tensor cores)");
    return PQMC_ERR_ARG;
  }
  if (e == 1 && !og_img) {
    PQMC_TRY(ozgemm_setup());
    og_stride = ozgemm_img_bytes(ns, ns);   // the largest product: ns x ns
    PQMC_CUDA(cudaMalloc((void**)&og_img, og_stride * C));
    PQMC_CUDA(cudaMalloc((void**)&d_og, sizeof(OgDesc) * C * 8));
  }
  engine = e;
  return PQMC_OK;
}

int BatchRecompute::gemm(char ta, char tb, int m, int n, int k, const std::vector<GemmArgs>& a, int slot,
                         int accumulate) {
  if (engine == 1 && !accumulate) {
    std::vector<OgDesc> od(C);
    for (int i = 0; i < C; ++i)
      od[i] = OgDesc{a[i].A, a[i].B, reinterpret_cast<float4*>(a[i].C), og_img + og_stride * i, err};
    OgDesc* dd = d_og + (size_t)slot * C;
    PQMC_CUDA(cudaMemcpyAsync(dd, od.data(), sizeof(OgDesc) * C, cudaMemcpyHostToDevice, stream));
    return ozgemm_batched(stream, ta, tb, m, n, k, a[0].lda, a[0].ldb, a[0].ldc, dd, C, a[0].out_df ? 0 : 1);
  }
  // split A and B of every chain into double-float once (B shares A's split
  // when they are the same matrix, as in the Gram matrix X^H X)
  const long na = (long)a[0].lda * (ta == 'C' ? m : k), nb = (long)a[0].ldb * (tb == 'C' ? k : n);
  const long cap = (long)ns * ne;
  std::vector<GemmArgs> g(a);
  std::vector<ConvArgs> cv;
  cv.reserve(2 * C);
  if (na <= cap && nb <= cap) {
    for (int i = 0; i < C; ++i) {
      float4* da = split_a + (size_t)i * cap;
      float4* db = split_b + (size_t)i * cap;
      cv.push_back(ConvArgs{a[i].A, da, na});
      g[i].Adf = da;
      if (a[i].B == a[i].A && na == nb) {
        g[i].Bdf = da;
      } else {
        cv.push_back(ConvArgs{a[i].B, db, nb});
        g[i].Bdf = db;
      }
    }
    ConvArgs* dc = d_conv + (size_t)slot * 2 * C;
    PQMC_CUDA(cudaMemcpyAsync(dc, cv.data(), sizeof(ConvArgs) * cv.size(), cudaMemcpyHostToDevice, stream));
    const long mx = std::max(na, nb);
    k_gemm_split<<<dim3((unsigned)std::min<long>((mx + 255) / 256, 256), (unsigned)cv.size()), 256, 0, stream>>>(dc);
    PQMC_LAUNCHED();
  }
  PQMC_CUDA(cudaMemcpyAsync(d_gemm + slot * C, g.data(), sizeof(GemmArgs) * C, cudaMemcpyHostToDevice, stream));
  return dfgemm_batched(stream, ta, tb, m, n, k, d_gemm + slot * C, C, accumulate);
}

// CholeskyQR2 of X_c (ns x ne) in place; d_c = |diag R|
int BatchRecompute::cholqr2(const std::vector<cplx*>& X, const std::vector<cplx*>& D) {
  std::vector<GemmArgs> ga(C);
  std::vector<CholArgs> ca(C);
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < C; ++i) ga[i] = GemmArgs{X[i], X[i], gram + (size_t)i * ne * ne, ns, ns, ne, 0, 1};
    PQMC_TRY(gemm('C', 'N', ne, ne, ns, ga, 0, 0));
    for (int i = 0; i < C; ++i)
      ca[i] = CholArgs{gram + (size_t)i * ne * ne, work_df + (size_t)i * ne * ne, rinv + (size_t)i * ne * ne, D[i],
                       status + i};
    PQMC_CUDA(cudaMemcpyAsync(d_chol, ca.data(), sizeof(CholArgs) * C, cudaMemcpyHostToDevice, stream));
    if (gj_cluster) {
      const int w = (ne + GJ_CL - 1) / GJ_CL;
      k_chol_cluster<<<C * GJ_CL, 256, sizeof(dfc) * (size_t)w * ne, stream>>>(d_chol, ne, pass);
    } else {
      k_chol_inv<<<C, 512, 0, stream>>>(d_chol, ne, pass);
    }
    PQMC_LAUNCHED();
    if (ne <= 32 * TRI_SLOTS)
      k_tri_inv_rows<<<dim3((ne + TRI_WARPS - 1) / TRI_WARPS, C), TRI_WARPS * 32, 0, stream>>>(d_chol, ne);
    else
      k_tri_inv<<<dim3((ne + TRI_WARPS - 1) / TRI_WARPS, C), TRI_WARPS * 32, sizeof(dfc) * TRI_WARPS * ne, stream>>>(
          d_chol, ne);
    PQMC_LAUNCHED();
    for (int i = 0; i < C; ++i)
      ga[i] = GemmArgs{X[i], rinv + (size_t)i * ne * ne, tmpX + (size_t)i * ns * ne, ns, ne, ns, 0, 2};
    PQMC_TRY(gemm('N', 'N', ns, ne, ne, ga, 1, 0));
    for (int i = 0; i < C; ++i)
      PQMC_CUDA(cudaMemcpyAsync(X[i], tmpX + (size_t)i * ns * ne, sizeof(cplx) * (size_t)ns * ne,
                                cudaMemcpyDeviceToDevice, stream));
  }
  return PQMC_OK;
}

// G = R (L R)^-1 L with L = XL^H; ln_cw; errors (cal_g_and_det_T0)
int BatchRecompute::g_and_det(const std::vector<cplx*>& XL, const std::vector<cplx*>& R,
                              const std::vector<cplx*>& Gcur, const std::vector<cplx*>& Gnew, bool compare, int blk1,
                              bool g_df) {
  std::vector<GemmArgs> ga(C);
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{XL[i], R[i], pbp + (size_t)i * ne * ne, ns, ns, ne};
  PQMC_TRY(gemm('C', 'N', ne, ne, ns, ga, 2, 0));
  std::vector<GJArgs> gj(C);
  for (int i = 0; i < C; ++i)
    gj[i] = GJArgs{pbp + (size_t)i * ne * ne, work_df + (size_t)i * ne * ne, logdet + i, piv + (size_t)i * ne,
                   perm + (size_t)i * ne, status + i};
  PQMC_CUDA(cudaMemcpyAsync(d_gj, gj.data(), sizeof(GJArgs) * C, cudaMemcpyHostToDevice, stream));
  if (gj_cluster) {
    const int w = (ne + GJ_CL - 1) / GJ_CL;
    k_gj_cluster<<<C * GJ_CL, 256, sizeof(dfc) * (size_t)w * ne, stream>>>(d_gj, ne);
  } else {
    k_gj_inverse<<<C, 512, 0, stream>>>(d_gj, ne);
  }
  PQMC_LAUNCHED();
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{R[i], pbp + (size_t)i * ne * ne, wmat + (size_t)i * ns * ne, ns, ne, ns};
  PQMC_TRY(gemm('N', 'N', ns, ne, ne, ga, 3, 0));
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{wmat + (size_t)i * ns * ne, XL[i], Gnew[i], ns, ns, ns, g_df ? 1 : 0};
  PQMC_TRY(gemm('N', 'C', ns, ns, ne, ga, 4, 0));
  std::vector<WeightArgs> wa(C);
  for (int i = 0; i < C; ++i)
    wa[i] = WeightArgs{cs[i]->sc, dblk(cs[i], blk1), cs[i]->d_logsum, blk1 - 1, cs[i]->nblock, logdet + i, Gcur[i],
                       Gnew[i], cs[i]->M.tr_weight, cs[i]->M.ncopy, g_df ? 1 : 0};
  PQMC_CUDA(cudaMemcpyAsync(d_weight, wa.data(), sizeof(WeightArgs) * C, cudaMemcpyHostToDevice, stream));
  k_bweight<<<C, 256, 0, stream>>>(d_weight, ne, (long)ns * ns, compare ? 1 : 0);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int BatchRecompute::propagate(const std::vector<cplx*>& X, int t_from, int t_to, bool forward) {
  const int nt = forward ? (t_to - t_from + 1) : (t_from - t_to + 1);
  if (nt < 1 || nt > ekv_slices) { set_error("batch propagate: %d slices (at most %d)", nt, ekv_slices); return PQMC_ERR_ARG; }
  std::vector<PropArgs> pa(C);
  for (int i = 0; i < C; ++i) pa[i] = PropArgs{cs[i]->M, X[i], cs[i]->expkv};
  PQMC_CUDA(cudaMemcpyAsync(d_prop, pa.data(), sizeof(PropArgs) * C, cudaMemcpyHostToDevice, stream));
  pqmc_chain* c0 = cs[0];
  const long total = (long)nt * c0->n_pf * c0->max_pla * 16;
  k_ekv_df<<<dim3((unsigned)std::min<long>((total + 255) / 256, 1024), C), 256, 0, stream>>>(d_prop, ekv_df, ekv_stride,
                                                                                         t_from, nt, forward ? 1 : 0);
  PQMC_LAUNCHED();
  int maxdim = 1;
  for (int f = 0; f < c0->n_pf; ++f) maxdim = std::max(maxdim, c0->h_pf_dim[f]);
  const dim3 grid((ne + PROP_NC - 1) / PROP_NC, C);
  const size_t smem = prop_smem(ns, c0->n_pf, c0->max_pla);
  const int fw = forward ? 1 : 0;
  switch (maxdim) {
    case 1: k_bprop_df<1><<<grid, 256, smem, stream>>>(d_prop, ekv_df, ekv_stride, ne, nt, fw); break;
    case 2: k_bprop_df<2><<<grid, 256, smem, stream>>>(d_prop, ekv_df, ekv_stride, ne, nt, fw); break;
    case 3: k_bprop_df<3><<<grid, 256, smem, stream>>>(d_prop, ekv_df, ekv_stride, ne, nt, fw); break;
    default: k_bprop_df<4><<<grid, 256, smem, stream>>>(d_prop, ekv_df, ekv_stride, ne, nt, fw); break;
  }
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// init_g_T0(1) (src/mod_evolution.f90:46-111) for every chain: the right
// string Q(2..nblock-1) from the Slater matrix upward, one block of ngroup
// slices and one CholeskyQR2 at a time for all chains together, then G at
// the top slice from L = P^H and R = Q(nblock-1).
int BatchRecompute::init_g() {
  pqmc_chain* c0 = cs[0];
  const int ng = c0->ngroup, nb = c0->nblock;
  if (c0->ntime % ng != 0) { set_error("batch init_g: ntime %% ngroup != 0"); return PQMC_ERR_ARG; }
  const size_t qb = sizeof(cplx) * (size_t)ns * ne;
  std::vector<cplx*> X(C), D(C), XL(C), Gc(C), Gn(C);
  for (int i = 0; i < C; ++i) {
    pqmc_chain* c = cs[i];
    PQMC_CUDA(cudaMemcpyAsync(qblk(c, 1), c->slater_q, qb, cudaMemcpyDeviceToDevice, stream));
    PQMC_CUDA(cudaMemcpyAsync(qblk(c, nb), c->slater_q, qb, cudaMemcpyDeviceToDevice, stream));
    PQMC_CUDA(cudaMemcpyAsync(dblk(c, 1), c->slater_d, sizeof(cplx) * ne, cudaMemcpyDeviceToDevice, stream));
    PQMC_CUDA(cudaMemcpyAsync(dblk(c, nb), c->slater_d, sizeof(cplx) * ne, cudaMemcpyDeviceToDevice, stream));
    X[i] = c->rmat;
    PQMC_CUDA(cudaMemcpyAsync(X[i], c->slater_q, qb, cudaMemcpyDeviceToDevice, stream));
  }
  for (int blk = 2; blk <= nb - 1; ++blk) {
    PQMC_TRY(propagate(X, (blk - 2) * ng + 1, (blk - 1) * ng, true));
    for (int i = 0; i < C; ++i) D[i] = dblk(cs[i], blk);
    PQMC_TRY(cholqr2(X, D));
    for (int i = 0; i < C; ++i)
      PQMC_CUDA(cudaMemcpyAsync(qblk(cs[i], blk), X[i], qb, cudaMemcpyDeviceToDevice, stream));
  }
  // per-block sums of log D on each chain's own stream, after the strings
  PQMC_CUDA(cudaStreamSynchronize(stream));
  for (auto* c : cs) {
    for (int b = 1; b <= nb; ++b) PQMC_TRY(block_log(c, b));
    PQMC_CUDA(cudaStreamSynchronize(c->stream));
  }
  for (int i = 0; i < C; ++i) {
    XL[i] = qblk(cs[i], nb);
    Gc[i] = cs[i]->g;
    Gn[i] = cs[i]->g_alt;
  }
  PQMC_TRY(g_and_det(XL, X, Gc, Gn, false, nb, false));
  for (auto* c : cs) {
    cplx* t = c->g;
    c->g = c->g_alt;
    c->g_alt = t;
  }
  PQMC_CUDA(cudaStreamSynchronize(stream));
  return PQMC_OK;
}

// get_g_scratch_T0 for every chain (each chain's current G is in c->g;
// the new G is written to c->g_alt and the pointers are swapped)
int BatchRecompute::scratch(int time, bool forward, int parity) {
  pqmc_chain* c0 = cs[0];
  const int ng = c0->ngroup;
  std::vector<cplx*> X(C), XL(C), D(C), R(C), Gc(C), Gn(C);
  size_t qb = sizeof(cplx) * (size_t)ns * ne;
  int blk;
  if (forward) {
    blk = time / ng + 1;
    if (time - ng < 1 || blk < 2 || blk + 1 > c0->nblock) { set_error("batch scratch: bad time %d", time); return PQMC_ERR_ARG; }
    for (int i = 0; i < C; ++i) {
      X[i] = cs[i]->rmat;
      PQMC_CUDA(cudaMemcpyAsync(X[i], qblk(cs[i], blk - 1), qb, cudaMemcpyDeviceToDevice, stream));
      D[i] = dblk(cs[i], blk);
    }
    PQMC_TRY(propagate(X, time - ng, time - 1, true));
    PQMC_TRY(cholqr2(X, D));
    for (int i = 0; i < C; ++i) {
      PQMC_CUDA(cudaMemcpyAsync(qblk(cs[i], blk), X[i], qb, cudaMemcpyDeviceToDevice, stream));
      XL[i] = qblk(cs[i], blk + 1);
      R[i] = X[i];
    }
  } else {
    blk = time / ng + 2;
    if (ng == 1) blk -= 1;
    if (time < 1 || time + ng - 1 > c0->ntime || blk < 2 || blk + 1 > c0->nblock) {
      set_error("batch scratch: bad time %d", time);
      return PQMC_ERR_ARG;
    }
    for (int i = 0; i < C; ++i) {
      X[i] = cs[i]->xmat;
      PQMC_CUDA(cudaMemcpyAsync(X[i], qblk(cs[i], blk + 1), qb, cudaMemcpyDeviceToDevice, stream));
      D[i] = dblk(cs[i], blk);
    }
    PQMC_TRY(propagate(X, time + ng - 1, time, false));
    PQMC_TRY(cholqr2(X, D));
    for (int i = 0; i < C; ++i) {
      PQMC_CUDA(cudaMemcpyAsync(qblk(cs[i], blk), X[i], qb, cudaMemcpyDeviceToDevice, stream));
      XL[i] = X[i];
      R[i] = qblk(cs[i], blk - 1);
    }
  }
  // the current G is the parity buffer; the new one goes to the other (the
  // caller flips the parity)
  for (int i = 0; i < C; ++i) {
    Gc[i] = parity ? cs[i]->g_alt : cs[i]->g;
    Gn[i] = parity ? cs[i]->g : cs[i]->g_alt;
  }
  return g_and_det(XL, R, Gc, Gn, true, blk, true);   // the mixed sweep keeps G in double-float form
}

}  // namespace pqmc

// ---------------------------------------------------------------------------
extern "C" int pqmc_recompute_gemm_check(char ta, char tb, int m, int n, int k, int count, const double* a, int lda,
                                         const double* b, int ldb, double* c, int ldc, int engine) {
  using namespace pqmc;
  const bool TA = ta == 'C', TB = tb == 'C';
  if (!a || !b || !c || (ta != 'N' && !TA) || (tb != 'N' && !TB) || m < 1 || n < 1 || k < 1 || count < 1 ||
      lda < (TA ? k : m) || ldb < (TB ? n : k) || ldc < m || (engine != 0 && engine != 1)) {
    set_error("recompute_gemm_check: need ta, tb in {N, C}, m, n, k, count >= 1, lda, ldb, ldc at least the rows "
              "of A, B, C, engine 0 or 1");
    return PQMC_ERR_ARG;
  }
  const size_t na = (size_t)lda * (TA ? m : k), nb = (size_t)ldb * (TB ? k : n), nc = (size_t)ldc * n;
  cplx *d_a = nullptr, *d_b = nullptr, *d_c = nullptr;
  GemmArgs* d_ga = nullptr;
  OgDesc* d_od = nullptr;
  unsigned char* d_img = nullptr;
  int* d_err = nullptr;
  auto run = [&]() -> int {
    PQMC_CUDA(cudaMalloc((void**)&d_a, sizeof(cplx) * na * count));
    PQMC_CUDA(cudaMalloc((void**)&d_b, sizeof(cplx) * nb * count));
    PQMC_CUDA(cudaMalloc((void**)&d_c, sizeof(cplx) * nc * count));
    PQMC_CUDA(cudaMalloc((void**)&d_err, sizeof(int)));
    PQMC_CUDA(cudaMemset(d_err, 0, sizeof(int)));
    PQMC_CUDA(cudaMemcpy(d_a, a, sizeof(cplx) * na * count, cudaMemcpyHostToDevice));
    PQMC_CUDA(cudaMemcpy(d_b, b, sizeof(cplx) * nb * count, cudaMemcpyHostToDevice));
    if (engine == 0) {
      std::vector<GemmArgs> ga(count);
      for (int i = 0; i < count; ++i) ga[i] = GemmArgs{d_a + na * i, d_b + nb * i, d_c + nc * i, lda, ldb, ldc, 0, 0};
      PQMC_CUDA(cudaMalloc((void**)&d_ga, sizeof(GemmArgs) * count));
      PQMC_CUDA(cudaMemcpy(d_ga, ga.data(), sizeof(GemmArgs) * count, cudaMemcpyHostToDevice));
      PQMC_TRY(dfgemm_batched(0, ta, tb, m, n, k, d_ga, count, 0));
    } else {
      PQMC_TRY(ozgemm_setup());
      const size_t ib = ozgemm_img_bytes(m, n);
      PQMC_CUDA(cudaMalloc((void**)&d_img, ib * count));
      std::vector<OgDesc> od(count);
      for (int i = 0; i < count; ++i)
        od[i] = OgDesc{d_a + na * i, d_b + nb * i, reinterpret_cast<float4*>(d_c + nc * i), d_img + ib * i, d_err};
      PQMC_CUDA(cudaMalloc((void**)&d_od, sizeof(OgDesc) * count));
      PQMC_CUDA(cudaMemcpy(d_od, od.data(), sizeof(OgDesc) * count, cudaMemcpyHostToDevice));
      PQMC_TRY(ozgemm_batched(0, ta, tb, m, n, k, lda, ldb, ldc, d_od, count, 1));
    }
    PQMC_CUDA(cudaDeviceSynchronize());
    int herr = 0;
    PQMC_CUDA(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      set_error("recompute_gemm_check: a wait of the tensor-core product gave up");
      return PQMC_ERR_TIMEOUT;
    }
    PQMC_CUDA(cudaMemcpy(c, d_c, sizeof(cplx) * nc * count, cudaMemcpyDeviceToHost));
    return PQMC_OK;
  };
  const int st = run();
  void* ps[] = {d_a, d_b, d_c, d_ga, d_od, d_img, d_err};
  for (void* p : ps)
    if (p) cudaFree(p);
  return st;
}
