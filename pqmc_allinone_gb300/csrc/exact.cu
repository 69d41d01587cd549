// exact.cu -- the exact round update (see exact.cuh): G <- G + G(:,S) M Z
// with M = Delta_S (I + G(S,S) Delta_S)^-1 and Z = E_S - G(S,:), from the
// double-float G the round started from.
#include <cuda_bf16.h>
#include <string.h>
#include <vector>
#include "df32.cuh"
#include "exact.cuh"
#include "ozaki.cuh"

namespace pqmc {

// ---------------------------------------------------------------------------
// Ozaki slices (ozaki.cuh) with OZ_S = 5 pieces: the exponent floor -80 keeps
// the deepest grid 2^(e-40) a normal FP32 power of two.
static_assert(-80 >= 8 * OZ_S - 126, "exponent floor");
__device__ __forceinline__ int oz_exp(float vmax) { return oz_exp_f<-80>(vmax); }
__device__ __forceinline__ void oz_split(float h, float l, int e, float* q) { oz_split_n<OZ_S>(h, l, e, q); }
// three accumulator levels (exact, exact, rounded) combined in double-float
__device__ __forceinline__ df oz_combine(float l0, float l1, float l2) {
  const df s = two_sum(l0, l1);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, l2));
}

// double-float complex helpers
__device__ __forceinline__ dfc dg_dfc(float4 g) { return dfc{df{g.x, g.z}, df{g.y, g.w}}; }
__device__ __forceinline__ float4 dfc_dg(dfc a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }
// acc + a*b, one renormalisation per component
__device__ __forceinline__ dfc dfc_mac(dfc acc, dfc a, dfc b) {
  return dfc_fms(acc, dfc{df_neg(a.re), df_neg(a.im)}, b);
}
// 1/a: conj(a) / |a|^2 with the reciprocal refined by one Newton step
__device__ __forceinline__ dfc dfc_inv(dfc a) {
  const df n = df_add(df_mul(a.re, a.re), df_mul(a.im, a.im));
  const float r0 = __frcp_rn(n.hi);
  const df e = df_sub(df{1.0f, 0.0f}, df_mulf(n, r0));   // 1 - n r0
  const df r = df_add(df{r0, 0.0f}, df_mulf(e, r0));
  return dfc{df_mul(a.re, r), df_neg(df_mul(a.im, r))};
}

// ---------------------------------------------------------------------------
// M = Delta_S W^-1, W = I + G(S,S) Delta_S, in two launches:
//   k_xinv  (one CTA per chain) forms W in double-float and inverts its
//           FP32 rounding by Gauss-Jordan over the moves' dim x dim blocks
//           (the block pivots are the moves' ratio matrices R_j, each
//           inverted by its adjugate): V0 = W^-1 to ~1e-6;
//   k_xres  (XR_CTAS per chain, a column slab each) one Newton step,
//           V1 = V0 + V0 (I - W V0), with the residual I - W V0 formed in
//           double-float from every product's exact parts, so V1 = W^-1 to
//           ~|I - W V0|^2; then M = Delta_S V1 and the Ozaki slices of M's
//           columns (the B operand of X = G(:,S) M).
// The rows of G(:,S) (the A operand of X) and the columns of Z = E_S - G(S,:)
// (the B operand of the flush) depend on G and S only and are cut by
// k_xslice, launched before both.
constexpr int XC_THREADS = 1024;
constexpr int XC_LD = UM_KP;   // leading dimension of the K x K matrices
constexpr int XR_CTAS = 8;     // column slabs of the Newton step per chain
constexpr int XR_W = UM_KP / XR_CTAS;
constexpr int XR_THREADS = UM_KP * XR_W;   // one residual entry per thread
constexpr size_t XI_SMEM = sizeof(float4) * 16 * UM_KP + sizeof(float2) * ((size_t)XC_LD * XC_LD + 8 * UM_KP) +
                           sizeof(int) * UM_KP;
constexpr size_t XR_SMEM = sizeof(float4) * ((size_t)XC_LD * XC_LD + 16 * UM_KP + (size_t)UM_KP * XR_W) +
                           sizeof(float2) * (size_t)XC_LD * XC_LD;

__global__ void __launch_bounds__(XC_THREADS, 1) k_xinv(const XDesc* X, int dim, int parity) {
  __shared__ XDesc sd;
  __shared__ float2 s_pb[16];
  extern __shared__ __align__(16) unsigned char xc_dyn[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sd = X[blockIdx.y];
  __syncthreads();
  const XDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;
  const int ns = d.ns;
  const float4* G = parity ? d.g_alt : d.g;
  {
    float4* s_dl = reinterpret_cast<float4*>(xc_dyn);                 // [n_acc][16] Delta blocks
    float2* Wf = reinterpret_cast<float2*>(s_dl + 16 * UM_KP);        // [K][XC_LD] FP32 W, inverted in place
    float2* s_row = Wf + (size_t)XC_LD * XC_LD;                       // [dim][UM_KP] pivot rows
    float2* s_col = s_row + 4 * UM_KP;                                // [dim][UM_KP] pivot columns
    int* s_site = reinterpret_cast<int*>(s_col + 4 * UM_KP);
    const int nb = K / dim;
    for (int k = tid; k < K; k += XC_THREADS) s_site[k] = d.acc_site[k];
    for (int e = tid; e < nb * 16; e += XC_THREADS) s_dl[e] = d.acc_delta[e];
    __syncthreads();
    // W(i, jb*dim + jj) = delta_ij + sum_m G(S_i, S_{jb dim + m}) Delta_jb(m, jj)
    for (int it = tid; it < K * nb; it += XC_THREADS) {
      const int i = it % K, jb = it / K;
      dfc gs[4];
#pragma unroll
      for (int m = 0; m < 4; ++m)
        if (m < dim) gs[m] = dg_dfc(G[s_site[i] + (size_t)ns * s_site[jb * dim + m]]);
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        if (jj >= dim) break;
        const int j = jb * dim + jj;
        dfc a = dfc{df{i == j ? 1.f : 0.f, 0.f}, df{0.f, 0.f}};
#pragma unroll
        for (int m = 0; m < 4; ++m)
          if (m < dim) a = dfc_mac(a, gs[m], dg_dfc(s_dl[jb * 16 + m + dim * jj]));
        d.wdf[j * XC_LD + i] = dfc_dg(a);   // column-major: k_xres reads W(i, k) for consecutive i
        Wf[i * XC_LD + j] = make_float2(a.re.hi, a.im.hi);
      }
    }
    __syncthreads();
    // FP32 Gauss-Jordan in place by blocks of the moves: the pivot block P is
    // inverted by its adjugate on 16 lanes, the multipliers F_i = W(i, bb)
    // P^-1 are formed once per row
    constexpr int CG = XC_THREADS / UM_KP;      // threads per row
    const int ri = tid / CG, cg = tid % CG;   // row ri, columns cg, cg + CG, ...
    for (int b = 0; b < nb; ++b) {
      const int b0 = b * dim;
      if (warp == 0) {
        if (lane < dim * dim) s_pb[lane] = Wf[(b0 + lane % dim) * XC_LD + b0 + lane / dim];   // column-major P
        __syncwarp();
        const float2 det = wf_det(dim, s_pb, lane);
        if (lane == 0 && !(det.x * det.x + det.y * det.y > 0.f)) atomicExch(d.err, PQMC_ERR_SINGULAR);
        wf_inverse(dim, s_pb, det, lane);   // s_pb <- P^-1
      }
      for (int e = tid; e < dim * K; e += XC_THREADS) {   // pivot rows and pivot columns before the step
        const int m = e / K, j = e % K;
        s_row[m * UM_KP + j] = Wf[(b0 + m) * XC_LD + j];
        s_col[m * UM_KP + j] = Wf[j * XC_LD + b0 + m];
      }
      __syncthreads();
      if (ri < K) {
        const bool piv_row = ri >= b0 && ri < b0 + dim;
        float2 f[4];   // piv_row: row ri - b0 of P^-1; else F_ri = W(ri, bb) P^-1
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          f[n] = make_float2(0.f, 0.f);
          if (n >= dim) continue;
          if (piv_row) {
            f[n] = s_pb[(ri - b0) + dim * n];
          } else {
#pragma unroll
            for (int m = 0; m < 4; ++m)
              if (m < dim) f[n] = fcfma(s_col[m * UM_KP + ri], s_pb[m + dim * n], f[n]);
          }
        }
        for (int j = cg; j < K; j += CG) {
          float2 v;
          if (j >= b0 && j < b0 + dim) {
            v = piv_row ? f[j - b0] : make_float2(-f[j - b0].x, -f[j - b0].y);
          } else {
            v = piv_row ? make_float2(0.f, 0.f) : Wf[ri * XC_LD + j];
#pragma unroll
            for (int m = 0; m < 4; ++m)
              if (m < dim) {
                const float2 r = s_row[m * UM_KP + j];
                v = piv_row ? fcfma(f[m], r, v) : fsb(v, fm(f[m], r));
              }
          }
          Wf[ri * XC_LD + j] = v;
        }
      }
      __syncthreads();
    }
    for (int e = tid; e < K * K; e += XC_THREADS) d.v0[(e / K) * XC_LD + e % K] = Wf[(e / K) * XC_LD + e % K];
    return;
  }
}

// k_xslice: the Ozaki slices of G(:,S) (the A operand of X = G(:,S) M) and
// of Z = E_S - G(S,:) (the B operand of the flush).  They depend on G and S
// only, so they run in their own light launch (256 threads, no dynamic
// shared memory, several CTAs per SM beside the other kernels) instead of
// inside the Newton step's 512-thread CTAs.
//   CTAs 0 .. XS_RCTAS-1 (per 16 rows): 16 threads per row, 4 k each; the
//   row's exponent from the largest |hi| over its K entries (a max over the
//   16 lanes of the row), then 8-byte stores of 4 BF16 per slice.
//   CTAs past them (per 8 columns): a warp per column of Z, 2 k per lane,
//   into the column tiles of the flush kernel in use (64 or 32 columns).
constexpr int XS_THREADS = 256;
constexpr int XS_ROWS = XS_THREADS / 16;   // rows of G(:,S) per CTA
constexpr int XS_COLS = XS_THREADS / 32;   // columns of Z per CTA
__global__ void __launch_bounds__(XS_THREADS, 4) k_xslice(const XDesc* X, int parity, int n_rcta, int ct) {
  const XDesc& d = X[blockIdx.y];
  const int K = *d.kcount;
  if (K == 0) return;
  const float4* G = parity ? d.g_alt : d.g;
  const int ns = d.ns, tid = threadIdx.x, lane = tid & 31;
  const int K16 = (K + 15) & ~15;
  const int* S = d.acc_site;
  if ((int)blockIdx.x < n_rcta) {
    // ---- rows of G(:,S): A operand of X = G(:,S) M ------------------------
    const int r = blockIdx.x * XS_ROWS + tid / 16, q = tid % 16;   // k = 4q .. 4q+3
    const bool row_ok = r < ns;
    float4 v[4];
    float m = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int k = 4 * q + u;
      v[u] = (row_ok && k < K) ? G[r + (size_t)ns * S[k]] : make_float4(0.f, 0.f, 0.f, 0.f);
      m = fmaxf(m, fmaxf(fabsf(v[u].x), fabsf(v[u].y)));
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));   // the row's 16 lanes
    if (!row_ok || 4 * q >= K16) return;
    const int e = oz_exp(m);
    const int t = r / 128, row = r % 128, nrg = um_rg(ns, t);
    uint32_t wr[OZ_S][2], wi[OZ_S][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float r0[OZ_S], r1[OZ_S], i0[OZ_S], i1[OZ_S];
      oz_split(v[2 * h].x, v[2 * h].z, e, r0);
      oz_split(v[2 * h + 1].x, v[2 * h + 1].z, e, r1);
      oz_split(v[2 * h].y, v[2 * h].w, e, i0);
      oz_split(v[2 * h + 1].y, v[2 * h + 1].w, e, i1);
#pragma unroll
      for (int sl = 0; sl < OZ_S; ++sl) {
        wr[sl][h] = oz_pack2(r0[sl], r1[sl]);
        wi[sl][h] = oz_pack2(i0[sl], i1[sl]);
      }
    }
    const int kg = q / 2, half = (q & 1) * 8;
#pragma unroll
    for (int sl = 0; sl < OZ_S; ++sl) {   // A' row = [Gr | Gi]
      unsigned char* im = d.img + (size_t)oz_slot_a1(ns, t, sl) * UM_IMG;
      *reinterpret_cast<uint2*>(im + um_off(row, kg * 8, nrg) + half) = make_uint2(wr[sl][0], wr[sl][1]);
      *reinterpret_cast<uint2*>(im + um_off(row, UM_KP + kg * 8, nrg) + half) = make_uint2(wi[sl][0], wi[sl][1]);
    }
    return;
  }
  // ---- columns of Z = E_S - G(S,:): B operand of the flush, a warp each ----
  const int c = ((int)blockIdx.x - n_rcta) * XS_COLS + (tid >> 5);
  if (c >= ns) return;
  dfc z[2];
  float m = 0.f;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    z[h] = dfc_zero();
    if (k < K) {
      const int sk = S[k];
      const dfc g = dg_dfc(G[sk + (size_t)ns * c]);
      z[h] = dfc{sk == c ? df_sub(df{1.f, 0.f}, g.re) : df_neg(g.re), df_neg(g.im)};
      m = fmaxf(m, fmaxf(fabsf(z[h].re.hi), fabsf(z[h].im.hi)));
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int e = oz_exp(m);
  // Z's column tiles are ct = 64 (k_xgemm<1>) or 32 (k_xflush2) columns wide,
  // padded to 8 or 4 column groups (zeros past Ns)
  const int tj = c / ct, cc = c % ct, ncg = ct == 64 ? um_cg(ns, tj) : 4, nrg = 2 * ncg;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    if (k >= K16) break;
    float qr[OZ_S], qi[OZ_S];
    oz_split(z[h].re.hi, z[h].re.lo, e, qr);
    oz_split(z[h].im.hi, z[h].im.lo, e, qi);
#pragma unroll
    for (int sl = 0; sl < OZ_S; ++sl) {
      // B' re row cc = [Zr | -Zi], im row 8 ncg + cc = [Zi | Zr]
      unsigned char* im = d.img + (size_t)oz_slot_b2(ns, tj, sl) * UM_IMG;
      *reinterpret_cast<__nv_bfloat16*>(im + um_off(cc, k, nrg)) = __float2bfloat16_rn(qr[sl]);
      *reinterpret_cast<__nv_bfloat16*>(im + um_off(cc, UM_KP + k, nrg)) = __float2bfloat16_rn(-qi[sl]);
      *reinterpret_cast<__nv_bfloat16*>(im + um_off(8 * ncg + cc, k, nrg)) = __float2bfloat16_rn(qi[sl]);
      *reinterpret_cast<__nv_bfloat16*>(im + um_off(8 * ncg + cc, UM_KP + k, nrg)) = __float2bfloat16_rn(qr[sl]);
    }
  }
}

// acc += a * b for a double-float real a and an FP32 b: the product's high
// part (exact with its FMA error term) enters acc.hi by a two-sum, the
// rounding errors and a.lo * b go to acc.lo (not renormalised)
__device__ __forceinline__ void df_mac_f(float& h, float& l, float ah, float al, float b) {
  const float p = __fmul_rn(ah, b);
  const float e = __fmaf_rn(ah, b, -p);
  const df s = two_sum(h, p);
  h = s.hi;
  l = __fmaf_rn(al, b, __fadd_rn(l, __fadd_rn(s.lo, e)));
}

__global__ void __launch_bounds__(XR_THREADS, 1) k_xres(const XDesc* X, int dim, int parity) {
  __shared__ XDesc sd;
  __shared__ int s_ce[XR_W];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_fail;
  extern __shared__ __align__(16) unsigned char xr_dyn[];
  const int tid = threadIdx.x;
  if (tid == 0) {
    sd = X[blockIdx.y];
    s_fail = 0;
    mbar_init(&s_bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const XDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;
  const int nb = K / dim;
  const int j0 = blockIdx.x * XR_W;   // this CTA's columns j0 .. j0 + XR_W - 1 of M
  float4* W = reinterpret_cast<float4*>(xr_dyn);                     // [K][XC_LD] double-float W, column-major
  float4* s_dl = W + (size_t)XC_LD * XC_LD;                           // [n_acc][16]
  float4* Rs = s_dl + 16 * UM_KP;                                     // [K][XR_W] residual, then V1, then M
  float2* V = reinterpret_cast<float2*>(Rs + (size_t)UM_KP * XR_W);   // [K][XC_LD] V0
  if (tid == 0) {   // the first K columns of W and rows of V0 (contiguous) and the Delta records by bulk copies
    const uint32_t bw = (uint32_t)(sizeof(float4) * XC_LD * K), bv = (uint32_t)(sizeof(float2) * XC_LD * K);
    const uint32_t bd = (uint32_t)(sizeof(float4) * 16 * nb);
    fence_proxy_async_global();
    mbar_arrive_tx(&s_bar, bw + bv + bd);
    bulk_g2s(W, d.wdf, bw, &s_bar);
    bulk_g2s(V, d.v0, bv, &s_bar);
    bulk_g2s(s_dl, d.acc_delta, bd, &s_bar);
    if (!mbar_wait_bounded(&s_bar, 0)) {
      s_fail = 1;
      mbar_wait_bounded(&s_bar, 0);   // a second bounded wait for the copies in flight
    }
  }
  __syncthreads();
  if (s_fail) {
    if (tid == 0) atomicExch(d.err, PQMC_ERR_TIMEOUT);
    return;
  }
  // residual R = I - W V0 on this slab, one entry per thread (row ri, column cq)
  const int ri = tid % UM_KP, cq = tid / UM_KP;
  const int j = j0 + cq;
  if (ri < K) {
    float rh0 = 0.f, rl0 = 0.f, rh1 = 0.f, rl1 = 0.f;
    for (int k = 0; k < K; ++k) {
      const float4 w = W[k * XC_LD + ri];   // {re_hi, im_hi, re_lo, im_lo}; consecutive ri: no bank conflicts
      const float2 v = j < K ? V[k * XC_LD + j] : make_float2(0.f, 0.f);
      df_mac_f(rh0, rl0, w.x, w.z, v.x);     // re += wr vr
      df_mac_f(rh0, rl0, -w.y, -w.w, v.y);   //       - wi vi
      df_mac_f(rh1, rl1, w.x, w.z, v.y);     // im += wr vi
      df_mac_f(rh1, rl1, w.y, w.w, v.x);     //       + wi vr
    }
    const df wr = quick_two_sum(rh0, rl0), wi = quick_two_sum(rh1, rl1);
    const df rr = df_sub(df{ri == j ? 1.f : 0.f, 0.f}, wr);   // I - W V0
    Rs[ri * XR_W + cq] = make_float4(rr.hi, -wi.hi, rr.lo, -wi.lo);
  }
  __syncthreads();
  // V1 = V0 + V0 R on the slab (R is small: its FP32 rounding suffices).
  // Threads take (row tid / XR_W, column tid % XR_W) here, so a warp reads 4
  // rows of V0 (a 4-way bank conflict, not 32) and consecutive R entries.
  const int ri2 = tid / XR_W, cq2 = tid % XR_W, j2 = j0 + cq2;
  float4 v1 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (ri2 < K) {
    float2 s = make_float2(0.f, 0.f);
    for (int k = 0; k < K; ++k) s = fcfma(V[ri2 * XC_LD + k], hi2(Rs[k * XR_W + cq2]), s);
    const float2 v0 = j2 < K ? V[ri2 * XC_LD + j2] : make_float2(0.f, 0.f);
    const df a = two_sum(v0.x, s.x), b = two_sum(v0.y, s.y);
    v1 = make_float4(a.hi, b.hi, a.lo, b.lo);
  }
  __syncthreads();
  if (ri2 < K) Rs[ri2 * XR_W + cq2] = v1;
  __syncthreads();
  // M = Delta_S V1 block row by block row
  for (int it = tid; it < nb * XR_W; it += XR_THREADS) {
    const int jb = it / XR_W, jl = it % XR_W;
    dfc w[4], m[4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if (a < dim) w[a] = dg_dfc(Rs[(jb * dim + a) * XR_W + jl]);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      if (a >= dim) break;
      m[a] = dfc_zero();
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (b < dim) m[a] = dfc_mac(m[a], dg_dfc(s_dl[jb * 16 + a + dim * b]), w[b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if (a < dim) Rs[(jb * dim + a) * XR_W + jl] = dfc_dg(m[a]);
  }
  __syncthreads();
  // Ozaki slices of M's columns j0.. (output columns of X): B' re row c =
  // [Mr | -Mi], im row 64 + c = [Mi | Mr]; columns at or past K are zero
  if (tid < XR_W) {
    float mx = 0.f;
    if (j0 + tid < K)
      for (int k = 0; k < K; ++k) {
        const float4 v = Rs[k * XR_W + tid];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
    s_ce[tid] = oz_exp(mx);
  }
  __syncthreads();
  const int K16 = (K + 15) & ~15, KG = K16 / 8;
  const int ns = d.ns;
  for (int it = tid; it < XR_W * KG; it += XR_THREADS) {
    const int jl = it % XR_W, kg = it / XR_W, c = j0 + jl;
    float rs[OZ_S][8], is[OZ_S][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kg * 8 + u;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (c < K && k < K) v = Rs[k * XR_W + jl];
      float qr[OZ_S], qi[OZ_S];
      oz_split(v.x, v.z, s_ce[jl], qr);
      oz_split(v.y, v.w, s_ce[jl], qi);
#pragma unroll
      for (int q = 0; q < OZ_S; ++q) {
        rs[q][u] = qr[q];
        is[q][u] = qi[q];
      }
    }
#pragma unroll
    for (int q = 0; q < OZ_S; ++q) {
      unsigned char* im = d.img + (size_t)oz_slot_b1(ns, q) * UM_IMG;
      float ni[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) ni[u] = -is[q][u];
      *reinterpret_cast<uint4*>(im + um_off(c, kg * 8, 16)) = oz_pack8(rs[q]);
      *reinterpret_cast<uint4*>(im + um_off(c, UM_KP + kg * 8, 16)) = oz_pack8(ni);
      *reinterpret_cast<uint4*>(im + um_off(64 + c, kg * 8, 16)) = oz_pack8(is[q]);
      *reinterpret_cast<uint4*>(im + um_off(64 + c, UM_KP + kg * 8, 16)) = oz_pack8(rs[q]);
    }
  }
}

// ---------------------------------------------------------------------------
// k_xgemm: one CTA per output tile, one CTA per SM (160 KB of images, 384
// tensor-memory columns).  Thread 0 streams the OZ_S A and OZ_S B half-images
// of a K half through shared memory and issues the products of slice pairs
// (i, j) with i + j < OZ_S into three FP32 accumulators: level 0 and level
// 1 (exact), levels 2.. (rounded at 2^-40 of the result).  MODE 0: X = G(:,S)
// M over a 128-row tile, written as the slice images of the flush's A
// operand (row exponents from the tile itself); MODE 1: the flush G += X Z
// over a 128 x 64 tile of G.
constexpr int XG_SMEM = 2 * OZ_S * (UM_IMG / 2);

__device__ __forceinline__ void um_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 8 consecutive FP32 columns of tensor memory (no wait)
__device__ __forceinline__ void um_ld8_nw(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// both modes run their epilogue (MODE 1: the G read-modify-write, MODE 0:
// the slicing of X) on 16 warps, 16 columns each in chunks of 8
constexpr int XG_THREADS = 512;
constexpr int XG_WB = 4;   // column blocks of 16 (warps per lane quarter)

template <int MODE>
__global__ void __launch_bounds__(XG_THREADS, 1) k_xgemm(const XDesc* X, int parity) {
  __shared__ XDesc sd;
  __shared__ __align__(8) uint64_t s_load[2], s_mma[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail, s_last;
  __shared__ float s_rmax[XG_WB][128];
  extern __shared__ __align__(1024) unsigned char xg_dyn[];   // OZ_S A half-images, then OZ_S B half-images
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    sd = X[blockIdx.y];
    s_fail = 0;
    s_last = -1;
    for (int h = 0; h < 2; ++h) {
      mbar_init(&s_load[h], 1);
      mbar_init(&s_mma[h], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  const XDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;   // uniform: no tensor memory taken
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&s_taddr))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const uint32_t taddr = s_taddr;
  const int ns = d.ns, RT = um_rtiles(ns);
  const int ti = MODE == 0 ? (int)blockIdx.x : (int)blockIdx.x % RT;
  const int tj = MODE == 0 ? 0 : (int)blockIdx.x / RT;
  const int nrg_a = um_rg(ns, ti);
  const int ncg = MODE == 0 ? 8 : um_cg(ns, tj), nrg_b = 2 * ncg;
  const int K16 = (K + 15) & ~15;
  if (tid == 0) {
    if (MODE == 1 && blockIdx.x == 0) atomicAdd(d.nflush, 1ull);
    const uint32_t ka = (uint32_t)nrg_a * 128, kb = (uint32_t)nrg_b * 128;   // bytes per K group of 8
    const uint32_t part_a = (uint32_t)(K16 / 8) * ka, part_b = (uint32_t)(K16 / 8) * kb;
    const uint32_t h2a = (uint32_t)(UM_KP / 8) * ka, h2b = (uint32_t)(UM_KP / 8) * kb;
    const uint32_t base = smem_addr(xg_dyn), idesc = um_idesc(16u * (uint32_t)ncg);
    constexpr uint32_t HALF = UM_IMG / 2;
    uint32_t started = 0;
    for (int half = 0; half < 2; ++half) {
      if (half == 1) {   // the products of half 0 have read the buffer
        if (!mbar_wait_bounded(&s_mma[0], 0)) {
          s_fail = 1;
          break;
        }
        um_fence_after();
      }
      mbar_arrive_tx(&s_load[half], (uint32_t)OZ_S * (part_a + part_b));
      for (int s = 0; s < OZ_S; ++s) {
        const int sa = MODE == 0 ? oz_slot_a1(ns, ti, s) : oz_slot_a2(ns, ti, s);
        const int sb = MODE == 0 ? oz_slot_b1(ns, s) : oz_slot_b2(ns, tj, s);
        bulk_g2s(xg_dyn + (size_t)s * HALF, d.img + (size_t)sa * UM_IMG + half * h2a, part_a, &s_load[half]);
        bulk_g2s(xg_dyn + (size_t)(OZ_S + s) * HALF, d.img + (size_t)sb * UM_IMG + half * h2b, part_b, &s_load[half]);
      }
      if (!mbar_wait_bounded(&s_load[half], 0)) {
        s_fail = 1;
        mbar_wait_bounded(&s_load[half], 0);   // a second bounded wait for the copies in flight
        break;
      }
      um_fence_after();
      for (int i = 0; i < OZ_S; ++i)
        for (int j = 0; i + j < OZ_S; ++j) {
          const int l = min(i + j, 2);
          for (int kk = 0; kk < K16 / 16; ++kk) {
            const uint64_t ad = um_desc(base + i * HALF + kk * 2 * ka, ka, 128);
            const uint64_t bd = um_desc(base + (OZ_S + j) * HALF + kk * 2 * kb, kb, 128);
            um_mma(taddr + (uint32_t)(l * 128), ad, bd, idesc, (started >> l) & 1u);
            started |= 1u << l;
          }
        }
      um_commit(&s_mma[half]);   // also tracks every earlier product
      s_last = half;
    }
  }
  const int q = warp & 3, hf = warp >> 2;   // lane quarter; column block of 16
  constexpr int XG_WC = 64 / XG_WB;           // columns per warp
  const int r = ti * 128 + q * 32 + lane;
  if (MODE == 1 && r < ns) {
    // the epilogue's G entries into L2 while thread 0 runs the copies and
    // products (a prefetch holds no registers and cannot fault: every
    // address is inside the chain's Ns x Ns tile)
    const float4* G = parity ? d.g_alt : d.g;
    const int col0 = tj * 64 + hf * XG_WC, ncol = min(XG_WC, ns - col0);
    for (int c = 0; c < ncol; ++c)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(G + r + (size_t)ns * (col0 + c)));
  }
  __syncthreads();
  const int last = s_last;
  if (last >= 0) {   // every exit path waits for the last commit (it tracks all earlier products)
    if (!mbar_wait_bounded(&s_mma[last], 0)) s_fail = 1;
    um_fence_after();
  }
  __syncthreads();
  const uint32_t tbase = taddr + ((uint32_t)(q * 32) << 16);
  if (!s_fail) {
    if (MODE == 1) {
      // G tile += (level 0 + level 1 + level 2) in double-float
      float4* G = parity ? d.g_alt : d.g;
      const int col0 = tj * 64 + hf * XG_WC;
      const int ncol = min(XG_WC, ns - col0);
#pragma unroll 1
      for (int ch = 0; ch < 2; ++ch) {
        const int c0 = ch * 8;
        if (ncol <= c0) break;   // warp-uniform
        float4 gv[8];
        if (r < ns) {
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c0 + c < ncol) gv[c] = G[r + (size_t)ns * (col0 + c0 + c)];
        }
        float re[3][8], im[3][8];
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          um_ld8_nw(tbase + l * 128 + hf * XG_WC + c0, re[l]);
          um_ld8_nw(tbase + l * 128 + 8 * ncg + hf * XG_WC + c0, im[l]);
        }
        um_wait_ld();
        if (r < ns) {
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            if (c0 + c >= ncol) continue;
            const df vr = oz_combine(re[0][c], re[1][c], re[2][c]);
            const df vi = oz_combine(im[0][c], im[1][c], im[2][c]);
            const float4 g = gv[c];
            const df nr = df_add(df{g.x, g.z}, vr), ni = df_add(df{g.y, g.w}, vi);
            G[r + (size_t)ns * (col0 + c0 + c)] = make_float4(nr.hi, ni.hi, nr.lo, ni.lo);
          }
        }
      }
    } else {
      // X tile (128 rows x 64 complex columns): row exponent over the four
      // column blocks, then the slices of the flush's A operand [Xr | Xi]
      float mx = 0.f;
#pragma unroll 1
      for (int ch = 0; ch < 2; ++ch) {
        const int c0 = hf * XG_WC + ch * 8;
        float re[3][8], im[3][8];
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          um_ld8_nw(tbase + l * 128 + c0, re[l]);
          um_ld8_nw(tbase + l * 128 + 64 + c0, im[l]);
        }
        um_wait_ld();
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const df vr = oz_combine(re[0][c], re[1][c], re[2][c]);
          const df vi = oz_combine(im[0][c], im[1][c], im[2][c]);
          mx = fmaxf(mx, fmaxf(fabsf(vr.hi), fabsf(vi.hi)));
        }
      }
      const int row = q * 32 + lane;
      s_rmax[hf][row] = mx;
      __syncthreads();
      float rmx = s_rmax[0][row];
#pragma unroll
      for (int h = 1; h < XG_WB; ++h) rmx = fmaxf(rmx, s_rmax[h][row]);
      const int e = oz_exp(rmx);
#pragma unroll 1
      for (int ch = 0; ch < 2; ++ch) {
        const int k = hf * XG_WC + ch * 8;   // the 8 columns of X are 8 inner indices of the flush
        float re[3][8], im[3][8];
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          um_ld8_nw(tbase + l * 128 + k, re[l]);
          um_ld8_nw(tbase + l * 128 + 64 + k, im[l]);
        }
        um_wait_ld();
        if (r < ns) {
          uint32_t wr[OZ_S][4], wi[OZ_S][4];   // slices packed two BF16 per word as they are cut
#pragma unroll
          for (int u2 = 0; u2 < 4; ++u2) {
            float qr0[OZ_S], qi0[OZ_S], qr1[OZ_S], qi1[OZ_S];
            {
              const df vr = oz_combine(re[0][2 * u2], re[1][2 * u2], re[2][2 * u2]);
              const df vi = oz_combine(im[0][2 * u2], im[1][2 * u2], im[2][2 * u2]);
              oz_split(vr.hi, vr.lo, e, qr0);
              oz_split(vi.hi, vi.lo, e, qi0);
            }
            {
              const df vr = oz_combine(re[0][2 * u2 + 1], re[1][2 * u2 + 1], re[2][2 * u2 + 1]);
              const df vi = oz_combine(im[0][2 * u2 + 1], im[1][2 * u2 + 1], im[2][2 * u2 + 1]);
              oz_split(vr.hi, vr.lo, e, qr1);
              oz_split(vi.hi, vi.lo, e, qi1);
            }
#pragma unroll
            for (int sl = 0; sl < OZ_S; ++sl) {
              wr[sl][u2] = oz_pack2(qr0[sl], qr1[sl]);
              wi[sl][u2] = oz_pack2(qi0[sl], qi1[sl]);
            }
          }
#pragma unroll
          for (int sl = 0; sl < OZ_S; ++sl) {
            unsigned char* im2 = d.img + (size_t)oz_slot_a2(ns, ti, sl) * UM_IMG;
            *reinterpret_cast<uint4*>(im2 + um_off(row, k, nrg_a)) = make_uint4(wr[sl][0], wr[sl][1], wr[sl][2], wr[sl][3]);
            *reinterpret_cast<uint4*>(im2 + um_off(row, UM_KP + k, nrg_a)) =
                make_uint4(wi[sl][0], wi[sl][1], wi[sl][2], wi[sl][3]);
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(d.err, PQMC_ERR_TIMEOUT);
  }
  um_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(taddr) : "memory");
}

// ---------------------------------------------------------------------------
// k_xflush2: the flush G += X Z over a 128 x 32 tile of G, two CTAs per SM.
// The three level accumulators take 3 x 64 tensor-memory columns (re at
// 0..31, im at 32..63 of each level), so one CTA allocates 256 and two share
// an SM's 512; the images stream through a 60 KB stage a quarter of the
// inner dimension at a time (4 k groups of A, 128 rows, and of B, 32 re + 32
// im rows, five slices each), and the epilogue reads 8 columns at a time
// (at most 128 registers).  One CTA's G read-modify-write then overlaps the
// other's copies and products.  The same 15 slice pairs and levels as
// k_xgemm<1>; level 2 sums in another order (stage by stage), so the two
// agree to its rounding, not bit for bit.
constexpr int XF_QK = 4;                          // k groups of 8 per stage
constexpr int XF_A = XF_QK * 16 * 128;            // one A slice of a stage (16 row groups)
constexpr int XF_B = XF_QK * 8 * 128;             // one B slice of a stage (8 row groups)
constexpr int XF_SMEM = OZ_S * (XF_A + XF_B);     // 60 KB of stages
// requested per CTA: 80 KB, so that at most two CTAs share an SM (three
// would fit by registers and by 60 KB each, but 3 x 256 tensor-memory
// columns exceed the SM's 512 and the third allocation would wait)
constexpr int XF_SMEM_LAUNCH = 80 * 1024;
static_assert(XF_SMEM <= XF_SMEM_LAUNCH, "the stages fit in the requested shared memory");

__global__ void __launch_bounds__(256, 2) k_xflush2(const XDesc* X, int parity) {
  __shared__ XDesc sd;
  __shared__ __align__(8) uint64_t s_load[4], s_mma[4];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail, s_last;
  extern __shared__ __align__(1024) unsigned char xf_dyn[];   // OZ_S A stages, then OZ_S B stages
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    sd = X[blockIdx.y];
    s_fail = 0;
    s_last = -1;
    for (int p = 0; p < 4; ++p) {
      mbar_init(&s_load[p], 1);
      mbar_init(&s_mma[p], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  const XDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;   // uniform: no tensor memory taken
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_addr(&s_taddr))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const uint32_t taddr = s_taddr;
  const int ns = d.ns, RT = um_rtiles(ns);
  const int ti = (int)blockIdx.x % RT, tj = (int)blockIdx.x / RT;
  const int nrg_a = um_rg(ns, ti);
  const int nkg = ((K + 15) & ~15) / 8;   // k groups of one half (even, <= 8)
  if (tid == 0) {
    if (blockIdx.x == 0) atomicAdd(d.nflush, 1ull);
    const uint32_t ka = (uint32_t)nrg_a * 128, kb = 8u * 128u;   // bytes per k group
    const uint32_t base = smem_addr(xf_dyn), idesc = um_idesc(64u);
    uint32_t started = 0;
    int phase = 0;
    for (int half = 0; half < 2 && !s_fail; ++half)
      for (int qk = 0; qk < 2 && !s_fail; ++qk) {
        const int kg0 = XF_QK * qk, nk = min(XF_QK, nkg - kg0);
        if (nk <= 0) continue;
        if (phase > 0) {   // the products of the previous stage have read the buffer
          if (!mbar_wait_bounded(&s_mma[phase - 1], 0)) {
            s_fail = 1;
            break;
          }
          um_fence_after();
        }
        const uint32_t ba = (uint32_t)nk * ka, bb = (uint32_t)nk * kb;
        const size_t ga = (size_t)(half * (UM_KP / 8) + kg0) * ka, gb = (size_t)(half * (UM_KP / 8) + kg0) * kb;
        mbar_arrive_tx(&s_load[phase], (uint32_t)OZ_S * (ba + bb));
        for (int sl = 0; sl < OZ_S; ++sl) {
          bulk_g2s(xf_dyn + (size_t)sl * XF_A, d.img + (size_t)oz_slot_a2(ns, ti, sl) * UM_IMG + ga, ba, &s_load[phase]);
          bulk_g2s(xf_dyn + (size_t)OZ_S * XF_A + (size_t)sl * XF_B, d.img + (size_t)oz_slot_b2(ns, tj, sl) * UM_IMG + gb,
                   bb, &s_load[phase]);
        }
        if (!mbar_wait_bounded(&s_load[phase], 0)) {
          s_fail = 1;
          mbar_wait_bounded(&s_load[phase], 0);   // a second bounded wait for the copies in flight
          break;
        }
        um_fence_after();
        for (int i = 0; i < OZ_S; ++i)
          for (int j = 0; i + j < OZ_S; ++j) {
            const int l = min(i + j, 2);
            for (int kk = 0; kk < nk / 2; ++kk) {
              const uint64_t ad = um_desc(base + i * XF_A + kk * 2 * ka, ka, 128);
              const uint64_t bd = um_desc(base + OZ_S * XF_A + j * XF_B + kk * 2 * kb, kb, 128);
              um_mma(taddr + (uint32_t)(l * 64), ad, bd, idesc, (started >> l) & 1u);
              started |= 1u << l;
            }
          }
        um_commit(&s_mma[phase]);   // also tracks every earlier product
        s_last = phase;
        ++phase;
      }
  }
  const int q = warp & 3, hf = warp >> 2;
  const int r = ti * 128 + q * 32 + lane;
  const int col0 = tj * 32 + hf * 16, ncol = min(16, ns - col0);
  float4* G = parity ? d.g_alt : d.g;
  if (r < ns)   // the epilogue's G entries into L2 while the products run
    for (int c = 0; c < ncol; ++c) asm volatile("prefetch.global.L2 [%0];" ::"l"(G + r + (size_t)ns * (col0 + c)));
  __syncthreads();
  const int last = s_last;
  if (last >= 0) {   // every exit path waits for the last commit (it tracks all earlier products)
    if (!mbar_wait_bounded(&s_mma[last], 0)) s_fail = 1;
    um_fence_after();
  }
  __syncthreads();
  const uint32_t tbase = taddr + ((uint32_t)(q * 32) << 16);
  if (!s_fail) {
#pragma unroll 1
    for (int ch = 0; ch < 2; ++ch) {
      const int c0 = ch * 8;
      if (ncol <= c0) break;   // warp-uniform
      float4 gv[8];   // the chunk's G entries, all loads issued before the first use
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (r < ns && c0 + c < ncol) gv[c] = G[r + (size_t)ns * (col0 + c0 + c)];
      float re[3][8], im[3][8];
#pragma unroll
      for (int l = 0; l < 3; ++l) {
        um_ld8_nw(tbase + l * 64 + hf * 16 + c0, re[l]);
        um_ld8_nw(tbase + l * 64 + 32 + hf * 16 + c0, im[l]);
      }
      um_wait_ld();
      if (r < ns) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c0 + c >= ncol) continue;
          const float4 g = gv[c];
          const df vr = oz_combine(re[0][c], re[1][c], re[2][c]);
          const df vi = oz_combine(im[0][c], im[1][c], im[2][c]);
          const df nr = df_add(df{g.x, g.z}, vr), ni = df_add(df{g.y, g.w}, vi);
          G[r + (size_t)ns * (col0 + c0 + c)] = make_float4(nr.hi, ni.hi, nr.lo, ni.lo);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(d.err, PQMC_ERR_TIMEOUT);
  }
  um_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(taddr) : "memory");
}

// ---------------------------------------------------------------------------
// k_xflushp: the flush G += X Z as a pipeline.  A CTA takes one 128-row tile
// of G and a range of its 32-column tiles (nsplit ranges per row tile).  The
// X slices of the row tile (5 slices x 2 halves of the inner dimension, at
// most 160 KB) stay resident in shared memory; the Z slices stream through
// three stages of a quarter of the inner dimension (20 KB each), and the
// three level accumulators of a tile alternate between two tensor-memory
// buffers (2 x 3 x 64 of 512 columns), so that one tile's epilogue (the G
// read-modify-write) overlaps the next tile's copies and products.
// Warps 0-7: epilogue (lane quarter warp & 3, 16 columns each); warp 8,
// lane 0: the bulk copies; warp 9, lane 0: the products.  The stages and
// the product order are those of k_xflush2, so the two give the same G bit
// for bit.  Every wait is bounded; a role that gives up sets the CTA's fail
// flag and the others stop at their next wait.
constexpr int XP_HS = 8 * 16 * 128;                 // one A slice half: 8 k groups x 16 row groups (16 KB)
constexpr int XP_A = OZ_S * 2 * XP_HS;              // resident A: 160 KB
static_assert(OZ_S * 2 * XP_HS + 3 * OZ_S * XF_B + 2048 <= 227 * 1024, "shared memory");
constexpr int XP_ST = OZ_S * XF_B;                  // one B stage: 5 slices x 4 k groups x 8 row groups (20 KB)
constexpr int XP_NB = 3;                            // B stages in flight
constexpr int XP_SMEM = XP_A + XP_NB * XP_ST;       // 220 KB
constexpr int XP_EPI = 8;                           // epilogue warps
constexpr int XP_THREADS = (XP_EPI + 2) * 32;
constexpr uint32_t XP_TBUF = 256;                   // tensor-memory columns per accumulator buffer

__global__ void __launch_bounds__(XP_THREADS, 1) k_xflushp(const XDesc* X, int parity, int nsplit) {
  __shared__ XDesc sd;
  __shared__ __align__(8) uint64_t s_afull, s_bfull[XP_NB], s_bempty[XP_NB], s_tfull[2], s_tempty[2], s_done;
  __shared__ uint32_t s_taddr;
  __shared__ volatile int s_fail;
  extern __shared__ __align__(1024) unsigned char xp_dyn[];   // resident A, then XP_NB B stages
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int RT0 = (int)gridDim.x / nsplit;                   // row tiles (the grid is RT x nsplit)
  const int ti = (int)blockIdx.x % RT0, sp = (int)blockIdx.x / RT0;
  if (tid == 0) {
    sd = X[blockIdx.y];
    s_fail = 0;
    mbar_init(&s_afull, 1);
    for (int b = 0; b < XP_NB; ++b) {
      mbar_init(&s_bfull[b], 1);
      mbar_init(&s_bempty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&s_tfull[b], 1);
      mbar_init(&s_tempty[b], XP_EPI);
    }
    mbar_init(&s_done, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const XDesc& d = sd;
  const int K = *d.kcount;
  const int ns = d.ns, CT = oz_ztiles(ns);
  const int tj0 = sp * CT / nsplit, tj1 = (sp + 1) * CT / nsplit, ntile = tj1 - tj0;
  if (K == 0 || ntile <= 0) return;   // uniform: no tensor memory taken
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&s_taddr))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const uint32_t taddr = s_taddr;
  const int nrg_a = um_rg(ns, ti);
  const int nkg = ((K + 15) & ~15) / 8;       // k groups of one half (even, <= 8)
  const int nq = (nkg + XF_QK - 1) / XF_QK;   // stages per half (1 or 2)
  const int nst = 2 * nq;                     // stages per tile
  const uint32_t ka = (uint32_t)nrg_a * 128, kb = 8u * 128u;   // bytes per k group of A and of B
  if (warp == XP_EPI) {
    // ---- copies ----
    if (lane == 0) {
      if (blockIdx.x == 0 && blockIdx.y == 0) atomicAdd(d.nflush, 1ull);
      mbar_arrive_tx(&s_afull, (uint32_t)(OZ_S * 2 * nkg) * ka);
      for (int sl = 0; sl < OZ_S; ++sl)
        for (int h = 0; h < 2; ++h)
          bulk_g2s(xp_dyn + (size_t)(sl * 2 + h) * XP_HS,
                   d.img + (size_t)oz_slot_a2(ns, ti, sl) * UM_IMG + (size_t)h * (UM_KP / 8) * ka, (uint32_t)nkg * ka,
                   &s_afull);
      const int total = ntile * nst;
      int last = -1;   // the last stage issued
      for (int g = 0; g < total && !s_fail; ++g) {
        const int buf = g % XP_NB, u = g / XP_NB;
        if (u >= 1 && !mbar_wait_bounded(&s_bempty[buf], (u - 1) & 1)) {
          s_fail = 1;
          break;
        }
        const int tj = tj0 + g / nst, sidx = g % nst, h = sidx / nq, qk = sidx % nq;
        const int nk = min(XF_QK, nkg - XF_QK * qk);
        unsigned char* dst = xp_dyn + XP_A + (size_t)buf * XP_ST;
        mbar_arrive_tx(&s_bfull[buf], (uint32_t)(OZ_S * nk) * kb);
        for (int sl = 0; sl < OZ_S; ++sl)
          bulk_g2s(dst + (size_t)sl * XF_B,
                   d.img + (size_t)oz_slot_b2(ns, tj, sl) * UM_IMG + (size_t)(h * (UM_KP / 8) + XF_QK * qk) * kb,
                   (uint32_t)nk * kb, &s_bfull[buf]);
        last = g;
      }
      // copies still in flight complete before the CTA exits: the last
      // XP_NB stages issued, one per buffer
      mbar_wait_bounded(&s_afull, 0);
      for (int g = max(0, last - XP_NB + 1); g <= last; ++g) mbar_wait_bounded(&s_bfull[g % XP_NB], (g / XP_NB) & 1);
    }
  } else if (warp == XP_EPI + 1) {
    // ---- products ----
    if (lane == 0) {
      const uint32_t base = smem_addr(xp_dyn), idesc = um_idesc(64u);
      if (!mbar_wait_bounded(&s_afull, 0)) s_fail = 1;
      um_fence_after();
      int g = 0;
      for (int lt = 0; lt < ntile && !s_fail; ++lt) {
        const int tb = lt & 1, v = lt >> 1;
        if (v >= 1) {
          if (!mbar_wait_bounded(&s_tempty[tb], (v - 1) & 1)) {
            s_fail = 1;
            break;
          }
          um_fence_after();
        }
        const uint32_t tacc = taddr + (uint32_t)tb * XP_TBUF;
        uint32_t started = 0;
        for (int sidx = 0; sidx < nst && !s_fail; ++sidx, ++g) {
          const int buf = g % XP_NB, u = g / XP_NB, h = sidx / nq, qk = sidx % nq;
          const int nk = min(XF_QK, nkg - XF_QK * qk);
          if (!mbar_wait_bounded(&s_bfull[buf], u & 1)) {
            s_fail = 1;
            break;
          }
          um_fence_after();
          const uint32_t bbase = base + XP_A + (uint32_t)buf * XP_ST;
          for (int i = 0; i < OZ_S; ++i)
            for (int j = 0; i + j < OZ_S; ++j) {
              const int l = min(i + j, 2);
              for (int kk = 0; kk < nk / 2; ++kk) {
                const uint64_t ad =
                    um_desc(base + (uint32_t)(i * 2 + h) * XP_HS + (uint32_t)(XF_QK * qk + 2 * kk) * ka, ka, 128);
                const uint64_t bd = um_desc(bbase + (uint32_t)j * XF_B + (uint32_t)(2 * kk) * kb, kb, 128);
                um_mma(tacc + (uint32_t)(l * 64), ad, bd, idesc, (started >> l) & 1u);
                started |= 1u << l;
              }
            }
          um_commit(&s_bempty[buf]);   // the stage's buffer is free once these products finish
        }
        if (!s_fail) um_commit(&s_tfull[tb]);   // the tile's accumulators are complete
      }
      // every product issued has finished before the tensor memory goes
      um_commit(&s_done);
      mbar_wait_bounded(&s_done, 0);
    }
  } else {
    // ---- epilogue: G += the tile's level sums, 16 columns per warp ----
    const int q = warp & 3, hf = warp >> 2;
    const int r = ti * 128 + q * 32 + lane;
    float4* G = parity ? d.g_alt : d.g;
    const uint32_t tl = taddr + ((uint32_t)(q * 32) << 16);
    for (int lt = 0; lt < ntile; ++lt) {
      const int tb = lt & 1, v = lt >> 1;
      const int col0 = (tj0 + lt) * 32 + hf * 16, ncol = min(16, ns - col0);
      // this tile's 16 G entries of the row, loaded while its products run
      // (all issued before the first use: 16 loads in flight, not a chain of
      // load-add-store)
      float4 gv[16];
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (r < ns && c < ncol) gv[c] = G[r + (size_t)ns * (col0 + c)];
      if (s_fail || !mbar_wait_bounded(&s_tfull[tb], v & 1)) {
        s_fail = 1;
        break;
      }
      um_fence_after();
      const uint32_t tacc = tl + (uint32_t)tb * XP_TBUF;
#pragma unroll
      for (int ch = 0; ch < 2; ++ch) {
        const int c0 = ch * 8;
        if (ncol <= c0) break;   // warp-uniform
        float re[3][8], im[3][8];
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          um_ld8_nw(tacc + l * 64 + hf * 16 + c0, re[l]);
          um_ld8_nw(tacc + l * 64 + 32 + hf * 16 + c0, im[l]);
        }
        um_wait_ld();
        if (r < ns) {
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            if (c0 + c >= ncol) continue;
            const float4 g = gv[c0 + c];
            const df vr = oz_combine(re[0][c], re[1][c], re[2][c]);
            const df vi = oz_combine(im[0][c], im[1][c], im[2][c]);
            const df nr = df_add(df{g.x, g.z}, vr), ni = df_add(df{g.y, g.w}, vi);
            G[r + (size_t)ns * (col0 + c0 + c)] = make_float4(nr.hi, ni.hi, nr.lo, ni.lo);
          }
        }
      }
      um_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&s_tempty[tb])) : "memory");
    }
  }
  __syncthreads();
  if (tid == 0 && s_fail) atomicExch(d.err, PQMC_ERR_TIMEOUT);
  um_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(taddr) : "memory");
}

int exact_setup() {
  PQMC_CUDA(raise_dyn_smem(k_xinv, (int)XI_SMEM));
  PQMC_CUDA(raise_dyn_smem(k_xres, (int)XR_SMEM));
  PQMC_CUDA(raise_dyn_smem(k_xgemm<0>, XG_SMEM));
  PQMC_CUDA(raise_dyn_smem(k_xgemm<1>, XG_SMEM));
  PQMC_CUDA(raise_dyn_smem(k_xflush2, XF_SMEM_LAUNCH));
  PQMC_CUDA(raise_dyn_smem(k_xflushp, XP_SMEM));
  return PQMC_OK;
}

int exact_core(const XDesc* d_x, int C, int ns, int dim, int parity, int ct, cudaStream_t st, bool prio,
               int prio_hi) {
  const int n_r = (ns + XS_ROWS - 1) / XS_ROWS, n_c = (ns + XS_COLS - 1) / XS_COLS;
  const int zw = ct == 64 ? 64 : 32;   // Z's tile width: 64 for k_xgemm<1>, 32 for k_xflush2 and k_xflushp
  PQMC_CUDA(launch_at(k_xslice, dim3(n_r + n_c, C), dim3(XS_THREADS), 0, st, prio, prio_hi, d_x, parity, n_r, zw));
  PQMC_LAUNCHED();
  PQMC_CUDA(launch_at(k_xinv, dim3(1, C), dim3(XC_THREADS), XI_SMEM, st, prio, prio_hi, d_x, dim, parity));
  PQMC_LAUNCHED();
  PQMC_CUDA(launch_at(k_xres, dim3(XR_CTAS, C), dim3(XR_THREADS), XR_SMEM, st, prio, prio_hi, d_x, dim, parity));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int exact_products(const XDesc* d_x, int C, int ns, int parity, int ct, cudaStream_t st, bool prio, int prio_hi) {
  const int RT = um_rtiles(ns);
  PQMC_CUDA(launch_at(k_xgemm<0>, dim3(RT, C), dim3(XG_THREADS), (size_t)XG_SMEM, st, prio, prio_hi, d_x, parity));
  PQMC_LAUNCHED();
  if (ct == 1 || ct == 2)   // the pipeline: ct ranges of Z tiles per row tile
    PQMC_CUDA(launch_at(k_xflushp, dim3(RT * ct, C), dim3(XP_THREADS), (size_t)XP_SMEM, st, prio, prio_hi, d_x,
                        parity, ct));
  else if (ct == 32)
    PQMC_CUDA(launch_at(k_xflush2, dim3(RT * oz_ztiles(ns), C), dim3(256), (size_t)XF_SMEM_LAUNCH, st, prio, prio_hi,
                        d_x, parity));
  else
    PQMC_CUDA(launch_at(k_xgemm<1>, dim3(RT * um_ctiles(ns), C), dim3(XG_THREADS), (size_t)XG_SMEM, st, prio,
                        prio_hi, d_x, parity));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

}  // namespace pqmc

// ---------------------------------------------------------------------------
// pqmc_exact_update_check: the exact round update of one round applied to a
// G given on the host (validation entry point, see include/pqmc_gb300.h).
namespace pqmc {
__global__ void k_x_to_df(const cplx* a, float4* b, long n) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    b[e] = dg_make(a[e]);
}
__global__ void k_x_from_df(const float4* a, cplx* b, long n) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    b[e] = dg_to_d(a[e]);
}
}  // namespace pqmc

extern "C" int pqmc_exact_update_check(int ns, int k, int dim, const int* sites, const double* delta, double* g) {
  return pqmc_exact_update_check_tile(ns, k, dim, sites, delta, g, 64);
}

extern "C" int pqmc_exact_update_check_tile(int ns, int k, int dim, const int* sites, const double* delta, double* g,
                                            int flush_tile) {
  using namespace pqmc;
  if (!sites || !delta || !g || dim < 1 || dim > 4 || k < dim || k > UM_KP || k % dim || ns < k ||
      ns > 4096 || (flush_tile != 32 && flush_tile != 64 && flush_tile != 1 && flush_tile != 2)) {
    set_error("exact_update_check: need 1 <= dim <= 4, dim <= k <= %d, k %% dim == 0, k <= ns <= 4096, "
              "flush tile 64, 32, 2 or 1", UM_KP);
    return PQMC_ERR_ARG;
  }
  for (int i = 0; i < k; ++i)
    if (sites[i] < 0 || sites[i] >= ns) {
      set_error("exact_update_check: site %d out of range", sites[i]);
      return PQMC_ERR_ARG;
    }
  PQMC_TRY(exact_setup());
  const size_t n2 = (size_t)ns * ns;
  const int nb = k / dim;
  cplx* d_g64 = nullptr;
  float4* d_g = nullptr;
  int* d_site = nullptr;
  float4* d_dl = nullptr;
  float4* d_w = nullptr;
  float2* d_v0 = nullptr;
  int* d_k = nullptr;
  unsigned char* d_img = nullptr;
  DevScalars* d_sc = nullptr;
  int* d_err = nullptr;
  unsigned long long* d_nf = nullptr;
  XDesc* d_x = nullptr;
  int st = PQMC_OK;
  auto run = [&]() -> int {
    PQMC_CUDA(cudaMalloc((void**)&d_g64, sizeof(cplx) * n2));
    PQMC_CUDA(cudaMalloc((void**)&d_g, sizeof(float4) * n2));
    PQMC_CUDA(cudaMalloc((void**)&d_site, sizeof(int) * k));
    PQMC_CUDA(cudaMalloc((void**)&d_dl, sizeof(float4) * 16 * nb));
    PQMC_CUDA(cudaMalloc((void**)&d_w, sizeof(float4) * UM_KP * UM_KP));
    PQMC_CUDA(cudaMalloc((void**)&d_v0, sizeof(float2) * UM_KP * UM_KP));
    PQMC_CUDA(cudaMalloc((void**)&d_k, sizeof(int)));
    PQMC_CUDA(cudaMalloc((void**)&d_img, oz_chain_bytes(ns)));
    PQMC_CUDA(cudaMalloc((void**)&d_sc, sizeof(DevScalars)));
    PQMC_CUDA(cudaMalloc((void**)&d_err, sizeof(int)));
    PQMC_CUDA(cudaMalloc((void**)&d_nf, sizeof(unsigned long long)));
    PQMC_CUDA(cudaMalloc((void**)&d_x, sizeof(XDesc)));
    PQMC_CUDA(cudaMemset(d_img, 0, oz_chain_bytes(ns)));
    PQMC_CUDA(cudaMemset(d_sc, 0, sizeof(DevScalars)));
    PQMC_CUDA(cudaMemset(d_err, 0, sizeof(int)));
    PQMC_CUDA(cudaMemset(d_nf, 0, sizeof(unsigned long long)));
    PQMC_CUDA(cudaMemcpy(d_g64, g, sizeof(cplx) * n2, cudaMemcpyHostToDevice));
    PQMC_CUDA(cudaMemcpy(d_site, sites, sizeof(int) * k, cudaMemcpyHostToDevice));
    PQMC_CUDA(cudaMemcpy(d_k, &k, sizeof(int), cudaMemcpyHostToDevice));
    // Delta blocks (dim x dim, column-major, FP64 complex) -> 16-entry double-float records
    std::vector<cplx> dl((size_t)16 * nb, mk(0.0));
    for (int b = 0; b < nb; ++b)
      for (int e = 0; e < dim * dim; ++e)
        dl[(size_t)16 * b + e] = mk(delta[2 * ((size_t)b * dim * dim + e)], delta[2 * ((size_t)b * dim * dim + e) + 1]);
    cplx* d_dl64 = nullptr;
    PQMC_CUDA(cudaMalloc((void**)&d_dl64, sizeof(cplx) * dl.size()));
    PQMC_CUDA(cudaMemcpy(d_dl64, dl.data(), sizeof(cplx) * dl.size(), cudaMemcpyHostToDevice));
    k_x_to_df<<<64, 256>>>(d_dl64, d_dl, (long)dl.size());
    PQMC_LAUNCHED();
    k_x_to_df<<<256, 256>>>(d_g64, d_g, (long)n2);
    PQMC_LAUNCHED();
    XDesc x;
    memset(&x, 0, sizeof(x));
    x.g = d_g;
    x.g_alt = d_g;
    x.ns = ns;
    x.ncopy = 1;
    x.tr_weight = 0;
    x.kmax = UM_KP;
    x.kcount = d_k;
    x.acc_site = d_site;
    x.acc_delta = d_dl;
    x.wdf = d_w;
    x.v0 = d_v0;
    x.img = d_img;
    x.sc = d_sc;
    x.err = d_err;
    x.nflush = d_nf;
    PQMC_CUDA(cudaMemcpy(d_x, &x, sizeof(XDesc), cudaMemcpyHostToDevice));
    PQMC_TRY(exact_core(d_x, 1, ns, dim, 0, flush_tile, 0, false, 0));
    PQMC_TRY(exact_products(d_x, 1, ns, 0, flush_tile, 0, false, 0));
    k_x_from_df<<<256, 256>>>(d_g, d_g64, (long)n2);
    PQMC_LAUNCHED();
    PQMC_CUDA(cudaDeviceSynchronize());
    cudaFree(d_dl64);
    int herr = 0;
    PQMC_CUDA(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr != 0) {
      set_error("exact_update_check: device error %d", herr);
      return herr;
    }
    PQMC_CUDA(cudaMemcpy(g, d_g64, sizeof(cplx) * n2, cudaMemcpyDeviceToHost));
    return PQMC_OK;
  };
  st = run();
  cudaFree(d_g64);
  cudaFree(d_g);
  cudaFree(d_site);
  cudaFree(d_dl);
  cudaFree(d_w);
  cudaFree(d_v0);
  cudaFree(d_k);
  cudaFree(d_img);
  cudaFree(d_sc);
  cudaFree(d_err);
  cudaFree(d_nf);
  cudaFree(d_x);
  return st;
}
