// batch.cu -- many independent chains in one device context (replica
// parallelism of src/Main_PQMC.f90:373-443 without MPI), advanced together
// one family step at a time.
//
// Mixed-precision family step (one launch per phase for all chains):
//   k_bdraw   ran2 stream of every chain for the step
//   k_bprep   per-plaquette proposal data (as phase 1 of k_update)
//   k_bscan   one CTA per chain walks its plaquettes in Markov order; an
//             accepted move appends a rank-dim column block to the FP32
//             delayed-update panels A (Ns x K) and B (K x Ns), so later
//             ratios see G + A B without touching G (delayed updates)
//   k_bflush  G += A B for every chain: split-BF16 tensor-core products
//             (3 bf16 terms per operand, 6 cross products) accumulated in
//             FP32, added to the FP64 G
//   k_bwrap   two-way wrap G <- A G B by the family: the FP32 correction
//             (A-I)(G B) + G (B-I) added to the FP64 G
// FP64 stays in G itself, in the 4x4 ratio / T = Delta R^-1 of accepted
// moves, and in the stabilised recompute and log-weight.
#include <cuda_bf16.h>
#include <string.h>
#include <vector>
#include "chain.cuh"
#include "linalg.cuh"
#include "rng.cuh"
#include "update_dev.cuh"
#include "recompute_b.cuh"

namespace pqmc {

struct BDesc {
  DevModel M;
  double* field;
  cplx* expkv;
  cplx* expkv_inv;
  cplx* g;       // parity 0 buffer
  cplx* g_alt;   // parity 1 buffer
  float2* A;     // (kmax, ns): A[q*ns + r]
  float2* B;     // (kmax, ns): B[q*ns + c]
  int kmax;
  int pad;
  PlaqPre* pre;
  DevScalars* sc;
  int* kcount;
  const int* wpla;   // wrap cover items of the family loop (per family, see host)
  const int* wsites;
  const int* wdim;
};

__device__ __forceinline__ float2 f2(cplx a) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ float2 fm(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 fa(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsb(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// ---------------------------------------------------------------------------
__global__ void k_bdraw(BDesc* D, int C, int pf) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const BDesc d = D[c];
  const int npla = d.M.pf_npla[pf];
  Ran2Dev rng;
  rng.iran = d.sc->rng[0]; rng.jran = d.sc->rng[1]; rng.kran = d.sc->rng[2];
  rng.mran = d.sc->rng[3]; rng.nran = d.sc->rng[4];
  for (int p = 0; p < npla; ++p) {
    if (d.M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
      d.pre[p].xnew = (double)rng.next();
      d.pre[p].dE = (double)rng.next();
    } else {
      d.pre[p].xnew = (double)rng.ran_sysm();
    }
    d.pre[p].r = (double)rng.next();
  }
  d.sc->rng[0] = rng.iran; d.sc->rng[1] = rng.jran; d.sc->rng[2] = rng.kran;
  d.sc->rng[3] = rng.mran; d.sc->rng[4] = rng.nran;
}

__device__ __forceinline__ double b_threshold(const DevModel& M, double dE, double r) {
  const int n = M.ncopy * (M.tr_weight ? 2 : 1);
  double q;
  if (M.metropolis) {
    q = M.greatest_decent ? exp(-dE) : r * exp(-dE);
  } else {
    double rr = r / (1.0 - r);
    if (!(rr <= exp(10.0))) return INFINITY;
    q = rr * exp(-dE);
  }
  if (n == 1) return q * q;
  if (n == 2) return q;
  return pow(q, 2.0 / n);
}

__global__ void __launch_bounds__(256) k_bprep(const BDesc* D, int pf, int t) {
  __shared__ BDesc sd;
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const BDesc& d = sd;
  const DevModel& M = d.M;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int npla = M.pf_npla[pf], dim = M.pf_dim[pf], pd = M.pdim;
  const int p = blockIdx.x * (blockDim.x >> 5) + warp;
  if (p >= npla) return;
  PlaqPre* pre = d.pre;
  const double* field = d.field;
  const bool closed = (M.expkv_kind != PQMC_EXPKV_GENERAL);
  const int b = M.bf[p + M.max_pla * pf];
  double jump;
  if (M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
    double u1 = pre[p].xnew, u2 = pre[p].dE;
    jump = M.jump * (sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
  } else {
    jump = M.jump * pre[p].xnew;
  }
  double xnew = field[b + (size_t)M.n_bf * t] + jump;
  double norm = 0.0, ch = 0.0, sh = 0.0;
  __syncwarp();
  if (lane == 0) {
    double dE = -M.delt * energy_diff(M, field, b, t, jump);
    pre[p].dE = dE;
    pre[p].thr = b_threshold(M, dE, pre[p].r);
    if (closed) {
      norm = closed_norm(M, pf, xnew);
      ch = cosh(norm);
      sh = sinh(norm);
    } else {
      dev_get_expkv(M, pf, p, xnew, false, pre[p].enew);
      dev_get_expkv(M, pf, p, xnew, true, pre[p].einv);
    }
  }
  norm = __shfl_sync(0xffffffffu, norm, 0);
  ch = __shfl_sync(0xffffffffu, ch, 0);
  sh = __shfl_sync(0xffffffffu, sh, 0);
  const int i = lane % dim, j = lane / dim;
  const bool act = lane < dim * dim;
  cplx en = mk(0.0);
  if (act) {
    if (closed) {
      en = closed_entry(M, pf, p, xnew, false, i, j, norm, ch, sh);
      pre[p].enew[lane] = en;
      pre[p].einv[lane] = closed_entry(M, pf, p, xnew, true, i, j, norm, ch, sh);
    } else {
      en = pre[p].enew[lane];
    }
  }
  __syncwarp();
  const size_t base = M.kv_base(p, pf, t);
  cplx a = mk(0.0);
  for (int k = 0; k < dim; ++k) {
    cplx ekj = shfl_c(en, k + dim * j);
    if (act) a = cadd(a, cmul(d.expkv_inv[base + i + pd * k], ekj));
  }
  if (act) {
    if (i == j) a = csub(a, mk(1.0));
    pre[p].delta[lane] = a;
    pre[p].deltaf[lane] = make_float2((float)a.x, (float)a.y);
  }
  if (lane == 0) pre[p].xnew = xnew;
}

// ---------------------------------------------------------------------------
// Sequential scan with delayed updates, one CTA per chain.  The scan resumes
// at the chain's next plaquette and stops when the panels hold `kd` columns
// (the delay depth); k_bflush then folds them into G and the next round
// continues.  Ratios, R^-1 and T are FP32 (the panels are FP32); the weight
// ln_cw is accumulated in FP64.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_KSTAGE = 512;   // max delay depth (panel columns)

__device__ __forceinline__ float2 fdiv1(float2 a) {   // 1/a
  float n = a.x * a.x + a.y * a.y;
  return make_float2(a.x / n, -a.y / n);
}

// 4x4 (or smaller) complex inverse in FP32 by Gauss-Jordan with partial
// pivoting on one thread
__device__ void finv_small(int n, float2* a) {
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

__device__ float2 fdet_small(int n, const float2* a) {
  if (n == 1) return a[0];
  if (n == 2) return fsb(fm(a[0], a[3]), fm(a[2], a[1]));
  // Gauss elimination with partial pivoting on a copy
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

__global__ void __launch_bounds__(SCAN_THREADS) k_bscan(const BDesc* D, int pf, int t, int parity, int kd, int* next_p) {
  __shared__ BDesc sd;
  if (threadIdx.x == 0) sd = D[blockIdx.x];
  __syncthreads();
  const BDesc& d = sd;
  const DevModel& M = d.M;
  const int ns = M.ns, npla = M.pf_npla[pf], dim = M.pf_dim[pf], pd = M.pdim;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int p0 = next_p[blockIdx.x];
  if (p0 >= npla) {
    if (tid == 0) *d.kcount = 0;
    return;
  }
  const cplx* G = parity ? d.g_alt : d.g;
  float2* A = d.A;
  float2* B = d.B;
  PlaqPre* pre = d.pre;
  __shared__ int s_S[4];
  __shared__ float2 s_g[16], s_r[16], s_T[16];
  __shared__ int s_dec;
  __shared__ float2 s_BS[4 * SCAN_KSTAGE];   // B(q, S_m)
  __shared__ float2 s_AS[4 * SCAN_KSTAGE];   // A(S_l, q)
  int K = 0;
  double lprod = 1.0;
  long long lexp = 0, pa = 0, na = 0;
  int p = p0;
  for (; p < npla; ++p) {
    if (K + dim > kd) break;
    if (tid < dim) s_S[tid] = M.site[tid + pd * (p + M.max_pla * pf)];
    __syncthreads();
    // stage A(S,:), B(:,S) for q < K (one round trip), and G(S,S)
    for (int e = tid; e < K * dim; e += blockDim.x) {
      int q = e / dim, m = e % dim;
      s_BS[e] = B[(size_t)q * ns + s_S[m]];
      s_AS[e] = A[(size_t)q * ns + s_S[m]];
    }
    if (tid < dim * dim) s_g[tid] = f2(G[s_S[tid % dim] + (size_t)ns * s_S[tid / dim]]);
    __syncthreads();
    const PlaqPre* pp = pre + p;
    if (warp == 0) {
      const int i = lane % dim, j = lane / dim;
      const bool act = lane < dim * dim;
      // G_eff(S,S) = G(S,S) + (A B)(S,S)
      float2 gv = make_float2(0.f, 0.f);
      if (act) {
        gv = s_g[lane];
        for (int q = 0; q < K; ++q) gv = fa(gv, fm(s_AS[q * dim + i], s_BS[q * dim + j]));
      }
      __syncwarp();
      if (act) s_g[lane] = gv;
      __syncwarp();
      // R = I + G_eff(S,S) Delta
      if (act) {
        float2 a = make_float2(i == j ? 1.f : 0.f, 0.f);
        for (int k = 0; k < dim; ++k) a = fa(a, fm(s_g[i + dim * k], pp->deltaf[k + dim * j]));
        s_r[lane] = a;
      }
      __syncwarp();
      int acc = 0;
      if (lane == 0) {
        float2 det = fdet_small(dim, s_r);
        double d2 = (double)det.x * det.x + (double)det.y * det.y;
        acc = d2 >= pp->thr;
        if (acc) {
          pa++;
          double relr;
          {
            double dr = det.x, di = det.y;
            double rr = dr, ri = di;
            if (M.tr_weight) { rr = dr * dr + di * di; ri = 0.0; }
            double ar = 1.0, ai = 0.0;
            for (int k = 0; k < M.ncopy; ++k) {
              double tr = ar * rr - ai * ri;
              ai = ar * ri + ai * rr;
              ar = tr;
            }
            relr = ar;
          }
          int ex;
          lprod *= frexp(relr, &ex);
          lexp += ex;
          lprod = frexp(lprod, &ex);
          lexp += ex;
          d.field[M.bf[p + M.max_pla * pf] + (size_t)M.n_bf * t] = pp->xnew;
          finv_small(dim, s_r);   // R^-1
        } else {
          na++;
        }
      }
      acc = __shfl_sync(0xffffffffu, acc, 0);
      __syncwarp();
      if (acc) {
        if (act) {
          float2 a = make_float2(0.f, 0.f);
          for (int k = 0; k < dim; ++k) a = fa(a, fm(pp->deltaf[i + dim * k], s_r[k + dim * j]));
          s_T[lane] = a;
        }
        const size_t base2 = M.kv_base(p, pf, t);
        if (lane < pd * pd) {
          int ii = lane % pd, jj = lane / pd;
          bool in = ii < dim && jj < dim;
          d.expkv[base2 + lane] = in ? pp->enew[ii + dim * jj] : mk(0.0);
          d.expkv_inv[base2 + lane] = in ? pp->einv[ii + dim * jj] : mk(0.0);
        }
      }
      if (lane == 0) s_dec = acc;
    }
    __syncthreads();
    if (!s_dec) continue;
    // new panel block: a(r,l) = sum_m Geff(r,S_m) T(m,l),  b(l,c) = delta(S_l,c) - Geff(S_l,c)
    for (int r = tid; r < ns; r += blockDim.x) {
      float2 gm[4], bl[4];
      for (int m = 0; m < dim; ++m) {
        gm[m] = f2(G[r + (size_t)ns * s_S[m]]);
        bl[m] = f2(G[s_S[m] + (size_t)ns * r]);
      }
#pragma unroll 4
      for (int q = 0; q < K; ++q) {
        float2 ar = A[(size_t)q * ns + r];
        float2 bc = B[(size_t)q * ns + r];
        for (int m = 0; m < dim; ++m) {
          gm[m] = fa(gm[m], fm(ar, s_BS[q * dim + m]));
          bl[m] = fa(bl[m], fm(s_AS[q * dim + m], bc));
        }
      }
      for (int l = 0; l < dim; ++l) {
        float2 a = make_float2(0.f, 0.f);
        for (int m = 0; m < dim; ++m) a = fa(a, fm(gm[m], s_T[m + dim * l]));
        A[(size_t)(K + l) * ns + r] = a;
        float2 bv = make_float2(-bl[l].x, -bl[l].y);
        if (r == s_S[l]) bv.x += 1.f;
        B[(size_t)(K + l) * ns + r] = bv;
      }
    }
    K += dim;
    __syncthreads();
  }
  if (tid == 0) {
    *d.kcount = K;
    next_p[blockIdx.x] = p;
    if (pa > 0) {
      double l = (lprod > 0.0) ? log(lprod) + (double)lexp * 0.69314718055994530942 : log(lprod);
      d.sc->ln_cw = cadd(d.sc->ln_cw, mk(l));
    }
    d.sc->pos_acc += pa;
    d.sc->neg_acc += na;
  }
}

// ---------------------------------------------------------------------------
// G += A B with split-BF16 tensor-core products (mma.sync m16n8k16, FP32
// accumulators), 64x64 complex output tile per CTA, 8 warps of 16x32.
constexpr int FB_M = 64, FB_N = 64, FB_K = 16, FB_LD = 24;

__device__ __forceinline__ void split3(float x, __nv_bfloat16* o) {
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  float r1 = x - __bfloat162float(h);
  __nv_bfloat16 m = __float2bfloat16_rn(r1);
  float r2 = r1 - __bfloat162float(m);
  o[0] = h;
  o[1] = m;
  o[2] = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(256) k_bflush(const BDesc* D, int parity) {
  __shared__ BDesc sd;
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const BDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;
  const int ns = d.M.ns;
  const int tiles_m = (ns + FB_M - 1) / FB_M, tiles_n = (ns + FB_N - 1) / FB_N;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  if (tn >= tiles_n) return;
  cplx* G = parity ? d.g_alt : d.g;
  // As[split][comp re,im][m][k], Bs[split][comp re,im,-im][n][k]
  __shared__ __align__(16) __nv_bfloat16 As[3][2][FB_M][FB_LD];
  __shared__ __align__(16) __nv_bfloat16 Bs[3][3][FB_N][FB_LD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;   // 4 x 2 warps
  const int g = lane >> 2, tq = lane & 3;
  float acc[4][2][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 4; ++e) acc[a][b][e] = 0.f;
  const int row0 = tm * FB_M, col0 = tn * FB_N;
  for (int k0 = 0; k0 < K; k0 += FB_K) {
    for (int e = tid; e < FB_M * FB_K; e += 256) {
      int r = e % FB_M, q = e / FB_M;
      float2 v = make_float2(0.f, 0.f);
      if (row0 + r < ns && k0 + q < K) v = d.A[(size_t)(k0 + q) * ns + row0 + r];
      __nv_bfloat16 sp[3];
      split3(v.x, sp);
      As[0][0][r][q] = sp[0]; As[1][0][r][q] = sp[1]; As[2][0][r][q] = sp[2];
      split3(v.y, sp);
      As[0][1][r][q] = sp[0]; As[1][1][r][q] = sp[1]; As[2][1][r][q] = sp[2];
    }
    for (int e = tid; e < FB_N * FB_K; e += 256) {
      int cix = e % FB_N, q = e / FB_N;
      float2 v = make_float2(0.f, 0.f);
      if (col0 + cix < ns && k0 + q < K) v = d.B[(size_t)(k0 + q) * ns + col0 + cix];
      __nv_bfloat16 sp[3];
      split3(v.x, sp);
      Bs[0][0][cix][q] = sp[0]; Bs[1][0][cix][q] = sp[1]; Bs[2][0][cix][q] = sp[2];
      split3(v.y, sp);
      Bs[0][1][cix][q] = sp[0]; Bs[1][1][cix][q] = sp[1]; Bs[2][1][cix][q] = sp[2];
      Bs[0][2][cix][q] = __hneg(sp[0]); Bs[1][2][cix][q] = __hneg(sp[1]); Bs[2][2][cix][q] = __hneg(sp[2]);
    }
    __syncthreads();
    uint32_t af[3][2][4];
    const int mr = wm * 16;
    for (int s = 0; s < 3; ++s)
      for (int cpt = 0; cpt < 2; ++cpt) {
        af[s][cpt][0] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g][2 * tq]);
        af[s][cpt][1] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g + 8][2 * tq]);
        af[s][cpt][2] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g][2 * tq + 8]);
        af[s][cpt][3] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g + 8][2 * tq + 8]);
      }
    const int SA[6] = {0, 0, 1, 0, 1, 2}, SB[6] = {0, 1, 0, 2, 1, 0};
    for (int nt = 0; nt < 4; ++nt) {
      const int nc = wn * 32 + nt * 8 + g;
      for (int pr = 0; pr < 6; ++pr) {
        const int sa = SA[pr], sb = SB[pr];
        uint32_t br[2], bi[2], bni[2];
        br[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][0][nc][2 * tq]);
        br[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][0][nc][2 * tq + 8]);
        bi[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][1][nc][2 * tq]);
        bi[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][1][nc][2 * tq + 8]);
        bni[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][2][nc][2 * tq]);
        bni[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][2][nc][2 * tq + 8]);
        mma_bf16(acc[nt][0], af[sa][0], br);    // re += Ar Br
        mma_bf16(acc[nt][0], af[sa][1], bni);   // re += Ai (-Bi)
        mma_bf16(acc[nt][1], af[sa][0], bi);    // im += Ar Bi
        mma_bf16(acc[nt][1], af[sa][1], br);    // im += Ai Br
      }
    }
    __syncthreads();
  }
  for (int nt = 0; nt < 4; ++nt)
    for (int e = 0; e < 4; ++e) {
      const int r = row0 + wm * 16 + g + ((e >> 1) ? 8 : 0);
      const int cc = col0 + wn * 32 + nt * 8 + 2 * tq + (e & 1);
      if (r < ns && cc < ns) {
        cplx* p = G + r + (size_t)ns * cc;
        *p = cadd(*p, mk((double)acc[nt][0][e], (double)acc[nt][1][e]));
      }
    }
}

// ---------------------------------------------------------------------------
// Two-way wrap with an FP32 correction on the FP64 G (left: A=expKV, B=expKV_inv).
__global__ void k_bwrap(const BDesc* D, int pf, int t, int left, int n_items, int parity) {
  __shared__ BDesc sd;
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const BDesc& d = sd;
  const long pair = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (pair >= (long)n_items * n_items) return;
  const DevModel& M = d.M;
  const int ir = (int)(pair % n_items), ic = (int)(pair / n_items);
  const int ns = M.ns, pd = M.pdim;
  const int dr = d.wdim[ir], dc = d.wdim[ic];
  const cplx* gin = parity ? d.g_alt : d.g;
  cplx* gout = parity ? d.g : d.g_alt;
  int Sr[4], Sc[4];
  for (int k = 0; k < dr; ++k) Sr[k] = d.wsites[4 * ir + k];
  for (int k = 0; k < dc; ++k) Sc[k] = d.wsites[4 * ic + k];
  cplx gd[16];
  float2 gf[16], gb[16];
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) {
      gd[a + 4 * b] = gin[Sr[a] + (size_t)ns * Sc[b]];
      gf[a + 4 * b] = f2(gd[a + 4 * b]);
    }
  const int pr = d.wpla[ir], pc = d.wpla[ic];
  const cplx* Am = (pr >= 0) ? (left ? d.expkv : d.expkv_inv) + M.kv_base(pr, pf, t) : nullptr;
  const cplx* Bm = (pc >= 0) ? (left ? d.expkv_inv : d.expkv) + M.kv_base(pc, pf, t) : nullptr;
  // gb = G B
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) {
      float2 s = make_float2(0.f, 0.f);
      if (Bm) {
        for (int k = 0; k < dc; ++k) s = fa(s, fm(gf[a + 4 * k], f2(Bm[k + pd * b])));
      } else {
        s = gf[a + 4 * b];
      }
      gb[a + 4 * b] = s;
    }
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) {
      float2 corr = make_float2(0.f, 0.f);
      if (Am)
        for (int k = 0; k < dr; ++k) {
          float2 am = f2(Am[a + pd * k]);
          if (k == a) am.x -= 1.f;
          corr = fa(corr, fm(am, gb[k + 4 * b]));
        }
      if (Bm)
        for (int k = 0; k < dc; ++k) {
          float2 bm = f2(Bm[k + pd * b]);
          if (k == b) bm.x -= 1.f;
          corr = fa(corr, fm(gf[a + 4 * k], bm));
        }
      gout[Sr[a] + (size_t)ns * Sc[b]] = cadd(gd[a + 4 * b], mk((double)corr.x, (double)corr.y));
    }
}

}  // namespace pqmc

// ===========================================================================
struct pqmc_batch {
  std::vector<pqmc_chain*> chains;
  int precision = PQMC_PREC_FP64;
  pqmc::BDesc* d_desc = nullptr;
  std::vector<pqmc::BDesc> h_desc;
  std::vector<float2*> panels;
  std::vector<int*> kcounts;
  int parity = 0;
  int kd = 64;            // delay depth (panel columns per flush)
  int* d_next = nullptr;  // per chain: next plaquette of the current family step
  cudaStream_t stream = nullptr;
  pqmc::BatchRecompute rec;
};

using namespace pqmc;

extern "C" int pqmc_create(const pqmc_model* model, pqmc_chain** out);
extern "C" int pqmc_destroy(pqmc_chain* c);
extern "C" int pqmc_sweep(pqmc_chain* c, int first_loop, int n_sweeps, int warmup, int meas_interval,
                          int meas_number, double* records, int n_records_cap, int* n_records);

static int batch_refresh(pqmc_batch* b) {
  // current G of every chain is c->g; rebuild descriptors, parity 0
  for (size_t i = 0; i < b->chains.size(); ++i) {
    b->h_desc[i].g = b->chains[i]->g;
    b->h_desc[i].g_alt = b->chains[i]->g_alt;
  }
  b->parity = 0;
  PQMC_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), sizeof(BDesc) * b->h_desc.size(), cudaMemcpyHostToDevice,
                            b->stream));
  return PQMC_OK;
}

static int batch_sync_parity(pqmc_batch* b) {
  // make c->g the current buffer of every chain
  if (b->parity) {
    for (auto* c : b->chains) {
      cplx* t = c->g;
      c->g = c->g_alt;
      c->g_alt = t;
    }
  }
  return batch_refresh(b);
}

static int bwrap(pqmc_batch* b, int pf, int time, bool left) {
  pqmc_chain* c0 = b->chains[0];
  const WrapItems& w = c0->wrap[pf];
  // the descriptors carry family 0's cover; point them at this family's
  for (auto& h : b->h_desc) {
    h.wpla = w.d_pla;
    h.wsites = w.d_sites;
    h.wdim = w.d_dim;
  }
  PQMC_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), sizeof(BDesc) * b->h_desc.size(), cudaMemcpyHostToDevice,
                            b->stream));
  long pairs = (long)w.n_items * w.n_items;
  dim3 grid((unsigned)((pairs + 63) / 64), (unsigned)b->chains.size());
  k_bwrap<<<grid, 64, 0, b->stream>>>(b->d_desc, pf, time - 1, left ? 1 : 0, w.n_items, b->parity);
  PQMC_LAUNCHED();
  b->parity ^= 1;
  return PQMC_OK;
}

static int bupdate(pqmc_batch* b, int pf, int time) {
  const int C = (int)b->chains.size();
  pqmc_chain* c0 = b->chains[0];
  const int npla = c0->h_pf_npla[pf], dim = c0->h_pf_dim[pf];
  k_bdraw<<<(C + 63) / 64, 64, 0, b->stream>>>(b->d_desc, C, pf);
  PQMC_LAUNCHED();
  k_bprep<<<dim3((npla + 7) / 8, C), 256, 0, b->stream>>>(b->d_desc, pf, time - 1);
  PQMC_LAUNCHED();
  PQMC_CUDA(cudaMemsetAsync(b->d_next, 0, sizeof(int) * C, b->stream));
  const int kd = std::max(dim, std::min(b->kd, b->h_desc[0].kmax));
  // enough rounds for the worst case (every proposal accepted)
  const int rounds = (npla * dim + (kd / dim) * dim - 1) / ((kd / dim) * dim);
  const int tiles = ((c0->ns + FB_M - 1) / FB_M) * ((c0->ns + FB_N - 1) / FB_N);
  for (int r = 0; r < rounds; ++r) {
    k_bscan<<<C, SCAN_THREADS, 0, b->stream>>>(b->d_desc, pf, time - 1, b->parity, kd, b->d_next);
    PQMC_LAUNCHED();
    k_bflush<<<dim3(tiles, C), 256, 0, b->stream>>>(b->d_desc, b->parity);
    PQMC_LAUNCHED();
  }
  return PQMC_OK;
}

static int bscratch(pqmc_batch* b, int time, bool forward, int loop) {
  (void)loop;
  PQMC_TRY(batch_sync_parity(b));
  PQMC_TRY(b->rec.scratch(time, forward));
  return batch_refresh(b);
}

extern "C" {

int pqmc_batch_create(const pqmc_model* const* models, int n_chains, int precision, pqmc_batch** out) {
  if (!models || !out || n_chains < 1) { set_error("batch_create: bad arguments"); return PQMC_ERR_ARG; }
  if (precision != PQMC_PREC_FP64 && precision != PQMC_PREC_MIXED) {
    set_error("batch_create: unknown precision %d", precision);
    return PQMC_ERR_ARG;
  }
  pqmc_batch* b = new pqmc_batch();
  b->precision = precision;
  for (int i = 0; i < n_chains; ++i) {
    pqmc_chain* c = nullptr;
    int st = pqmc_create(models[i], &c);
    if (st != PQMC_OK) {
      for (auto* x : b->chains) pqmc_destroy(x);
      delete b;
      return st;
    }
    b->chains.push_back(c);
  }
  pqmc_chain* c0 = b->chains[0];
  if (precision == PQMC_PREC_MIXED) {
    for (auto* c : b->chains)
      if (c->ns != c0->ns || c->n_pf != c0->n_pf || c->ntime != c0->ntime || c->ngroup != c0->ngroup ||
          c->h_pf_npla != c0->h_pf_npla || c->h_pf_dim != c0->h_pf_dim) {
        set_error("batch_create: mixed-precision batches need chains of one geometry");
        pqmc_batch_destroy(b);
        return PQMC_ERR_ARG;
      }
  }
  PQMC_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  int kmax = 0;
  for (int f = 0; f < c0->n_pf; ++f) kmax = std::max(kmax, c0->h_pf_npla[f] * c0->h_pf_dim[f]);
  if (kmax > SCAN_KSTAGE) { set_error("batch_create: family too large for the staged panels"); return PQMC_ERR_ARG; }
  b->h_desc.resize(n_chains);
  for (int i = 0; i < n_chains; ++i) {
    pqmc_chain* c = b->chains[i];
    BDesc& h = b->h_desc[i];
    memset(&h, 0, sizeof(h));
    h.M = c->M;
    h.field = c->field;
    h.expkv = c->expkv;
    h.expkv_inv = c->expkv_inv;
    h.g = c->g;
    h.g_alt = c->g_alt;
    h.kmax = kmax;
    h.pre = c->pre;
    h.sc = c->sc;
    float2* pan = nullptr;
    int* kc = nullptr;
    if (precision == PQMC_PREC_MIXED) {
      PQMC_CUDA(cudaMalloc((void**)&pan, sizeof(float2) * (size_t)2 * kmax * c->ns));
      PQMC_CUDA(cudaMalloc((void**)&kc, sizeof(int)));
      h.A = pan;
      h.B = pan + (size_t)kmax * c->ns;
      h.kcount = kc;
    }
    b->panels.push_back(pan);
    b->kcounts.push_back(kc);
  }
  PQMC_CUDA(cudaMalloc((void**)&b->d_desc, sizeof(BDesc) * n_chains));
  PQMC_CUDA(cudaMalloc((void**)&b->d_next, sizeof(int) * n_chains));
  if (precision == PQMC_PREC_MIXED) PQMC_TRY(b->rec.setup(b->chains, b->stream));
  PQMC_TRY(batch_refresh(b));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  *out = b;
  return PQMC_OK;
}

int pqmc_batch_destroy(pqmc_batch* b) {
  if (!b) return PQMC_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto* c : b->chains) pqmc_destroy(c);
  for (auto* p : b->panels)
    if (p) cudaFree(p);
  for (auto* k : b->kcounts)
    if (k) cudaFree(k);
  if (b->d_desc) cudaFree(b->d_desc);
  if (b->d_next) cudaFree(b->d_next);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PQMC_OK;
}

int pqmc_batch_set_delay(pqmc_batch* b, int kd) {
  if (!b || kd < 1 || kd > SCAN_KSTAGE) { set_error("batch_set_delay: depth must be in 1..%d", SCAN_KSTAGE); return PQMC_ERR_ARG; }
  b->kd = kd;
  return PQMC_OK;
}

int pqmc_batch_chain(pqmc_batch* b, int i, pqmc_chain** chain) {
  if (!b || !chain || i < 0 || i >= (int)b->chains.size()) { set_error("batch_chain: bad index"); return PQMC_ERR_ARG; }
  *chain = b->chains[i];
  return PQMC_OK;
}

int pqmc_batch_sweep(pqmc_batch* b, int loop) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  for (auto* c : b->chains)
    if (!c->have_g) { set_error("batch_sweep before init_g"); return PQMC_ERR_STATE; }
  if (b->precision == PQMC_PREC_FP64) {
    for (auto* c : b->chains) PQMC_TRY(pqmc_sweep(c, loop, 1, 1 << 30, 1, 0, nullptr, 0, nullptr));
    return PQMC_OK;
  }
  // every chain finished its own previous work on its stream
  for (auto* c : b->chains) PQMC_CUDA(cudaStreamSynchronize(c->stream));
  PQMC_TRY(batch_refresh(b));
  pqmc_chain* c0 = b->chains[0];
  const bool forward = (loop % 2) == 0;
  for (int tc = 1; tc <= c0->ntime; ++tc) {
    int time;
    if (!forward) {
      time = c0->ntime - tc + 1;
      for (int pf = c0->n_pf - 1; pf >= 0; --pf) {
        PQMC_TRY(bwrap(b, pf, time, false));
        if (c0->M.local_update && c0->h_pf_v_exist[pf]) PQMC_TRY(bupdate(b, pf, time));
      }
    } else {
      time = tc;
      for (int pf = 0; pf < c0->n_pf; ++pf) {
        if (c0->M.local_update && c0->h_pf_v_exist[pf]) PQMC_TRY(bupdate(b, pf, time));
        PQMC_TRY(bwrap(b, pf, time, true));
      }
    }
    if (tc % c0->ngroup == 0) PQMC_TRY(bscratch(b, forward ? time + 1 : time, forward, loop));
  }
  PQMC_TRY(batch_sync_parity(b));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  return PQMC_OK;
}

}  // extern "C"
