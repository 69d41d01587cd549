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
#include <string.h>
#include <vector>
#include "chain.cuh"
#include "df32.cuh"
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
};

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_dfgemm(const GemmArgs* args, int m, int n, int k, int accumulate) {
  const GemmArgs g = args[blockIdx.z];
  __shared__ dfc sA[16][33];
  __shared__ dfc sB[16][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = blockIdx.x * 32, col0 = blockIdx.y * 32;
  dfc acc[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) acc[i][j] = dfc_zero();
  for (int kk = 0; kk < k; kk += 16) {
    for (int e = threadIdx.x; e < 16 * 32; e += 256) {
      int r = e & 31, q = e >> 5;
      int gr = row0 + r, gk = kk + q;
      cplx v = mk(0.0);
      if (gr < m && gk < k) v = TA ? cconj(g.A[gk + (size_t)g.lda * gr]) : g.A[gr + (size_t)g.lda * gk];
      sA[q][r] = dfc_make(v);
    }
    for (int e = threadIdx.x; e < 16 * 32; e += 256) {
      int q = e & 15, cc = e >> 4;
      int gc = col0 + cc, gk = kk + q;
      cplx v = mk(0.0);
      if (gc < n && gk < k) v = TB ? cconj(g.B[gc + (size_t)g.ldb * gk]) : g.B[gk + (size_t)g.ldb * gc];
      sB[q][cc] = dfc_make(v);
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < 16; ++q) {
      dfc a0 = sA[q][tx], a1 = sA[q][tx + 16];
      dfc b0 = sB[q][ty], b1 = sB[q][ty + 16];
      acc[0][0] = dfc_add(acc[0][0], dfc_mul(a0, b0));
      acc[1][0] = dfc_add(acc[1][0], dfc_mul(a1, b0));
      acc[0][1] = dfc_add(acc[0][1], dfc_mul(a0, b1));
      acc[1][1] = dfc_add(acc[1][1], dfc_mul(a1, b1));
    }
    __syncthreads();
  }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      int r = row0 + tx + 16 * i, c = col0 + ty + 16 * j;
      if (r < m && c < n) {
        cplx* p = g.C + r + (size_t)g.ldc * c;
        if (accumulate) {
          dfc v = dfc_add(acc[i][j], dfc_make(*p));
          *p = dfc_to_d(v);
        } else {
          *p = dfc_to_d(acc[i][j]);
        }
      }
    }
}

int dfgemm_batched(cudaStream_t s, char ta, char tb, int m, int n, int k, const GemmArgs* d_args, int count,
                   int accumulate) {
  dim3 grid((m + 31) / 32, (n + 31) / 32, count);
  bool TA = ta == 'C', TB = tb == 'C';
  if (!TA && !TB) k_dfgemm<false, false><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else if (TA && !TB) k_dfgemm<true, false><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else if (!TA && TB) k_dfgemm<false, true><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
  else k_dfgemm<true, true><<<grid, 256, 0, s>>>(d_args, m, n, k, accumulate);
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
    // trailing update: L(i,k) -= L(i,j) conj(L(k,j)) for j < k <= i
    const int m = n - j - 1;
    const long tri = (long)m * (m + 1) / 2;
    for (long e = threadIdx.x; e < tri; e += blockDim.x) {
      // map e -> (ii, kk) with kk <= ii, both in [0, m)
      int ii = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
      while ((long)(ii + 1) * (ii + 2) / 2 <= e) ++ii;
      while ((long)ii * (ii + 1) / 2 > e) --ii;
      int kk = (int)(e - (long)ii * (ii + 1) / 2);
      int i = j + 1 + ii, k = j + 1 + kk;
      dfc lij = L[i + (size_t)n * j], lkj = L[k + (size_t)n * j];
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
  // R = L^H (upper) to `rinv`; it is inverted in place by k_gj_inverse
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    if (i <= j) {
      dfc v = L[j + (size_t)n * i];
      a.rinv[i + (size_t)n * j] = mk(df_to_d(v.re), -df_to_d(v.im));
    } else {
      a.rinv[i + (size_t)n * j] = mk(0.0);
    }
  }
  if (threadIdx.x == 0 && s_bad) *a.status = 1;
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

__global__ void k_bprop_df(const PropArgs* args, int t_from, int t_to, int forward) {
  const PropArgs a = args[blockIdx.y];
  const DevModel& M = a.M;
  extern __shared__ dfc colv[];
  const int ns = M.ns, pd = M.pdim;
  cplx* x = a.X + (size_t)ns * blockIdx.x;
  for (int r = threadIdx.x; r < ns; r += blockDim.x) colv[r] = dfc_make(x[r]);
  __syncthreads();
  const int nt = forward ? (t_to - t_from + 1) : (t_from - t_to + 1);
  for (int it = 0; it < nt; ++it) {
    const int t = (forward ? t_from + it : t_from - it) - 1;
    for (int f = 0; f < M.n_pf; ++f) {
      const int pf = forward ? f : M.n_pf - 1 - f;
      const int dim = M.pf_dim[pf], npla = M.pf_npla[pf];
      for (int p = threadIdx.x; p < npla; p += blockDim.x) {
        int S[4];
        dfc v[4];
        for (int k = 0; k < dim; ++k) {
          S[k] = M.site[k + pd * (p + M.max_pla * pf)];
          v[k] = colv[S[k]];
        }
        const cplx* E = a.expkv + M.kv_base(p, pf, t);
        for (int r = 0; r < dim; ++r) {
          dfc s = dfc_zero();
          for (int k = 0; k < dim; ++k) {
            cplx e = forward ? E[r + pd * k] : cconj(E[k + pd * r]);
            s = dfc_add(s, dfc_mul(dfc_make(e), v[k]));
          }
          colv[S[r]] = s;
        }
      }
      __syncthreads();
    }
  }
  for (int r = threadIdx.x; r < ns; r += blockDim.x) x[r] = dfc_to_d(colv[r]);
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
};

__global__ void k_bweight(const WeightArgs* args, int ndcount, long ng, int compare) {
  const WeightArgs a = args[blockIdx.x];
  __shared__ double rre[256], rim[256], rmx[256];
  double sr = 0.0, sim = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < ndcount; i += blockDim.x) {
    cplx l = clog_(a.d_block[i]);
    sr += l.x;
    sim += l.y;
  }
  if (compare)
    for (long e = threadIdx.x; e < ng; e += blockDim.x) mx = fmax(mx, cabsd(csub(a.gold[e], a.gnew[e])));
  rre[threadIdx.x] = sr;
  rim[threadIdx.x] = sim;
  rmx[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rre[threadIdx.x] += rre[threadIdx.x + s];
      rim[threadIdx.x] += rim[threadIdx.x + s];
      rmx[threadIdx.x] = fmax(rmx[threadIdx.x], rmx[threadIdx.x + s]);
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
                status};
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
  return PQMC_OK;
}

static inline cplx* qblk(pqmc_chain* c, int b1) { return c->q_string + (size_t)c->ns * c->nelec * (b1 - 1); }
static inline cplx* dblk(pqmc_chain* c, int b1) { return c->d_string + (size_t)c->nelec * (b1 - 1); }

int BatchRecompute::gemm(char ta, char tb, int m, int n, int k, const std::vector<GemmArgs>& a, int slot,
                         int accumulate) {
  PQMC_CUDA(cudaMemcpyAsync(d_gemm + slot * C, a.data(), sizeof(GemmArgs) * C, cudaMemcpyHostToDevice, stream));
  return dfgemm_batched(stream, ta, tb, m, n, k, d_gemm + slot * C, C, accumulate);
}

// CholeskyQR2 of X_c (ns x ne) in place; d_c = |diag R|
int BatchRecompute::cholqr2(const std::vector<cplx*>& X, const std::vector<cplx*>& D) {
  std::vector<GemmArgs> ga(C);
  std::vector<CholArgs> ca(C);
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < C; ++i) ga[i] = GemmArgs{X[i], X[i], gram + (size_t)i * ne * ne, ns, ns, ne};
    PQMC_TRY(gemm('C', 'N', ne, ne, ns, ga, 0, 0));
    for (int i = 0; i < C; ++i)
      ca[i] = CholArgs{gram + (size_t)i * ne * ne, work_df + (size_t)i * ne * ne, rinv + (size_t)i * ne * ne, D[i],
                       status + i};
    PQMC_CUDA(cudaMemcpyAsync(d_chol, ca.data(), sizeof(CholArgs) * C, cudaMemcpyHostToDevice, stream));
    k_chol_inv<<<C, 512, 0, stream>>>(d_chol, ne, pass);
    PQMC_LAUNCHED();
    {
      std::vector<GJArgs> gj(C);
      for (int i = 0; i < C; ++i)
        gj[i] = GJArgs{rinv + (size_t)i * ne * ne, work_df + (size_t)i * ne * ne, logdet + i, piv + (size_t)i * ne,
                       perm + (size_t)i * ne, status + i};
      PQMC_CUDA(cudaMemcpyAsync(d_gj + C, gj.data(), sizeof(GJArgs) * C, cudaMemcpyHostToDevice, stream));
      k_gj_inverse<<<C, 512, 0, stream>>>(d_gj + C, ne);
      PQMC_LAUNCHED();
    }
    for (int i = 0; i < C; ++i) ga[i] = GemmArgs{X[i], rinv + (size_t)i * ne * ne, tmpX + (size_t)i * ns * ne, ns, ne, ns};
    PQMC_TRY(gemm('N', 'N', ns, ne, ne, ga, 1, 0));
    for (int i = 0; i < C; ++i)
      PQMC_CUDA(cudaMemcpyAsync(X[i], tmpX + (size_t)i * ns * ne, sizeof(cplx) * (size_t)ns * ne,
                                cudaMemcpyDeviceToDevice, stream));
  }
  return PQMC_OK;
}

// G = R (L R)^-1 L with L = XL^H; ln_cw; errors (cal_g_and_det_T0)
int BatchRecompute::g_and_det(const std::vector<cplx*>& XL, const std::vector<cplx*>& R,
                              const std::vector<cplx*>& Gcur, const std::vector<cplx*>& Gnew, bool compare, int blk1) {
  std::vector<GemmArgs> ga(C);
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{XL[i], R[i], pbp + (size_t)i * ne * ne, ns, ns, ne};
  PQMC_TRY(gemm('C', 'N', ne, ne, ns, ga, 2, 0));
  std::vector<GJArgs> gj(C);
  for (int i = 0; i < C; ++i)
    gj[i] = GJArgs{pbp + (size_t)i * ne * ne, work_df + (size_t)i * ne * ne, logdet + i, piv + (size_t)i * ne,
                   perm + (size_t)i * ne, status + i};
  PQMC_CUDA(cudaMemcpyAsync(d_gj, gj.data(), sizeof(GJArgs) * C, cudaMemcpyHostToDevice, stream));
  k_gj_inverse<<<C, 512, 0, stream>>>(d_gj, ne);
  PQMC_LAUNCHED();
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{R[i], pbp + (size_t)i * ne * ne, wmat + (size_t)i * ns * ne, ns, ne, ns};
  PQMC_TRY(gemm('N', 'N', ns, ne, ne, ga, 3, 0));
  for (int i = 0; i < C; ++i) ga[i] = GemmArgs{wmat + (size_t)i * ns * ne, XL[i], Gnew[i], ns, ns, ns};
  PQMC_TRY(gemm('N', 'C', ns, ns, ne, ga, 4, 0));
  std::vector<WeightArgs> wa(C);
  for (int i = 0; i < C; ++i)
    wa[i] = WeightArgs{cs[i]->sc, dblk(cs[i], blk1), cs[i]->d_logsum, blk1 - 1, cs[i]->nblock, logdet + i, Gcur[i],
                       Gnew[i], cs[i]->M.tr_weight, cs[i]->M.ncopy};
  PQMC_CUDA(cudaMemcpyAsync(d_weight, wa.data(), sizeof(WeightArgs) * C, cudaMemcpyHostToDevice, stream));
  k_bweight<<<C, 256, 0, stream>>>(d_weight, ne, (long)ns * ns, compare ? 1 : 0);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int BatchRecompute::propagate(const std::vector<cplx*>& X, int t_from, int t_to, bool forward) {
  std::vector<PropArgs> pa(C);
  for (int i = 0; i < C; ++i) pa[i] = PropArgs{cs[i]->M, X[i], cs[i]->expkv};
  PQMC_CUDA(cudaMemcpyAsync(d_prop, pa.data(), sizeof(PropArgs) * C, cudaMemcpyHostToDevice, stream));
  dim3 grid(ne, C);
  k_bprop_df<<<grid, 128, sizeof(dfc) * ns, stream>>>(d_prop, t_from, t_to, forward ? 1 : 0);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// get_g_scratch_T0 for every chain (each chain's current G is in c->g;
// the new G is written to c->g_alt and the pointers are swapped)
int BatchRecompute::scratch(int time, bool forward) {
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
  for (int i = 0; i < C; ++i) {
    Gc[i] = cs[i]->g;
    Gn[i] = cs[i]->g_alt;
  }
  PQMC_TRY(g_and_det(XL, R, Gc, Gn, true, blk));
  for (auto* c : cs) {
    cplx* t = c->g;
    c->g = c->g_alt;
    c->g_alt = t;
  }
  return PQMC_OK;
}

}  // namespace pqmc
