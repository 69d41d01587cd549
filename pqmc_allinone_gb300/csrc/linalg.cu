// linalg.cu -- FP64 complex dense kernels for the stabilisation path:
// GEMM, Householder QR with Q formation (zgeqrf/zungqr conventions), LU with
// partial pivoting (zgetf2 conventions), multi-RHS LU solve and log-det.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so every routine
// spreads its work over all SMs: the factorisations are cooperative kernels
// (one grid barrier per elimination stage), the products are tiled GEMMs.
#include <cooperative_groups.h>
#include "linalg.cuh"

namespace cg = cooperative_groups;

namespace pqmc {

// ---------------------------------------------------------------------------
// C = alpha * op(A) * op(B) + beta * C, op in {N, C (conjugate transpose)}.
// 32x32 output tile per CTA, 256 threads, 2x2 outputs per thread, k-tiles of
// 16 staged in shared memory.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_zgemm(int m, int n, int k, cplx alpha, const cplx* __restrict__ A,
                                                int lda, const cplx* __restrict__ B, int ldb, cplx beta,
                                                cplx* __restrict__ C, int ldc) {
  __shared__ cplx sA[16][33];
  __shared__ cplx sB[16][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = blockIdx.x * 32, col0 = blockIdx.y * 32;
  cplx acc[2][2] = {{mk(0), mk(0)}, {mk(0), mk(0)}};
  for (int kk = 0; kk < k; kk += 16) {
    // A tile: rows row0..row0+31, k kk..kk+15 -> sA[k][row]
    for (int e = threadIdx.x; e < 16 * 32; e += 256) {
      int r = e & 31, q = e >> 5;
      int gr = row0 + r, gk = kk + q;
      cplx v = mk(0);
      if (gr < m && gk < k) v = TA ? cconj(A[gk + (size_t)lda * gr]) : A[gr + (size_t)lda * gk];
      sA[q][r] = v;
    }
    for (int e = threadIdx.x; e < 16 * 32; e += 256) {
      int q = e & 15, c = e >> 4;
      int gc = col0 + c, gk = kk + q;
      cplx v = mk(0);
      if (gc < n && gk < k) v = TB ? cconj(B[gc + (size_t)ldb * gk]) : B[gk + (size_t)ldb * gc];
      sB[q][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      cplx a0 = sA[q][tx], a1 = sA[q][tx + 16];
      cplx b0 = sB[q][ty], b1 = sB[q][ty + 16];
      acc[0][0] = cfma(a0, b0, acc[0][0]);
      acc[1][0] = cfma(a1, b0, acc[1][0]);
      acc[0][1] = cfma(a0, b1, acc[0][1]);
      acc[1][1] = cfma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      int r = row0 + tx + 16 * i, c = col0 + ty + 16 * j;
      if (r < m && c < n) {
        cplx* p = C + r + (size_t)ldc * c;
        cplx v = cmul(alpha, acc[i][j]);
        if (beta.x != 0.0 || beta.y != 0.0) v = cfma(beta, *p, v);
        *p = v;
      }
    }
}

int zgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, cplx alpha, const cplx* A, int lda,
          const cplx* B, int ldb, cplx beta, cplx* C, int ldc) {
  dim3 grid((m + 31) / 32, (n + 31) / 32);
  bool TA = (ta == 'C'), TB = (tb == 'C');
  if (!TA && !TB) k_zgemm<false, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (TA && !TB) k_zgemm<true, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (!TA && TB) k_zgemm<false, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else k_zgemm<true, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// block-wide sum of a double (all threads get the result)
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) red[32] = t;
  __syncthreads();
  double r = red[32];
  __syncthreads();
  return r;
}

// block-wide max of a double (all threads get the result)
__device__ __forceinline__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
  if (threadIdx.x == 0) red[32] = t;
  __syncthreads();
  double r = red[32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ cplx block_csum(cplx v, double* red) {
  double re = block_sum(v.x, red);
  double im = block_sum(v.y, red);
  return mk(re, im);
}

// ---------------------------------------------------------------------------
// Householder QR in place (zgeqr2): column i reflector by block 0, then every
// block applies H_i^H to its share of the trailing columns.  Then Q formation
// (zung2r).  A is m x n (lda = m), m >= n.  d receives diag(R) (real in the
// LAPACK convention).  Matches zqdr (src/mod_matrixlib.f90:323-334) with the
// unit-diagonal R discarded as the reference does for the hot path.  With
// Rout the upper triangle of R (n x n, diagonal = d) is copied out before Q
// is formed, and with lndet ln det Q = sum over the reflectors of
// ln det(I - tau v v^H) = ln(-tau / conj(tau)) (a phase; 0 for tau = 0).
// scaled: the reflector norms are taken as max |x| * |x / max|, as LAPACK's
// dznrm2 avoids overflow, for columns whose entries pass 1e154 (the graded
// finite-temperature strings); the projector path keeps the plain sum.
__global__ void __launch_bounds__(256) k_house_qr(int m, int n, cplx* A, cplx* tau, cplx* d, cplx* Rout,
                                                  cplx* lndet, int scaled) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double red[33];
  for (int i = 0; i < n; ++i) {
    cplx* col = A + (size_t)m * i;
    if (blockIdx.x == 0) {
      // zlarfg on col[i..m-1]
      double xnorm;
      if (scaled) {
        double mx = 0.0;
        for (int k = i + 1 + threadIdx.x; k < m; k += blockDim.x) mx = fmax(mx, fmax(fabs(col[k].x), fabs(col[k].y)));
        mx = block_max(mx, red);
        double ss = 0.0;
        if (mx > 0.0)
          for (int k = i + 1 + threadIdx.x; k < m; k += blockDim.x) {
            const double a = col[k].x / mx, b = col[k].y / mx;
            ss += a * a + b * b;
          }
        xnorm = mx * sqrt(block_sum(ss, red));
      } else {
        double ss = 0.0;
        for (int k = i + 1 + threadIdx.x; k < m; k += blockDim.x) ss += cabs2(col[k]);
        xnorm = sqrt(block_sum(ss, red));
      }
      cplx alpha = col[i];
      __shared__ cplx s_scale;
      __shared__ double s_beta;
      __shared__ int s_zero;
      if (threadIdx.x == 0) {
        if (xnorm == 0.0 && alpha.y == 0.0) {
          tau[i] = mk(0.0);
          s_zero = 1;
          s_beta = alpha.x;
        } else {
          double w = fmax(fabs(alpha.x), fmax(fabs(alpha.y), xnorm));
          double a1 = alpha.x / w, a2 = alpha.y / w, a3 = xnorm / w;
          double nrm = w * sqrt(a1 * a1 + a2 * a2 + a3 * a3);
          double beta = alpha.x >= 0.0 ? -nrm : nrm;
          tau[i] = mk((beta - alpha.x) / beta, -alpha.y / beta);
          s_scale = cdiv(mk(1.0), csub(alpha, mk(beta)));
          s_beta = beta;
          s_zero = 0;
        }
        d[i] = mk(s_beta);
      }
      __syncthreads();
      if (!s_zero)
        for (int k = i + 1 + threadIdx.x; k < m; k += blockDim.x) col[k] = cmul(s_scale, col[k]);
      __syncthreads();
      if (threadIdx.x == 0) col[i] = mk(s_beta);
    }
    grid.sync();
    // apply H_i^H = I - conj(tau) v v^H to columns j > i; v = [1; col[i+1..]]
    const cplx ct = cconj(tau[i]);
    for (int j = i + 1 + blockIdx.x; j < n; j += gridDim.x) {
      cplx* cj = A + (size_t)m * j;
      cplx w = mk(0.0);
      for (int k = i + threadIdx.x; k < m; k += blockDim.x) {
        cplx v = (k == i) ? mk(1.0) : col[k];
        w = cadd(w, cmulc(v, cj[k]));
      }
      w = block_csum(w, red);
      cplx f = cmul(ct, w);
      for (int k = i + threadIdx.x; k < m; k += blockDim.x) {
        cplx v = (k == i) ? mk(1.0) : col[k];
        cj[k] = csub(cj[k], cmul(v, f));
      }
    }
    grid.sync();
  }
  if (Rout) {
    for (int j = blockIdx.x; j < n; j += gridDim.x)
      for (int k = threadIdx.x; k < n; k += blockDim.x) Rout[k + (size_t)n * j] = k <= j ? A[k + (size_t)m * j] : mk(0.0);
    grid.sync();
  }
  if (lndet && blockIdx.x == 0 && threadIdx.x == 0) {
    double ph = 0.0;
    for (int i = 0; i < n; ++i) {
      const cplx t = tau[i];
      if (t.x != 0.0 || t.y != 0.0) {
        const cplx z = cdiv(cneg(t), cconj(t));
        ph += atan2(z.y, z.x);
      }
    }
    lndet[0] = mk(0.0, ph);
  }
  // zung2r: Q = H_1 ... H_n applied to the first n unit columns
  for (int i = n - 1; i >= 0; --i) {
    cplx* col = A + (size_t)m * i;
    const cplx t = tau[i];
    for (int j = i + 1 + blockIdx.x; j < n; j += gridDim.x) {
      cplx* cj = A + (size_t)m * j;
      cplx w = mk(0.0);
      for (int k = i + threadIdx.x; k < m; k += blockDim.x) {
        cplx v = (k == i) ? mk(1.0) : col[k];
        w = cadd(w, cmulc(v, cj[k]));
      }
      w = block_csum(w, red);
      cplx f = cmul(t, w);
      for (int k = i + threadIdx.x; k < m; k += blockDim.x) {
        cplx v = (k == i) ? mk(1.0) : col[k];
        cj[k] = csub(cj[k], cmul(v, f));
      }
    }
    grid.sync();
    if (blockIdx.x == (i % gridDim.x)) {
      for (int k = threadIdx.x; k < m; k += blockDim.x) {
        if (k > i) col[k] = cmul(cneg(t), col[k]);
        else if (k == i) col[k] = csub(mk(1.0), t);
        else col[k] = mk(0.0);
      }
    }
    grid.sync();
  }
}

// ---------------------------------------------------------------------------
// LU with partial pivoting in place (zgetf2), n x n, lda = n.  ipiv 0-based.
// info[0] = first zero pivot (1-based) or 0.  lcol is an n-vector of scratch.
__global__ void __launch_bounds__(256) k_lu(int n, cplx* A, int* ipiv, int* info, cplx* lcol) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double sv[256];
  __shared__ int si[256];
  if (blockIdx.x == 0 && threadIdx.x == 0) info[0] = 0;
  for (int j = 0; j < n; ++j) {
    cplx* cj = A + (size_t)n * j;
    if (blockIdx.x == 0) {
      double best = -1.0;
      int bi = j;
      for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
        double v = fabs(cj[i].x) + fabs(cj[i].y);
        if (v > best) { best = v; bi = i; }
      }
      sv[threadIdx.x] = best;
      si[threadIdx.x] = bi;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
          double ov = sv[threadIdx.x + s];
          int oi = si[threadIdx.x + s];
          if (ov > sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x])) {
            sv[threadIdx.x] = ov;
            si[threadIdx.x] = oi;
          }
        }
        __syncthreads();
      }
      const int jp = si[0];
      const cplx piv = cj[jp];
      const bool zero = (piv.x == 0.0 && piv.y == 0.0);
      if (threadIdx.x == 0) {
        ipiv[j] = jp;
        if (zero && info[0] == 0) info[0] = j + 1;
      }
      // swapped + scaled column j, published in lcol (rows > j)
      cplx rec = zero ? mk(0.0) : cdiv(mk(1.0), piv);
      for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
        cplx v = (i == jp) ? cj[j] : cj[i];
        lcol[i] = zero ? v : cmul(v, rec);
      }
      __syncthreads();
      for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) cj[i] = lcol[i];
      if (threadIdx.x == 0) cj[j] = piv;
    }
    grid.sync();
    const int jp = ipiv[j];
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
      if (k == j) continue;
      cplx* ck = A + (size_t)n * k;
      if (jp != j && threadIdx.x == 0) {
        cplx t = ck[j];
        ck[j] = ck[jp];
        ck[jp] = t;
      }
      __syncthreads();
      if (k > j) {
        const cplx u = ck[j];
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) ck[i] = csub(ck[i], cmul(lcol[i], u));
      }
      __syncthreads();
    }
    grid.sync();
  }
}

// Solve A X = B in place on B (n x nrhs, ldb = n) from the LU factors.
// One warp per right-hand side.
__global__ void k_lu_solve(int n, int nrhs, const cplx* __restrict__ LU, const int* __restrict__ ipiv,
                           cplx* B, int ldb) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= nrhs) return;
  cplx* b = B + (size_t)ldb * c;
  if (lane == 0)
    for (int j = 0; j < n; ++j) {
      int p = ipiv[j];
      if (p != j) { cplx t = b[j]; b[j] = b[p]; b[p] = t; }
    }
  __syncwarp();
  // forward: unit lower
  for (int i = 1; i < n; ++i) {
    cplx s = mk(0.0);
    for (int j = lane; j < i; j += 32) s = cfma(LU[i + (size_t)n * j], b[j], s);
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) b[i] = csub(b[i], s);
    __syncwarp();
  }
  for (int i = n - 1; i >= 0; --i) {
    cplx s = mk(0.0);
    for (int j = i + 1 + lane; j < n; j += 32) s = cfma(LU[i + (size_t)n * j], b[j], s);
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) b[i] = cdiv(csub(b[i], s), LU[i + (size_t)n * i]);
    __syncwarp();
  }
}

// log det from the LU factors: the reference forms the product of the
// diagonal (zdet_lapack, src/mod_matrixlib.f90:624-653) and takes its log;
// when the product leaves the double range the sum of logs is used.
__global__ void k_lu_logdet(int n, const cplx* LU, const int* ipiv, cplx* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int s = 1;
  cplx d = mk(1.0), ls = mk(0.0);
  for (int i = 0; i < n; ++i) {
    if (ipiv[i] != i) s = -s;
    cplx u = LU[i + (size_t)n * i];
    d = cmul(d, u);
    ls = cadd(ls, clog_(u));
  }
  if (s < 0) {
    d = cneg(d);
    ls = cadd(ls, mk(0.0, 3.14159265358979323846));
  }
  double ad = cabsd(d);
  out[0] = (ad > 1e-290 && ad < 1e290) ? clog_(d) : ls;
}

int coop_grid(const void* fn, int threads, int want) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
  int cap = nsm * (per > 0 ? per : 1);
  if (want > cap) want = cap;
  if (want > nsm) want = nsm;
  return want < 1 ? 1 : want;
}

int house_qr(cudaStream_t s, int m, int n, cplx* A, cplx* tau, cplx* d) {
  return house_qr_r(s, m, n, A, tau, d, nullptr, nullptr);
}

int house_qr_r(cudaStream_t s, int m, int n, cplx* A, cplx* tau, cplx* d, cplx* R, cplx* lndet) {
  int nb = coop_grid((const void*)k_house_qr, 256, n);
  int scaled = (R != nullptr || lndet != nullptr) ? 1 : 0;
  void* args[] = {&m, &n, &A, &tau, &d, &R, &lndet, &scaled};
  PQMC_CUDA(cudaLaunchCooperativeKernel((const void*)k_house_qr, nb, 256, args, 0, s));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int lu_factor(cudaStream_t s, int n, cplx* A, int* ipiv, int* info, cplx* lcol) {
  int nb = coop_grid((const void*)k_lu, 256, n);
  void* args[] = {&n, &A, &ipiv, &info, &lcol};
  PQMC_CUDA(cudaLaunchCooperativeKernel((const void*)k_lu, nb, 256, args, 0, s));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int lu_solve(cudaStream_t s, int n, int nrhs, const cplx* LU, const int* ipiv, cplx* B, int ldb) {
  int wpb = 4;
  k_lu_solve<<<(nrhs + wpb - 1) / wpb, 32 * wpb, 0, s>>>(n, nrhs, LU, ipiv, B, ldb);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int lu_logdet(cudaStream_t s, int n, const cplx* LU, const int* ipiv, cplx* out) {
  k_lu_logdet<<<1, 32, 0, s>>>(n, LU, ipiv, out);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// conjugate transpose copy: out(n,m) = a(m,n)^H
__global__ void k_herm_t(int m, int n, const cplx* __restrict__ a, cplx* __restrict__ out) {
  __shared__ cplx t[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = bx + threadIdx.x, c = by + k;
    if (r < m && c < n) t[k][threadIdx.x] = a[r + (size_t)m * c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = by + threadIdx.x, c = bx + k;   // out row r (< n), col c (< m)
    if (r < n && c < m) out[r + (size_t)n * c] = cconj(t[threadIdx.x][k]);
  }
}

int herm_t(cudaStream_t s, int m, int n, const cplx* a, cplx* out) {
  dim3 g((m + 31) / 32, (n + 31) / 32), b(32, 8);
  k_herm_t<<<g, b, 0, s>>>(m, n, a, out);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

}  // namespace pqmc
