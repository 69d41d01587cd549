// finite_t.cu -- the finite-temperature Green's function path of one chain:
// init_g_FT, cal_g_and_det_FT, get_g_scratch_FT and cal_new_weight_FT
// (src/mod_evolution.f90:409-785), selected per chain by
// pqmc_set_temperature as set_temperature selects the procedure pointers
// (:30-45).  FP64 throughout, on the single-chain kernels of chain.cu and
// linalg.cu.
//
// Strings (1-based blocks, nblock = ntime/ngroup + 2; block b sits at slice
// t_b = ngroup (b - 1)):
//   right string, blocks below the current time: B(t_b, 0) = Q D R;
//   left string, blocks above it: B(beta, t_b) = R_l D Q_l, stored in
//   adjoint form as Q := Q_l^H, R := R_l^H (B(beta, t)^H = Q D R), so that
//   both strings grow by the same step: X = B(slices) Q_old D_old (the
//   left string propagates with B^H), X P = Q' R' with the columns
//   pre-sorted by decreasing norm (pre-pivoting, Bai, Lee, Li and Xu,
//   "Stable solutions of linear systems involving long chain of matrix
//   multiplications", Linear Algebra Appl. 435 (2011)), D' = |diag R'|,
//   R_new = D'^-1 R' P^T R_old.
// The reference decomposes the strings with the singular value
// decomposition (zudv); a graded product keeps its small scales only under
// a column-pivoted (or pre-pivoted) QR, which is what this file uses.
// Three further departures from the reference's unfinished branch, each a
// correction: init_g_FT's last call takes block nblock (B(beta,beta) = 1)
// as the left factor instead of the right string's own adjoint (:485-489);
// the left string's unitary factor goes to Q_l, not to R_l (:711-713); and
// cal_new_weight_FT scales column i by D(i) alone (:763-765).
//
//   g = (1 + B(t,0) B(beta,t))^-1, g_h = 1 - g,
//   1 + Q_r D_r R_r Y^H D_l X^H = Q_r Dr_gt M Dl_gt X^H,
//   M = Dr_gt^-1 Q_r^H X Dl_gt^-1 + Dr_lt R_r Y^H Dl_lt
// (the scale split of :527-570, with X = Q_l^H, Y = R_l^H), M factored by
// LU with partial pivoting (it is well conditioned after the split):
//   g = X Dl_gt^-1 M^-1 Dr_gt^-1 Q_r^H,
//   ln det(1 + B) = ln det Q_r + sum ln Dr_gt + ln det M + sum ln Dl_gt
//                   + conj(ln det X).
#include "chain.cuh"
#include "linalg.cuh"

namespace pqmc {

struct FtState {
  cplx* q = nullptr;     // (Ns, Ns, nblock)
  cplx* r = nullptr;     // (Ns, Ns, nblock)
  cplx* d = nullptr;     // (Ns, nblock)
  cplx* lnq = nullptr;   // (nblock) ln det of each block's Q
  cplx* x = nullptr;     // (Ns, Ns) work
  cplx* y = nullptr;
  cplx* t1 = nullptr;
  cplx* t2 = nullptr;
  cplx* qa = nullptr;    // cal_new_weight's own string
  cplx* ra = nullptr;
  cplx* da = nullptr;
  cplx* tau = nullptr;   // (Ns)
  cplx* dtmp = nullptr;
  cplx* lcol = nullptr;
  cplx* scal = nullptr;  // [0] ln det M, [1] sum ln Dr_gt, [2] sum ln Dl_gt, [3] ln det Q of qa
  int* ipiv = nullptr;
  int* perm = nullptr;
  double* norm = nullptr;
};

// ---------------------------------------------------------------------------
__global__ void k_ft_eye(int n, cplx* A) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x)
    A[e] = mk(e % n == e / n ? 1.0 : 0.0);
}

__global__ void k_ft_fill(int n, cplx* v, cplx val) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = val;
}

// X(:, j) *= d(j), and norm(j) = |X(:, j)| after the scaling, taken as
// max |x| * |x / max| (the entries of a graded string pass 1e154, where
// the plain sum of squares overflows); one CTA of 256 threads per column
__global__ void k_ft_colscale_norm(int n, cplx* X, const cplx* __restrict__ d, double* norm) {
  __shared__ double red[256];
  const int j = blockIdx.x;
  const cplx dj = d[j];
  cplx* x = X + (size_t)n * j;
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cplx v = cmul(x[i], dj);
    x[i] = v;
    mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
  }
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  mx = red[0];
  __syncthreads();
  double s = 0.0;
  if (mx > 0.0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double a = x[i].x / mx, b = x[i].y / mx;
      s += a * a + b * b;
    }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) norm[j] = mx * sqrt(red[0]);
}

// perm(rank) = j with columns ranked by decreasing norm, ties by index; a
// NaN norm ranks below every number, so (norm, index) is a total order and
// the ranks are a permutation of 0..n-1 whatever the norms hold
__global__ void k_ft_rank(int n, const double* __restrict__ norm, int* perm) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double v = isnan(norm[j]) ? -1.0 : norm[j];
  int rank = 0;
  for (int k = 0; k < n; ++k) {
    const double w = isnan(norm[k]) ? -1.0 : norm[k];
    rank += (w > v || (w == v && k < j)) ? 1 : 0;
  }
  perm[rank] = j;
}

// Y(:, i) = X(:, perm(i))
__global__ void k_ft_gather_cols(int n, const cplx* __restrict__ X, const int* __restrict__ perm, cplx* Y) {
  const int i = blockIdx.x;
  const cplx* src = X + (size_t)n * perm[i];
  cplx* dst = Y + (size_t)n * i;
  for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
}

// D(i) = |R(i,i)|
__global__ void k_ft_rdiag(int n, const cplx* __restrict__ R, cplx* D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) D[i] = mk(cabsd(R[i + (size_t)n * i]));
}

// R(i, :) /= D(i) (in place; D from k_ft_rdiag, so no entry of R is read
// after another thread has scaled it)
__global__ void k_ft_rscale(int n, cplx* R, const cplx* __restrict__ D) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    const double di = D[e % n].x;
    if (di > 0.0) R[e] = cscale(R[e], 1.0 / di);
  }
}

// B(i, :) = A(perm(i), :)  (B = P^T A)
__global__ void k_ft_rowperm(int n, const cplx* __restrict__ A, const int* __restrict__ perm, cplx* B) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n);
    const long j = e / n;
    B[e] = A[perm[i] + (size_t)n * j];
  }
}

__device__ __forceinline__ cplx ft_gt(cplx d) { return cabsd(d) > 1.0 ? d : mk(1.0); }
__device__ __forceinline__ cplx ft_lt(cplx d) { return cabsd(d) > 1.0 ? mk(1.0) : d; }

// M = Dr_gt^-1 A1 Dl_gt^-1 + Dr_lt A2 Dl_lt (in place on A1)
__global__ void k_ft_mix(int n, cplx* A1, const cplx* __restrict__ A2, const cplx* __restrict__ dl,
                         const cplx* __restrict__ dr) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    const cplx a = cdiv(cdiv(A1[e], ft_gt(dr[i])), ft_gt(dl[j]));
    A1[e] = cadd(a, cmul(cmul(ft_lt(dr[i]), A2[e]), ft_lt(dl[j])));
  }
}

// Z(i, :) /= gt(d(i))
__global__ void k_ft_rowdiv_gt(int n, cplx* Z, const cplx* __restrict__ d) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x)
    Z[e] = cdiv(Z[e], ft_gt(d[e % n]));
}

// g_h = 1 - g in place
__global__ void k_ft_one_minus(int n, cplx* G) {
  const long nn = (long)n * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    const cplx v = cneg(G[e]);
    G[e] = (e % n == e / n) ? cadd(v, mk(1.0)) : v;
  }
}

// out[0] = sum ln Dr_gt, out[1] = sum ln Dl_gt (one CTA)
__global__ void k_ft_sumlog_gt(int n, const cplx* __restrict__ dr, const cplx* __restrict__ dl, cplx* out) {
  __shared__ double a[256], b[256], c[256], e[256];
  double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cplx lr = clog_(ft_gt(dr[i])), ll = clog_(ft_gt(dl[i]));
    ar += lr.x; ai += lr.y; br += ll.x; bi += ll.y;
  }
  a[threadIdx.x] = ar; b[threadIdx.x] = ai; c[threadIdx.x] = br; e[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      a[threadIdx.x] += a[threadIdx.x + o];
      b[threadIdx.x] += b[threadIdx.x + o];
      c[threadIdx.x] += c[threadIdx.x + o];
      e[threadIdx.x] += e[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = mk(a[0], b[0]);
    out[1] = mk(c[0], e[0]);
  }
}

// logdet = ln det M + ln det Q_r + conj(ln det X), sumlogd = the Dgt sums
__global__ void k_ft_lnparts(DevScalars* sc, const cplx* __restrict__ scal, const cplx* __restrict__ lnq_r,
                             const cplx* __restrict__ lnq_l) {
  sc->logdet = cadd(cadd(scal[0], lnq_r[0]), cconj(lnq_l[0]));
  sc->sumlogd = cadd(scal[1], scal[2]);
}

// ---------------------------------------------------------------------------
static inline cplx* fq(pqmc_chain* c, int b) { return c->ft->q + (size_t)c->ns * c->ns * (b - 1); }
static inline cplx* fr(pqmc_chain* c, int b) { return c->ft->r + (size_t)c->ns * c->ns * (b - 1); }
static inline cplx* fd(pqmc_chain* c, int b) { return c->ft->d + (size_t)c->ns * (b - 1); }
static inline cplx* flq(pqmc_chain* c, int b) { return c->ft->lnq + (b - 1); }

static int ew_grid(long n) {
  long b = (n + 255) / 256;
  return (int)(b < 1024 ? b : 1024);
}

// One string step: X = B(slices) Qin Din (forward: slices t_from..t_to
// ascending; backward: B^H, slices t_from..t_to descending), pre-pivoted
// QR, Qout = Q, Dout = |diag R|, Rout = D^-1 R P^T Rin.  Qout/Dout/Rout may
// alias Qin/Din/Rin.
static int ft_step(pqmc_chain* c, const cplx* qin, const cplx* din, const cplx* rin, bool forward, int t_from,
                   int t_to, cplx* qout, cplx* dout, cplx* rout, cplx* lnq_out) {
  FtState& f = *c->ft;
  const int n = c->ns;
  cudaStream_t s = c->stream;
  const size_t mb = sizeof(cplx) * (size_t)n * n;
  PQMC_CUDA(cudaMemcpyAsync(f.x, qin, mb, cudaMemcpyDeviceToDevice, s));
  PQMC_TRY(launch_propagate(c, f.x, n, t_from, t_to, forward));
  k_ft_colscale_norm<<<n, 256, 0, s>>>(n, f.x, din, f.norm);
  PQMC_LAUNCHED();
  k_ft_rank<<<(n + 127) / 128, 128, 0, s>>>(n, f.norm, f.perm);
  PQMC_LAUNCHED();
  k_ft_gather_cols<<<n, 128, 0, s>>>(n, f.x, f.perm, f.y);
  PQMC_LAUNCHED();
  PQMC_TRY(house_qr_r(s, n, n, f.y, f.tau, f.dtmp, f.t1, lnq_out));
  k_ft_rdiag<<<(n + 127) / 128, 128, 0, s>>>(n, f.t1, dout);
  PQMC_LAUNCHED();
  k_ft_rscale<<<ew_grid((long)n * n), 256, 0, s>>>(n, f.t1, dout);
  PQMC_LAUNCHED();
  k_ft_rowperm<<<ew_grid((long)n * n), 256, 0, s>>>(n, rin, f.perm, f.t2);
  PQMC_LAUNCHED();
  PQMC_TRY(zgemm(s, 'N', 'N', n, n, n, mk(1.0), f.t1, n, f.t2, n, mk(0.0), rout, n));
  PQMC_CUDA(cudaMemcpyAsync(qout, f.y, mb, cudaMemcpyDeviceToDevice, s));
  return PQMC_OK;
}

// cal_g_and_det_FT with the left factors in adjoint form (X = Q_l^H,
// Y = R_l^H); G into g_alt (then swapped in) when cal_g, compared with the
// fast-updated G and ln_cw when compare.
static int ft_cal_g_and_det(pqmc_chain* c, const cplx* x, const cplx* dl, const cplx* y, const cplx* lnq_l,
                            const cplx* qr, const cplx* dr, const cplx* rr, const cplx* lnq_r, bool cal_g,
                            bool compare) {
  FtState& f = *c->ft;
  const int n = c->ns;
  cudaStream_t s = c->stream;
  const long nn = (long)n * n;
  PQMC_TRY(zgemm(s, 'C', 'N', n, n, n, mk(1.0), qr, n, x, n, mk(0.0), f.t1, n));   // Q_r^H X
  PQMC_TRY(zgemm(s, 'N', 'C', n, n, n, mk(1.0), rr, n, y, n, mk(0.0), f.t2, n));   // R_r Y^H
  k_ft_mix<<<ew_grid(nn), 256, 0, s>>>(n, f.t1, f.t2, dl, dr);
  PQMC_LAUNCHED();
  PQMC_TRY(lu_factor(s, n, f.t1, f.ipiv, &c->sc->lu_info, f.lcol));
  PQMC_TRY(lu_logdet(s, n, f.t1, f.ipiv, f.scal));
  k_ft_sumlog_gt<<<1, 256, 0, s>>>(n, dr, dl, f.scal + 1);
  PQMC_LAUNCHED();
  k_ft_lnparts<<<1, 1, 0, s>>>(c->sc, f.scal, lnq_r, lnq_l);
  PQMC_LAUNCHED();
  if (cal_g) {
    PQMC_TRY(herm_t(s, n, n, qr, f.t2));                                        // Q_r^H
    k_ft_rowdiv_gt<<<ew_grid(nn), 256, 0, s>>>(n, f.t2, dr);
    PQMC_LAUNCHED();
    PQMC_TRY(lu_solve(s, n, n, f.t1, f.ipiv, f.t2, n));                         // M^-1 Dr_gt^-1 Q_r^H
    k_ft_rowdiv_gt<<<ew_grid(nn), 256, 0, s>>>(n, f.t2, dl);
    PQMC_LAUNCHED();
    PQMC_TRY(zgemm(s, 'N', 'N', n, n, n, mk(1.0), x, n, f.t2, n, mk(0.0), c->g_alt, n));
    k_ft_one_minus<<<ew_grid(nn), 256, 0, s>>>(n, c->g_alt);
    PQMC_LAUNCHED();
    if (compare) {
      double* e = reinterpret_cast<double*>(f.lcol);
      PQMC_CUDA(cudaMemsetAsync(e, 0, 3 * sizeof(double), s));
      k_maxdiff<<<152, 256, 0, s>>>(nn, c->g, c->g_alt, e);
      PQMC_LAUNCHED();
      k_set_errg<<<1, 1, 0, s>>>(c->sc, e);
      PQMC_LAUNCHED();
    }
  }
  k_finish_weight<<<1, 1, 0, s>>>(c->sc, c->M.tr_weight, c->M.ncopy, compare ? 1 : 0);
  PQMC_LAUNCHED();
  if (cal_g) {
    cplx* t = c->g;
    c->g = c->g_alt;
    c->g_alt = t;
  }
  int info = 0;
  PQMC_CUDA(cudaMemcpyAsync(&info, &c->sc->lu_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  PQMC_CUDA(cudaStreamSynchronize(s));
  if (info != 0) {
    set_error("cal_g_and_det_FT: zero pivot %d in the scale-separated middle matrix", info);
    return PQMC_ERR_SINGULAR;
  }
  return PQMC_OK;
}

static int ft_identity_block(pqmc_chain* c, int b) {
  const int n = c->ns;
  cudaStream_t s = c->stream;
  k_ft_eye<<<ew_grid((long)n * n), 256, 0, s>>>(n, fq(c, b));
  PQMC_LAUNCHED();
  k_ft_eye<<<ew_grid((long)n * n), 256, 0, s>>>(n, fr(c, b));
  PQMC_LAUNCHED();
  k_ft_fill<<<(n + 255) / 256, 256, 0, s>>>(n, fd(c, b), mk(1.0));
  PQMC_LAUNCHED();
  k_ft_fill<<<1, 32, 0, s>>>(1, flq(c, b), mk(0.0));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// init_g_FT(start_time), src/mod_evolution.f90:411-489
int do_init_g_ft(pqmc_chain* c, int start_time) {
  const int nb = c->nblock, ng = c->ngroup;
  k_scalars_zero<<<1, 1, 0, c->stream>>>(c->sc);
  PQMC_LAUNCHED();
  PQMC_TRY(ft_identity_block(c, 1));
  PQMC_TRY(ft_identity_block(c, nb));
  const int start_block = start_time / ng + 1;
  const int start_by_block = (start_block - 1) * ng + 1;
  if (start_time < 1 || start_time > c->ntime || start_by_block > start_time) {
    set_error("init_g_FT: start_time %d outside 1..%d", start_time, c->ntime);
    return PQMC_ERR_ARG;
  }
  for (int p0 = start_by_block; p0 <= c->ntime; p0 += ng) {
    const int blk = (p0 + ng - 2) / ng + 2;
    PQMC_TRY(ft_step(c, fq(c, blk - 1), fd(c, blk - 1), fr(c, blk - 1), true, p0, p0 + ng - 1, fq(c, blk),
                     fd(c, blk), fr(c, blk), flq(c, blk)));
  }
  PQMC_TRY(ft_cal_g_and_det(c, fq(c, nb), fd(c, nb), fr(c, nb), flq(c, nb), fq(c, nb - 1), fd(c, nb - 1),
                            fr(c, nb - 1), flq(c, nb - 1), true, false));
  c->have_g = true;
  return PQMC_OK;
}

// get_g_scratch_FT(time, forward, loop), src/mod_evolution.f90:631-745
int do_g_scratch_ft(pqmc_chain* c, int time, bool forward) {
  const int ng = c->ngroup;
  if (forward ? (time - ng < 1 || time - 1 > c->ntime) : (time < 1 || time + ng - 1 > c->ntime)) {
    set_error("g_scratch_FT: slices of time %d outside 1..%d", time, c->ntime);
    return PQMC_ERR_ARG;
  }
  if (forward) {
    const int blk = time / ng + 1;
    if (blk < 2 || blk + 1 > c->nblock) { set_error("g_scratch_FT: block %d out of range", blk); return PQMC_ERR_ARG; }
    PQMC_TRY(ft_step(c, fq(c, blk - 1), fd(c, blk - 1), fr(c, blk - 1), true, time - ng, time - 1, fq(c, blk),
                     fd(c, blk), fr(c, blk), flq(c, blk)));
    return ft_cal_g_and_det(c, fq(c, blk + 1), fd(c, blk + 1), fr(c, blk + 1), flq(c, blk + 1), fq(c, blk),
                            fd(c, blk), fr(c, blk), flq(c, blk), true, true);
  }
  int blk = time / ng + 2;
  if (ng == 1) blk -= 1;
  if (blk < 2 || blk + 1 > c->nblock) { set_error("g_scratch_FT: block %d out of range", blk); return PQMC_ERR_ARG; }
  PQMC_TRY(ft_step(c, fq(c, blk + 1), fd(c, blk + 1), fr(c, blk + 1), false, time + ng - 1, time, fq(c, blk),
                   fd(c, blk), fr(c, blk), flq(c, blk)));
  return ft_cal_g_and_det(c, fq(c, blk), fd(c, blk), fr(c, blk), flq(c, blk), fq(c, blk - 1), fd(c, blk - 1),
                          fr(c, blk - 1), flq(c, blk - 1), true, true);
}

// cal_new_weight_FT, src/mod_evolution.f90:748-785: the right string of the
// whole interval from block 1, in the chain's own work buffers (the strings
// and G are left intact); ln_cw is set.
int do_new_weight_ft(pqmc_chain* c) {
  FtState& f = *c->ft;
  const int n = c->ns, ng = c->ngroup, nb = c->nblock;
  cudaStream_t s = c->stream;
  const size_t mb = sizeof(cplx) * (size_t)n * n;
  PQMC_CUDA(cudaMemcpyAsync(f.qa, fq(c, 1), mb, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemcpyAsync(f.ra, fr(c, 1), mb, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemcpyAsync(f.da, fd(c, 1), sizeof(cplx) * n, cudaMemcpyDeviceToDevice, s));
  for (int p0 = 1; p0 <= c->ntime; p0 += ng)
    PQMC_TRY(ft_step(c, f.qa, f.da, f.ra, true, p0, p0 + ng - 1, f.qa, f.da, f.ra, f.scal + 3));
  return ft_cal_g_and_det(c, fq(c, nb), fd(c, nb), fr(c, nb), flq(c, nb), f.qa, f.da, f.ra, f.scal + 3, false,
                          false);
}

template <typename T>
static int ft_alloc(T** p, size_t n) {
  if (cudaMalloc((void**)p, sizeof(T) * n) != cudaSuccess) {
    set_error("finite-T buffers: cudaMalloc of %zu bytes failed", sizeof(T) * n);
    return PQMC_ERR_NOMEM;
  }
  return PQMC_OK;
}

int ft_free(pqmc_chain* c) {
  if (!c->ft) return PQMC_OK;
  FtState& f = *c->ft;
  void* ptrs[] = {f.q, f.r, f.d, f.lnq, f.x, f.y, f.t1, f.t2, f.qa, f.ra, f.da, f.tau, f.dtmp, f.lcol, f.scal,
                  f.ipiv, f.perm, f.norm};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete c->ft;
  c->ft = nullptr;
  return PQMC_OK;
}

static int ft_setup(pqmc_chain* c) {
  if (c->ft) return PQMC_OK;
  if (c->ntime % c->ngroup != 0) {
    set_error("set_temperature: the finite-temperature strings need ntime (%d) to be a multiple of ngroup (%d)",
              c->ntime, c->ngroup);
    return PQMC_ERR_ARG;
  }
  c->ft = new FtState();
  FtState& f = *c->ft;
  const size_t n = c->ns, nn = n * n, nb = c->nblock;
  int st = PQMC_OK;
  if (st == PQMC_OK) st = ft_alloc(&f.q, nn * nb);
  if (st == PQMC_OK) st = ft_alloc(&f.r, nn * nb);
  if (st == PQMC_OK) st = ft_alloc(&f.d, n * nb);
  if (st == PQMC_OK) st = ft_alloc(&f.lnq, nb);
  cplx** work[] = {&f.x, &f.y, &f.t1, &f.t2, &f.qa, &f.ra};
  for (cplx** w : work)
    if (st == PQMC_OK) st = ft_alloc(w, nn);
  if (st == PQMC_OK) st = ft_alloc(&f.da, n);
  if (st == PQMC_OK) st = ft_alloc(&f.tau, n);
  if (st == PQMC_OK) st = ft_alloc(&f.dtmp, n);
  if (st == PQMC_OK) st = ft_alloc(&f.lcol, n + 2);
  if (st == PQMC_OK) st = ft_alloc(&f.scal, 4);
  if (st == PQMC_OK) st = ft_alloc(&f.ipiv, n);
  if (st == PQMC_OK) st = ft_alloc(&f.perm, n);
  if (st == PQMC_OK) st = ft_alloc(&f.norm, n);
  if (st != PQMC_OK) {
    ft_free(c);
    return st;
  }
  // every block starts as the identity string (init_g_FT :427-434)
  for (int b = 1; b <= c->nblock; ++b) PQMC_TRY(ft_identity_block(c, b));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

}  // namespace pqmc

using namespace pqmc;

extern "C" {

int pqmc_set_temperature(pqmc_chain* c, int proj) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (c->in_batch) {
    set_error("set_temperature: chains of a batch run the projector path only");
    return PQMC_ERR_STATE;
  }
  if (proj) {
    c->finite_t = false;
    c->have_g = false;
    return ft_free(c);
  }
  PQMC_TRY(ft_setup(c));
  c->finite_t = true;
  c->have_g = false;
  return PQMC_OK;
}

int pqmc_get_temperature(pqmc_chain* c, int* proj) {
  if (!c || !proj) { set_error("null argument"); return PQMC_ERR_ARG; }
  *proj = c->finite_t ? 0 : 1;
  return PQMC_OK;
}

int pqmc_init_g_ft(pqmc_chain* c, int start_time) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->finite_t) { set_error("init_g_FT: the chain is on the projector path (pqmc_set_temperature(c, 0) first)"); return PQMC_ERR_STATE; }
  return do_init_g_ft(c, start_time);
}

int pqmc_get_g_scratch_ft(pqmc_chain* c, int time, int forward, int loop, double* err_out) {
  (void)loop;
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->finite_t) { set_error("get_g_scratch_FT: the chain is on the projector path"); return PQMC_ERR_STATE; }
  if (!c->have_g) { set_error("get_g_scratch_FT before init_g_FT"); return PQMC_ERR_STATE; }
  PQMC_TRY(do_g_scratch_ft(c, time, forward != 0));
  if (err_out) {
    DevScalars h;
    PQMC_CUDA(cudaMemcpy(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost));
    err_out[0] = h.err_g;
    err_out[1] = h.err_w;
  }
  return PQMC_OK;
}

int pqmc_cal_new_weight_ft(pqmc_chain* c, double* ln_cw_out) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->finite_t) { set_error("cal_new_weight_FT: the chain is on the projector path"); return PQMC_ERR_STATE; }
  if (!c->have_g) { set_error("cal_new_weight_FT before init_g_FT"); return PQMC_ERR_STATE; }
  PQMC_TRY(do_new_weight_ft(c));
  if (ln_cw_out) {
    DevScalars h;
    PQMC_CUDA(cudaMemcpy(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost));
    ln_cw_out[0] = h.ln_cw.x;
    ln_cw_out[1] = h.ln_cw.y;
  }
  return PQMC_OK;
}

int pqmc_get_qdr_ft(pqmc_chain* c, int block, double* q, double* d, double* r) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->ft) { set_error("get_qdr_FT: no finite-temperature strings"); return PQMC_ERR_STATE; }
  if (block < 1 || block > c->nblock) { set_error("get_qdr_FT: block %d outside 1..%d", block, c->nblock); return PQMC_ERR_ARG; }
  const size_t n = c->ns;
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  if (q) PQMC_CUDA(cudaMemcpy(q, fq(c, block), sizeof(cplx) * n * n, cudaMemcpyDeviceToHost));
  if (d) PQMC_CUDA(cudaMemcpy(d, fd(c, block), sizeof(cplx) * n, cudaMemcpyDeviceToHost));
  if (r) PQMC_CUDA(cudaMemcpy(r, fr(c, block), sizeof(cplx) * n * n, cudaMemcpyDeviceToHost));
  return PQMC_OK;
}

}  // extern "C"
