// chain.cu -- one Markov chain of the projector-DQMC hot path on the GPU:
// local updates (src/mod_update.f90:13-245,475-500), B-string wraps and
// propagation (src/mod_evolution.f90:236-328), stabilised recompute
// (:46-195, :330-408) and the C-ABI that replaces those subroutines.
#include <cooperative_groups.h>
#include <stdarg.h>
#include <string.h>
#include <mutex>
#include <string>
#include "chain.cuh"
#include "linalg.cuh"
#include "rng.cuh"

namespace cg = cooperative_groups;

namespace pqmc {

std::atomic<int64_t> g_launches{0};
static thread_local std::string t_err;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_err = buf;
}

static __device__ __forceinline__ cplx ldg_c(const cplx* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// init_expKV for every (family, plaquette, slice) (mod_phonon_field.f90:423-450)
// expKV / expKV_inv of slices t0 .. t0+nt-1 (0-based) from the field
__global__ void k_init_expkv(DevModel M, const double* __restrict__ field, cplx* expkv, cplx* expkv_inv, int t0,
                             int nt) {
  const long total = (long)M.n_pf * M.max_pla * nt;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    int p = (int)(e % M.max_pla);
    int pf = (int)((e / M.max_pla) % M.n_pf);
    int t = t0 + (int)(e / ((long)M.max_pla * M.n_pf));
    if (p >= M.pf_npla[pf]) continue;
    double bf = M.pf_v_exist[pf] ? field[M.bf[p + M.max_pla * pf] + (size_t)M.n_bf * t] : 0.0;
    const int dim = M.pf_dim[pf];
    cplx m[16];
    size_t base = M.kv_base(p, pf, t);
    dev_get_expkv(M, pf, p, bf, false, m);
    for (int j = 0; j < M.pdim; ++j)
      for (int i = 0; i < M.pdim; ++i)
        expkv[base + i + M.pdim * j] = (i < dim && j < dim) ? m[i + dim * j] : mk(0.0);
    dev_get_expkv(M, pf, p, bf, true, m);
    for (int j = 0; j < M.pdim; ++j)
      for (int i = 0; i < M.pdim; ++i)
        expkv_inv[base + i + M.pdim * j] = (i < dim && j < dim) ? m[i + dim * j] : mk(0.0);
  }
}

int launch_init_expkv(pqmc_chain* c, int t0, int nt) {
  if (nt <= 0) nt = c->ntime - t0;
  long total = (long)c->n_pf * c->max_pla * nt;
  int blocks = (int)((total + 127) / 128);
  if (blocks > 4096) blocks = 4096;
  k_init_expkv<<<blocks, 128, 0, c->stream>>>(c->M, c->field, c->expkv, c->expkv_inv, t0, nt);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// Two-way wrap of G by one family (left_evolve/right_evolve with two_way,
// src/mod_evolution.f90:236-328): out(Sr,Sc) = A_r G(Sr,Sc) B_c over all
// pairs of cover items; left: A = expKV, B = expKV_inv; right: swapped.
__global__ void k_wrap(DevModel M, int pf, int t, int left, int n_items, const int* __restrict__ ipla,
                       const int* __restrict__ isites, const int* __restrict__ idim,
                       const cplx* __restrict__ expkv, const cplx* __restrict__ expkv_inv,
                       const cplx* __restrict__ gin, cplx* __restrict__ gout) {
  const long pair = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (pair >= (long)n_items * n_items) return;
  const int ir = (int)(pair % n_items), ic = (int)(pair / n_items);
  const int ns = M.ns, pd = M.pdim;
  const int dr = idim[ir], dc = idim[ic];
  int Sr[4], Sc[4];
  for (int k = 0; k < dr; ++k) Sr[k] = isites[4 * ir + k];
  for (int k = 0; k < dc; ++k) Sc[k] = isites[4 * ic + k];
  cplx g[16], h[16];
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) g[a + 4 * b] = gin[Sr[a] + (size_t)ns * Sc[b]];
  const int pr = ipla[ir], pc = ipla[ic];
  const cplx* A = (pr >= 0) ? (left ? expkv : expkv_inv) + M.kv_base(pr, pf, t) : nullptr;
  const cplx* B = (pc >= 0) ? (left ? expkv_inv : expkv) + M.kv_base(pc, pf, t) : nullptr;
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) {
      cplx s;
      if (A) {
        s = mk(0.0);
        for (int k = 0; k < dr; ++k) s = cfma(A[a + pd * k], g[k + 4 * b], s);
      } else {
        s = g[a + 4 * b];
      }
      h[a + 4 * b] = s;
    }
  for (int b = 0; b < dc; ++b)
    for (int a = 0; a < dr; ++a) {
      cplx s;
      if (B) {
        s = mk(0.0);
        for (int k = 0; k < dc; ++k) s = cfma(h[a + 4 * k], B[k + pd * b], s);
      } else {
        s = h[a + 4 * b];
      }
      gout[Sr[a] + (size_t)ns * Sc[b]] = s;
    }
}

int launch_wrap(pqmc_chain* c, int pf, int time, bool left) {
  const WrapItems& w = c->wrap[pf];
  long pairs = (long)w.n_items * w.n_items;
  int threads = 64;
  int blocks = (int)((pairs + threads - 1) / threads);
  k_wrap<<<blocks, threads, 0, c->stream>>>(c->M, pf, time - 1, left ? 1 : 0, w.n_items, w.d_pla, w.d_sites,
                                            w.d_dim, c->expkv, c->expkv_inv, c->g, c->g_alt);
  PQMC_LAUNCHED();
  cplx* t = c->g;
  c->g = c->g_alt;
  c->g_alt = t;
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// One-way propagation of an Ns x n matrix X through slices [t_from..t_to]
// (1-based, inclusive).  forward: left_evolve(.false.) on rmat, slices
// ascending, families 1..n_pf, X(S,:) <- E X(S,:).  backward: right_evolve
// (.false.) on lmat = X^H, slices descending, families n_pf..1,
// X(S,:) <- E^H X(S,:).  One CTA per column; the column lives in shared memory.
__global__ void k_propagate(DevModel M, cplx* X, int ldx, int t_from, int t_to, int forward,
                            const cplx* __restrict__ expkv) {
  extern __shared__ cplx col[];
  const int ns = M.ns, pd = M.pdim;
  cplx* x = X + (size_t)ldx * blockIdx.x;
  for (int r = threadIdx.x; r < ns; r += blockDim.x) col[r] = x[r];
  __syncthreads();
  const int nt = forward ? (t_to - t_from + 1) : (t_from - t_to + 1);
  for (int it = 0; it < nt; ++it) {
    const int t = (forward ? t_from + it : t_from - it) - 1;
    for (int f = 0; f < M.n_pf; ++f) {
      const int pf = forward ? f : M.n_pf - 1 - f;
      const int dim = M.pf_dim[pf], npla = M.pf_npla[pf];
      for (int p = threadIdx.x; p < npla; p += blockDim.x) {
        int S[4];
        cplx v[4];
        for (int k = 0; k < dim; ++k) {
          S[k] = M.site[k + pd * (p + M.max_pla * pf)];
          v[k] = col[S[k]];
        }
        const cplx* E = expkv + M.kv_base(p, pf, t);
        for (int a = 0; a < dim; ++a) {
          cplx s = mk(0.0);
          for (int k = 0; k < dim; ++k) {
            cplx e = forward ? E[a + pd * k] : cconj(E[k + pd * a]);
            s = cfma(e, v[k], s);
          }
          col[S[a]] = s;
        }
      }
      __syncthreads();
    }
  }
  for (int r = threadIdx.x; r < ns; r += blockDim.x) x[r] = col[r];
}

int launch_propagate(pqmc_chain* c, cplx* X, int n, int t_from, int t_to, bool forward) {
  int threads = 128;
  size_t smem = sizeof(cplx) * (size_t)c->ns;
  k_propagate<<<n, threads, smem, c->stream>>>(c->M, X, c->ns, t_from, t_to, forward ? 1 : 0, c->expkv);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// small reductions for the weight bookkeeping
__global__ void k_sumlog(int n, const cplx* __restrict__ d, cplx* out, int accumulate) {
  __shared__ double rr[256], ri[256];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    cplx l = clog_(d[i]);
    a += l.x;
    b += l.y;
  }
  rr[threadIdx.x] = a;
  ri[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rr[threadIdx.x] += rr[threadIdx.x + s];
      ri[threadIdx.x] += ri[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = accumulate ? cadd(out[0], mk(rr[0], ri[0])) : mk(rr[0], ri[0]);
}

// sum of log D over one block of the D string, written to out[0]
__global__ void k_blocklog(int n, const cplx* __restrict__ d, cplx* out) {
  __shared__ double rr[256], ri[256];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    cplx l = clog_(d[i]);
    a += l.x;
    b += l.y;
  }
  rr[threadIdx.x] = a;
  ri[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rr[threadIdx.x] += rr[threadIdx.x + s];
      ri[threadIdx.x] += ri[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = mk(rr[0], ri[0]);
}

// sumlogd = sum over blocks of the per-block sums (sum(log(D_string)), :346)
__global__ void k_sumvec(int n, const cplx* __restrict__ v, cplx* out) {
  if (threadIdx.x != 0) return;
  cplx s = mk(0.0);
  for (int i = 0; i < n; ++i) s = cadd(s, v[i]);
  out[0] = s;
}

int block_log(pqmc_chain* c, int blk1) {
  k_blocklog<<<1, 256, 0, c->stream>>>(c->nelec, c->d_string + (size_t)c->nelec * (blk1 - 1),
                                        c->d_logsum + (blk1 - 1));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

__device__ __forceinline__ cplx branch_reduce(cplx z) {
  // cmplx(real(z), mod(aimag(z), 2*pi)) with PI of nrtype in REAL(SP)
  const double two_pi_sp = (double)(2.0f * 3.14159265358979323846f);
  return mk(z.x, fmod(z.y, two_pi_sp));
}

// ln_cw = (log det PBP + sum log D) (TR, ncopy), then branch reduction;
// errors against the fast-update values (mod_evolution.f90:345-356,179-193)
__global__ void k_finish_weight(DevScalars* sc, int tr_weight, int ncopy, int compare) {
  cplx l = cadd(sc->logdet, sc->sumlogd);
  if (tr_weight) l = cadd(l, cconj(l));
  l = cscale(l, (double)ncopy);
  cplx nw = branch_reduce(l);
  if (compare) {
    double e = fabs(nw.x - sc->ln_cw.x);
    sc->err_w = e;
    sc->err_fast = e;
    if (e > sc->err_fast_max) sc->err_fast_max = e;
  }
  sc->ln_cw = nw;
}

// out[0] = max |a - b| (atomicMax on the bit pattern of a non-negative
// double), out[1] += sum |a - b|^2, out[2] += sum |b|^2
__global__ void k_maxdiff(long n, const cplx* __restrict__ a, const cplx* __restrict__ b, double* out) {
  __shared__ double red[256], rd[256], rb[256];
  double m = 0.0, sd = 0.0, sb = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const cplx bi = b[i], di = csub(a[i], bi);
    m = fmax(m, cabsd(di));
    sd += cabs2(di);
    sb += cabs2(bi);
  }
  red[threadIdx.x] = m;
  rd[threadIdx.x] = sd;
  rb[threadIdx.x] = sb;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
      rd[threadIdx.x] += rd[threadIdx.x + s];
      rb[threadIdx.x] += rb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicMax((unsigned long long*)out, __double_as_longlong(red[0]));
    atomicAdd(out + 1, rd[0]);
    atomicAdd(out + 2, rb[0]);
  }
}

__global__ void k_set_errg(DevScalars* sc, const double* e) {
  double v = e[0];
  sc->err_g = v;
  sc->err_fast = v;
  if (v > sc->err_fast_max) sc->err_fast_max = v;
  const double rel = e[2] > 0.0 ? sqrt(e[1] / e[2]) : 0.0;
  sc->err_g_rel = rel;
  if (rel > sc->err_g_rel_max) sc->err_g_rel_max = rel;
}

__global__ void k_scalars_zero(DevScalars* sc) {
  sc->ln_cw = mk(0.0);
  sc->logdet = mk(0.0);
  sc->sumlogd = mk(0.0);
}

// cal_g_and_det_T0 with the left factor held as X = lmat^H (Ns x nelec)
static int cal_g_and_det(pqmc_chain* c, const cplx* X, const cplx* R, bool compare) {
  const int ns = c->ns, ne = c->nelec;
  cudaStream_t s = c->stream;
  PQMC_TRY(zgemm(s, 'C', 'N', ne, ne, ns, mk(1.0), X, ns, R, ns, mk(0.0), c->pbp, ne));
  PQMC_TRY(lu_factor(s, ne, c->pbp, c->ipiv, &c->sc->lu_info, c->lcol));
  PQMC_TRY(lu_logdet(s, ne, c->pbp, c->ipiv, &c->sc->logdet));
  k_sumvec<<<1, 32, 0, s>>>(c->nblock, c->d_logsum, &c->sc->sumlogd);
  PQMC_LAUNCHED();
  PQMC_TRY(herm_t(s, ns, ne, X, c->lmat));
  PQMC_TRY(lu_solve(s, ne, ns, c->pbp, c->ipiv, c->lmat, ne));
  PQMC_TRY(zgemm(s, 'N', 'N', ns, ns, ne, mk(1.0), R, ns, c->lmat, ne, mk(0.0), c->g_alt, ns));
  if (compare) {
    double* e = reinterpret_cast<double*>(c->lcol);   // scratch scalar
    PQMC_CUDA(cudaMemsetAsync(e, 0, 3 * sizeof(double), s));
    k_maxdiff<<<152, 256, 0, s>>>((long)ns * ns, c->g, c->g_alt, e);
    PQMC_LAUNCHED();
    k_set_errg<<<1, 1, 0, s>>>(c->sc, e);
    PQMC_LAUNCHED();
  }
  k_finish_weight<<<1, 1, 0, s>>>(c->sc, c->M.tr_weight, c->M.ncopy, compare ? 1 : 0);
  PQMC_LAUNCHED();
  cplx* t = c->g;
  c->g = c->g_alt;
  c->g_alt = t;
  int info = 0;
  PQMC_CUDA(cudaMemcpyAsync(&info, &c->sc->lu_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  PQMC_CUDA(cudaStreamSynchronize(s));
  if (info != 0) {
    set_error("cal_g_and_det: zero pivot %d in P^H B P", info);
    return PQMC_ERR_SINGULAR;
  }
  return PQMC_OK;
}

static inline cplx* Qblk(pqmc_chain* c, int blk1) {  // 1-based block
  return c->q_string + (size_t)c->ns * c->nelec * (blk1 - 1);
}
static inline cplx* Dblk(pqmc_chain* c, int blk1) { return c->d_string + (size_t)c->nelec * (blk1 - 1); }

// init_g_T0(start_time), src/mod_evolution.f90:46-111; a chain set to
// finite temperature takes init_g_FT instead (the procedure pointer of
// set_temperature, :30-45)
int do_init_g(pqmc_chain* c, int start_time) {
  if (c->finite_t) return do_init_g_ft(c, start_time);
  const int ns = c->ns, ne = c->nelec, nb = c->nblock;
  cudaStream_t s = c->stream;
  size_t qb = sizeof(cplx) * (size_t)ns * ne;
  k_scalars_zero<<<1, 1, 0, s>>>(c->sc);
  PQMC_LAUNCHED();
  PQMC_CUDA(cudaMemcpyAsync(Qblk(c, 1), c->slater_q, qb, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemcpyAsync(Qblk(c, nb), c->slater_q, qb, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemcpyAsync(Dblk(c, 1), c->slater_d, sizeof(cplx) * ne, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemcpyAsync(Dblk(c, nb), c->slater_d, sizeof(cplx) * ne, cudaMemcpyDeviceToDevice, s));
  for (int b = 1; b <= nb; ++b) PQMC_TRY(block_log(c, b));
  int start_block = start_time / c->ngroup + 1;
  int start_by_block = (start_block - 1) * c->ngroup + 1;
  if (start_by_block > start_time) {
    set_error("init_g: start_time_by_block > start_time");
    return PQMC_ERR_ARG;
  }
  PQMC_CUDA(cudaMemcpyAsync(c->rmat, Qblk(c, start_block), qb, cudaMemcpyDeviceToDevice, s));
  int p = start_by_block;
  while (p <= c->ntime) {
    int next_mult = ((p + c->ngroup - 1) / c->ngroup) * c->ngroup;
    int end = next_mult <= c->ntime ? next_mult : c->ntime;
    PQMC_TRY(launch_propagate(c, c->rmat, ne, p, end, true));
    if (end % c->ngroup == 0) {
      int blk = (end - 1) / c->ngroup + 2;
      PQMC_TRY(house_qr(s, ns, ne, c->rmat, c->tau, Dblk(c, blk)));
      PQMC_TRY(block_log(c, blk));
      PQMC_CUDA(cudaMemcpyAsync(Qblk(c, blk), c->rmat, qb, cudaMemcpyDeviceToDevice, s));
    }
    p = end + 1;
  }
  PQMC_TRY(cal_g_and_det(c, Qblk(c, nb), c->rmat, false));
  c->have_g = true;
  return PQMC_OK;
}

// get_g_scratch_T0(time, forward, loop), src/mod_evolution.f90:113-195
int do_g_scratch(pqmc_chain* c, int time, bool forward, int loop) {
  (void)loop;
  if (c->finite_t) return do_g_scratch_ft(c, time, forward);
  const int ns = c->ns, ne = c->nelec;
  if (forward ? (time - c->ngroup < 1 || time - 1 > c->ntime) : (time < 1 || time + c->ngroup - 1 > c->ntime)) {
    set_error("g_scratch: slices of time %d outside 1..%d", time, c->ntime);
    return PQMC_ERR_ARG;
  }
  cudaStream_t s = c->stream;
  size_t qb = sizeof(cplx) * (size_t)ns * ne;
  if (forward) {
    int blk = time / c->ngroup + 1;
    if (blk < 2 || blk + 1 > c->nblock) { set_error("g_scratch: block %d out of range", blk); return PQMC_ERR_ARG; }
    PQMC_CUDA(cudaMemcpyAsync(c->rmat, Qblk(c, blk - 1), qb, cudaMemcpyDeviceToDevice, s));
    PQMC_TRY(launch_propagate(c, c->rmat, ne, time - c->ngroup, time - 1, true));
    PQMC_TRY(house_qr(s, ns, ne, c->rmat, c->tau, Dblk(c, blk)));
    PQMC_TRY(block_log(c, blk));
    PQMC_CUDA(cudaMemcpyAsync(Qblk(c, blk), c->rmat, qb, cudaMemcpyDeviceToDevice, s));
    return cal_g_and_det(c, Qblk(c, blk + 1), c->rmat, true);
  }
  int blk = time / c->ngroup + 2;
  if (c->ngroup == 1) blk -= 1;
  if (blk < 2 || blk + 1 > c->nblock) { set_error("g_scratch: block %d out of range", blk); return PQMC_ERR_ARG; }
  PQMC_CUDA(cudaMemcpyAsync(c->xmat, Qblk(c, blk + 1), qb, cudaMemcpyDeviceToDevice, s));
  PQMC_TRY(launch_propagate(c, c->xmat, ne, time + c->ngroup - 1, time, false));
  PQMC_TRY(house_qr(s, ns, ne, c->xmat, c->tau, Dblk(c, blk)));
  PQMC_TRY(block_log(c, blk));
  PQMC_CUDA(cudaMemcpyAsync(Qblk(c, blk), c->xmat, qb, cudaMemcpyDeviceToDevice, s));
  return cal_g_and_det(c, c->xmat, Qblk(c, blk - 1), true);
}

// cal_new_weight_T0, src/mod_evolution.f90:359-408
int do_new_weight(pqmc_chain* c) {
  if (c->finite_t) return do_new_weight_ft(c);
  const int ns = c->ns, ne = c->nelec, nb = c->nblock;
  cudaStream_t s = c->stream;
  size_t qb = sizeof(cplx) * (size_t)ns * ne;
  PQMC_CUDA(cudaMemcpyAsync(c->xmat, Qblk(c, nb), qb, cudaMemcpyDeviceToDevice, s));
  k_sumlog<<<1, 256, 0, s>>>(ne, Dblk(c, nb), &c->sc->sumlogd, 0);
  PQMC_LAUNCHED();
  int p = c->ntime;
  while (p >= 1) {
    int lo = p - c->ngroup + 1;
    if (lo >= 1) {
      PQMC_TRY(launch_propagate(c, c->xmat, ne, p, lo, false));
      PQMC_TRY(house_qr(s, ns, ne, c->xmat, c->tau, c->dtmp));
      k_sumlog<<<1, 256, 0, s>>>(ne, c->dtmp, &c->sc->sumlogd, 1);
      PQMC_LAUNCHED();
      p = lo - 1;
    } else {
      PQMC_TRY(launch_propagate(c, c->xmat, ne, p, 1, false));
      p = 0;
    }
  }
  k_sumlog<<<1, 256, 0, s>>>(ne, Dblk(c, 1), &c->sc->sumlogd, 1);
  PQMC_LAUNCHED();
  PQMC_TRY(zgemm(s, 'C', 'N', ne, ne, ns, mk(1.0), c->xmat, ns, Qblk(c, 1), ns, mk(0.0), c->pbp, ne));
  PQMC_TRY(lu_factor(s, ne, c->pbp, c->ipiv, &c->sc->lu_info, c->lcol));
  PQMC_TRY(lu_logdet(s, ne, c->pbp, c->ipiv, &c->sc->logdet));
  k_finish_weight<<<1, 1, 0, s>>>(c->sc, c->M.tr_weight, c->M.ncopy, 0);
  PQMC_LAUNCHED();
  int info = 0;
  PQMC_CUDA(cudaMemcpyAsync(&info, &c->sc->lu_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  PQMC_CUDA(cudaStreamSynchronize(s));
  if (info != 0) { set_error("cal_new_weight: zero pivot %d", info); return PQMC_ERR_SINGULAR; }
  return PQMC_OK;
}

// cal_new_weight_T0 of the current field from the trial state alone (no
// init_g_T0 needed), with the orthonormal left factor kept every ngroup
// slices: ck[k] (Ns x nelec) is the factor at slice boundary k*ngroup, for
// k = 0 .. ntime/ngroup (the adjoint's checkpoints).  Blocks are aligned to
// multiples of ngroup from the bottom; the weight equals do_new_weight's up
// to rounding.  Leaves G and the Q/D strings alone; ln_cw is set.
int do_new_weight_ck(pqmc_chain* c, cplx* ck) {
  const int ns = c->ns, ne = c->nelec, nt = c->ntime, ng = c->ngroup;
  cudaStream_t s = c->stream;
  const size_t qb = sizeof(cplx) * (size_t)ns * ne;
  PQMC_CUDA(cudaMemcpyAsync(c->xmat, c->slater_q, qb, cudaMemcpyDeviceToDevice, s));
  k_sumlog<<<1, 256, 0, s>>>(ne, c->slater_d, &c->sc->sumlogd, 0);
  PQMC_LAUNCHED();
  if (nt % ng == 0) PQMC_CUDA(cudaMemcpyAsync(ck + (size_t)ns * ne * (nt / ng), c->xmat, qb, cudaMemcpyDeviceToDevice, s));
  for (int p = nt; p >= 1;) {
    const int lo = ((p - 1) / ng) * ng + 1;   // slices [lo, p]
    PQMC_TRY(launch_propagate(c, c->xmat, ne, p, lo, false));
    PQMC_TRY(house_qr(s, ns, ne, c->xmat, c->tau, c->dtmp));
    k_sumlog<<<1, 256, 0, s>>>(ne, c->dtmp, &c->sc->sumlogd, 1);
    PQMC_LAUNCHED();
    PQMC_CUDA(cudaMemcpyAsync(ck + (size_t)ns * ne * ((lo - 1) / ng), c->xmat, qb, cudaMemcpyDeviceToDevice, s));
    p = lo - 1;
  }
  k_sumlog<<<1, 256, 0, s>>>(ne, c->slater_d, &c->sc->sumlogd, 1);
  PQMC_LAUNCHED();
  PQMC_TRY(zgemm(s, 'C', 'N', ne, ne, ns, mk(1.0), c->xmat, ns, c->slater_q, ns, mk(0.0), c->pbp, ne));
  PQMC_TRY(lu_factor(s, ne, c->pbp, c->ipiv, &c->sc->lu_info, c->lcol));
  PQMC_TRY(lu_logdet(s, ne, c->pbp, c->ipiv, &c->sc->logdet));
  k_finish_weight<<<1, 1, 0, s>>>(c->sc, c->M.tr_weight, c->M.ncopy, 0);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
template <typename T>
static int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
  if (e != cudaSuccess) {
    set_error("cudaMalloc(%zu) -> %s", sizeof(T) * n, cudaGetErrorString(e));
    return PQMC_ERR_NOMEM;
  }
  return PQMC_OK;
}

int chain_alloc(pqmc_chain* c, const pqmc_model* m, cudaStream_t s) {
  if (!m || m->max_dim < 1 || m->max_dim > PQMC_MAX_DIM || m->ns <= 0 || m->nelec <= 0 || m->nelec > m->ns ||
      m->ngroup <= 0 || m->ntime <= 0 || m->n_pf <= 0 || m->max_pla <= 0 || m->n_bf <= 0 || m->ncopy < 1) {
    set_error("pqmc_create: invalid model sizes");
    return PQMC_ERR_ARG;
  }
  c->stream = s;
  c->ns = m->ns; c->nelec = m->nelec; c->ntime = m->ntime; c->ngroup = m->ngroup;
  c->nblock = m->ntime / m->ngroup + 2;
  c->n_pf = m->n_pf; c->pdim = m->max_dim; c->max_pla = m->max_pla; c->n_bf = m->n_bf;
  const int npf = m->n_pf, pd = m->max_dim, mp = m->max_pla;
  c->h_pf_dim.assign(m->pf_dim, m->pf_dim + npf);
  c->h_pf_npla.assign(m->pf_npla, m->pf_npla + npf);
  c->h_pf_v_exist.assign(m->pf_v_exist, m->pf_v_exist + npf);
  for (int f = 0; f < npf; ++f)
    if (m->pf_dim[f] < 1 || m->pf_dim[f] > pd || m->pf_npla[f] < 0 || m->pf_npla[f] > mp) {
      set_error("pqmc_create: family %d has dim %d / n_plaquette %d out of range", f + 1, m->pf_dim[f], m->pf_npla[f]);
      return PQMC_ERR_ARG;
    }
  for (int f = 0; f < npf; ++f)
    for (int p = 0; p < m->pf_npla[f]; ++p) {
      for (int k = 0; k < m->pf_dim[f]; ++k) {
        int st = m->pla_site_list[k + pd * (p + mp * f)];
        if (st < 0 || st >= m->ns) { set_error("pqmc_create: site index %d out of range", st); return PQMC_ERR_ARG; }
      }
      int b = m->bf_list[p + mp * f];
      if (m->pf_v_exist[f] && (b < 0 || b >= m->n_bf)) { set_error("pqmc_create: boson index %d out of range", b); return PQMC_ERR_ARG; }
    }
  // model tables in one blob
  size_t n_int = (size_t)4 * npf + (size_t)pd * mp * npf + 2 * (size_t)mp * npf;
  size_t n_cx = 2 * (size_t)npf + 2 * (size_t)pd * pd * npf + (size_t)pd * pd * mp * npf;
  size_t bytes = n_cx * sizeof(cplx) + n_int * sizeof(int);
  PQMC_CUDA(cudaMalloc(&c->d_model_blob, bytes));
  std::vector<char> h(bytes);
  cplx* hc = reinterpret_cast<cplx*>(h.data());
  size_t off = 0;
  auto putc = [&](const double* src, size_t n) {
    size_t at = off;
    memcpy(hc + off, src, sizeof(cplx) * n);
    off += n;
    return at;
  };
  size_t o_kc = putc(m->pf_k_coe, npf), o_vc = putc(m->pf_v_coe, npf);
  size_t o_km = putc(m->pf_kmat, (size_t)pd * pd * npf), o_vm = putc(m->pf_vmat, (size_t)pd * pd * npf);
  size_t o_bc = putc(m->bc_phases, (size_t)pd * pd * mp * npf);
  int* hi = reinterpret_cast<int*>(hc + off);
  size_t ioff = 0;
  auto puti = [&](const int32_t* src, size_t n) {
    size_t at = ioff;
    memcpy(hi + ioff, src, sizeof(int) * n);
    ioff += n;
    return at;
  };
  size_t o_dim = puti(m->pf_dim, npf), o_npla = puti(m->pf_npla, npf);
  size_t o_ke = puti(m->pf_k_exist, npf), o_ve = puti(m->pf_v_exist, npf);
  size_t o_site = puti(m->pla_site_list, (size_t)pd * mp * npf);
  size_t o_bf = puti(m->bf_list, (size_t)mp * npf);
  size_t o_cr = puti(m->boundary_crossing, (size_t)mp * npf);
  PQMC_CUDA(cudaMemcpy(c->d_model_blob, h.data(), bytes, cudaMemcpyHostToDevice));
  cplx* dc = reinterpret_cast<cplx*>(c->d_model_blob);
  int* di = reinterpret_cast<int*>(dc + off);
  DevModel& M = c->M;
  M.ns = c->ns; M.nelec = c->nelec; M.ntime = c->ntime; M.ngroup = c->ngroup; M.nblock = c->nblock;
  M.n_pf = npf; M.pdim = pd; M.max_pla = mp; M.n_bf = m->n_bf;
  M.expkv_kind = m->expkv_kind; M.ncopy = m->ncopy; M.tr_weight = m->tr_weight; M.metropolis = m->metropolis;
  M.greatest_decent = m->greatest_decent; M.local_update = m->local_update; M.proposal_kind = m->proposal_kind;
  M.delt = m->delt; M.mass = m->mass; M.stiff = m->stiff; M.biased = m->biased_phonon; M.jump = m->jump_distance;
  M.k_coe = dc + o_kc; M.v_coe = dc + o_vc; M.kmat = dc + o_km; M.vmat = dc + o_vm; M.bcp = dc + o_bc;
  M.pf_dim = di + o_dim; M.pf_npla = di + o_npla; M.pf_k_exist = di + o_ke; M.pf_v_exist = di + o_ve;
  M.site = di + o_site; M.bf = di + o_bf; M.cross = di + o_cr;
  // state
  const size_t nkv = (size_t)pd * pd * mp * npf * c->ntime;
  PQMC_TRY(dalloc(&c->field, (size_t)c->n_bf * c->ntime));
  PQMC_TRY(dalloc(&c->expkv, nkv));
  PQMC_TRY(dalloc(&c->expkv_inv, nkv));
  PQMC_TRY(dalloc(&c->g, (size_t)c->ns * c->ns));
  PQMC_TRY(dalloc(&c->g_alt, (size_t)c->ns * c->ns));
  PQMC_TRY(dalloc(&c->q_string, (size_t)c->ns * c->nelec * c->nblock));
  PQMC_TRY(dalloc(&c->d_string, (size_t)c->nelec * c->nblock));
  PQMC_TRY(dalloc(&c->d_logsum, (size_t)c->nblock));
  PQMC_CUDA(cudaMemset(c->d_logsum, 0, sizeof(cplx) * (size_t)c->nblock));
  PQMC_TRY(dalloc(&c->slater_q, (size_t)c->ns * c->nelec));
  PQMC_TRY(dalloc(&c->slater_d, (size_t)c->nelec));
  PQMC_TRY(dalloc(&c->rmat, (size_t)c->ns * c->nelec));
  PQMC_TRY(dalloc(&c->xmat, (size_t)c->ns * c->nelec));
  PQMC_TRY(dalloc(&c->lmat, (size_t)c->ns * c->nelec));
  PQMC_TRY(dalloc(&c->pbp, (size_t)c->nelec * c->nelec));
  PQMC_TRY(dalloc(&c->tau, (size_t)c->nelec));
  PQMC_TRY(dalloc(&c->dtmp, (size_t)c->nelec));
  PQMC_TRY(dalloc(&c->lcol, (size_t)c->nelec + 2));
  PQMC_TRY(dalloc(&c->ipiv, (size_t)c->nelec));
  PQMC_TRY(dalloc(&c->ctl, 2));
  PQMC_TRY(dalloc(&c->sc, 1));
  PQMC_CUDA(cudaMemset(c->g, 0, sizeof(cplx) * (size_t)c->ns * c->ns));
  PQMC_CUDA(cudaMemset(c->field, 0, sizeof(double) * (size_t)c->n_bf * c->ntime));
  {
    std::vector<cplx> ones((size_t)c->nelec * c->nblock, mk(1.0));
    PQMC_CUDA(cudaMemcpy(c->d_string, ones.data(), sizeof(cplx) * ones.size(), cudaMemcpyHostToDevice));
  }
  DevScalars hs;
  memset(&hs, 0, sizeof(hs));
  hs.err_fast_max = 1e-6;   // err_fast_max initial value (src/input.f90:53)
  hs.rng[0] = hs.rng[1] = hs.rng[2] = hs.rng[3] = hs.rng[4] = 1;
  PQMC_CUDA(cudaMemcpy(c->sc, &hs, sizeof(hs), cudaMemcpyHostToDevice));
  // wrap cover items: every site of the lattice belongs to one item per family
  c->wrap.resize(npf);
  for (int f = 0; f < npf; ++f) {
    std::vector<int> owner(c->ns, -1);
    std::vector<int> ipla, isites, idim;
    for (int p = 0; p < m->pf_npla[f]; ++p) {
      ipla.push_back(p);
      idim.push_back(m->pf_dim[f]);
      for (int k = 0; k < 4; ++k) {
        int st = k < m->pf_dim[f] ? m->pla_site_list[k + pd * (p + mp * f)] : 0;
        isites.push_back(st);
        if (k < m->pf_dim[f]) {
          if (owner[st] >= 0) { set_error("pqmc_create: family %d covers site %d twice", f + 1, st); return PQMC_ERR_ARG; }
          owner[st] = p;
        }
      }
    }
    for (int st = 0; st < c->ns; ++st)
      if (owner[st] < 0) {
        ipla.push_back(-1);
        idim.push_back(1);
        isites.push_back(st);
        isites.push_back(0); isites.push_back(0); isites.push_back(0);
      }
    WrapItems& w = c->wrap[f];
    w.n_items = (int)ipla.size();
    PQMC_TRY(dalloc(&w.d_pla, ipla.size()));
    PQMC_TRY(dalloc(&w.d_sites, isites.size()));
    PQMC_TRY(dalloc(&w.d_dim, idim.size()));
    PQMC_CUDA(cudaMemcpy(w.d_pla, ipla.data(), sizeof(int) * ipla.size(), cudaMemcpyHostToDevice));
    PQMC_CUDA(cudaMemcpy(w.d_sites, isites.data(), sizeof(int) * isites.size(), cudaMemcpyHostToDevice));
    PQMC_CUDA(cudaMemcpy(w.d_dim, idim.data(), sizeof(int) * idim.size(), cudaMemcpyHostToDevice));
  }
  // one boson per plaquette within a family: the proposals of a family are
  // then independent of each other until the determinant ratio
  for (int f = 0; f < npf; ++f) {
    if (!m->pf_v_exist[f]) continue;
    std::vector<int> seen(c->n_bf, 0);
    for (int p = 0; p < m->pf_npla[f]; ++p)
      if (seen[m->bf_list[p + mp * f]]++) {
        set_error("pqmc_create: family %d couples boson %d to two plaquettes", f + 1, m->bf_list[p + mp * f]);
        return PQMC_ERR_ARG;
      }
  }
  PQMC_TRY(dalloc(&c->pre, (size_t)mp));
  return update_setup(c);
}

int chain_free(pqmc_chain* c) {
  ft_free(c);
  void* ptrs[] = {c->d_logsum, c->pre, c->d_model_blob, c->field, c->expkv, c->expkv_inv, c->g, c->g_alt, c->q_string, c->d_string,
                  c->slater_q, c->slater_d, c->rmat, c->xmat, c->lmat, c->pbp, c->tau, c->dtmp, c->lcol,
                  c->ipiv, c->ctl, c->sc, c->m_cell_sites, c->m_cell_bf, c->m_cell_xnb, c->m_cell_ynb,
                  c->m_cell_cross, c->m_c2_of, c->m_kphase, c->m_acc, c->m_gtmp};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& w : c->wrap) {
    cudaFree(w.d_pla);
    cudaFree(w.d_sites);
    cudaFree(w.d_dim);
  }
  return PQMC_OK;
}

}  // namespace pqmc

namespace pqmc {
__global__ void k_propagate_one(DevModel M, cplx* X, int ldx, int t, int pf, int forward,
                                const cplx* __restrict__ expkv);
}

// ===========================================================================
// C-ABI
using namespace pqmc;

#define CHK_CHAIN(c)                                                           \
  do {                                                                         \
    if (!(c)) { set_error("null chain handle"); return PQMC_ERR_ARG; }         \
  } while (0)

extern "C" {

const char* pqmc_version(void) { return "pqmc_gb300 1.0 (sm_103a)"; }
const char* pqmc_last_error(void) { return t_err.c_str(); }
int64_t pqmc_kernel_launches(void) { return g_launches.load(); }

int pqmc_create(const pqmc_model* model, pqmc_chain** out) {
  if (!out) { set_error("null out"); return PQMC_ERR_ARG; }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    set_error("pqmc_create: no CUDA device");
    return PQMC_ERR_CUDA;
  }
  pqmc_chain* c = new pqmc_chain();
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    set_error("stream creation failed");
    return PQMC_ERR_CUDA;
  }
  int st = chain_alloc(c, model, s);
  if (st != PQMC_OK) {
    chain_free(c);
    cudaStreamDestroy(s);
    delete c;
    return st;
  }
  c->hmodel = *model;
  c->hmodel.pf_dim = c->hmodel.pf_npla = c->hmodel.pf_k_exist = c->hmodel.pf_v_exist = nullptr;
  c->hmodel.pf_k_coe = c->hmodel.pf_v_coe = c->hmodel.pf_kmat = c->hmodel.pf_vmat = nullptr;
  c->hmodel.pla_site_list = c->hmodel.bf_list = c->hmodel.boundary_crossing = nullptr;
  c->hmodel.bc_phases = nullptr;
  *out = c;
  return PQMC_OK;
}

int pqmc_destroy(pqmc_chain* c) {
  if (!c) return PQMC_OK;
  cudaStreamSynchronize(c->stream);
  chain_free(c);
  cudaStreamDestroy(c->stream);
  delete c;
  return PQMC_OK;
}

int pqmc_set_field(pqmc_chain* c, const double* f) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(c->field, f, sizeof(double) * (size_t)c->n_bf * c->ntime, cudaMemcpyHostToDevice,
                            c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_set_field_slices(pqmc_chain* c, int first_time, int n_times, const double* f) {
  CHK_CHAIN(c);
  if (!f || first_time < 1 || n_times < 1 || first_time + n_times - 1 > c->ntime) {
    set_error("set_field_slices: slices %d..%d outside 1..%d", first_time, first_time + n_times - 1, c->ntime);
    return PQMC_ERR_ARG;
  }
  PQMC_CUDA(cudaMemcpyAsync(c->field + (size_t)c->n_bf * (first_time - 1), f, sizeof(double) * (size_t)c->n_bf * n_times,
                            cudaMemcpyHostToDevice, c->stream));
  PQMC_TRY(launch_init_expkv(c, first_time - 1, n_times));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_get_field_slices(pqmc_chain* c, int first_time, int n_times, double* f) {
  CHK_CHAIN(c);
  if (!f || first_time < 1 || n_times < 1 || first_time + n_times - 1 > c->ntime) {
    set_error("get_field_slices: slices %d..%d outside 1..%d", first_time, first_time + n_times - 1, c->ntime);
    return PQMC_ERR_ARG;
  }
  PQMC_CUDA(cudaMemcpyAsync(f, c->field + (size_t)c->n_bf * (first_time - 1), sizeof(double) * (size_t)c->n_bf * n_times,
                            cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_get_field(pqmc_chain* c, double* f) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(f, c->field, sizeof(double) * (size_t)c->n_bf * c->ntime, cudaMemcpyDeviceToHost,
                            c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_set_slater(pqmc_chain* c, const double* q, const double* d) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(c->slater_q, q, sizeof(cplx) * (size_t)c->ns * c->nelec, cudaMemcpyHostToDevice,
                            c->stream));
  PQMC_CUDA(cudaMemcpyAsync(c->slater_d, d, sizeof(cplx) * (size_t)c->nelec, cudaMemcpyHostToDevice, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_get_g(pqmc_chain* c, double* g) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(g, c->g, sizeof(cplx) * (size_t)c->ns * c->ns, cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_set_g(pqmc_chain* c, const double* g) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(c->g, g, sizeof(cplx) * (size_t)c->ns * c->ns, cudaMemcpyHostToDevice, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_get_state(pqmc_chain* c, pqmc_state* out) {
  CHK_CHAIN(c);
  if (!out) { set_error("null state"); return PQMC_ERR_ARG; }
  DevScalars h;
  PQMC_CUDA(cudaMemcpyAsync(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  out->ln_cw[0] = h.ln_cw.x;
  out->ln_cw[1] = h.ln_cw.y;
  out->err_fast_max = h.err_fast_max;
  out->err_fast = h.err_fast;
  out->err_g = h.err_g;
  out->err_g_rel_max = h.err_g_rel_max;
  out->positive_accept = h.pos_acc;
  out->negative_accept = h.neg_acc;
  for (int k = 0; k < 5; ++k) out->rng[k] = h.rng[k];
  out->reserved = 0;
  return PQMC_OK;
}

int pqmc_set_state(pqmc_chain* c, const pqmc_state* st) {
  CHK_CHAIN(c);
  if (!st) { set_error("null state"); return PQMC_ERR_ARG; }
  DevScalars h;
  PQMC_CUDA(cudaMemcpyAsync(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  h.err_fast_max = st->err_fast_max;
  h.err_fast = st->err_fast;
  h.err_g = st->err_g;
  h.err_g_rel_max = st->err_g_rel_max;
  h.pos_acc = st->positive_accept;
  h.neg_acc = st->negative_accept;
  for (int k = 0; k < 5; ++k) h.rng[k] = st->rng[k];
  PQMC_CUDA(cudaMemcpyAsync(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_set_rng(pqmc_chain* c, const int32_t rng[5]) {
  CHK_CHAIN(c);
  PQMC_CUDA(cudaMemcpyAsync(c->sc->rng, rng, sizeof(int32_t) * 5, cudaMemcpyHostToDevice, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_get_qd(pqmc_chain* c, int block, double* q, double* d) {
  CHK_CHAIN(c);
  if (block < 1 || block > c->nblock) { set_error("block %d out of range", block); return PQMC_ERR_ARG; }
  if (q)
    PQMC_CUDA(cudaMemcpyAsync(q, c->q_string + (size_t)c->ns * c->nelec * (block - 1),
                              sizeof(cplx) * (size_t)c->ns * c->nelec, cudaMemcpyDeviceToHost, c->stream));
  if (d)
    PQMC_CUDA(cudaMemcpyAsync(d, c->d_string + (size_t)c->nelec * (block - 1), sizeof(cplx) * (size_t)c->nelec,
                              cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_init_expkv(pqmc_chain* c) {
  CHK_CHAIN(c);
  PQMC_TRY(launch_init_expkv(c, 0, c->ntime));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_init_g(pqmc_chain* c, int start_time) {
  CHK_CHAIN(c);
  if (start_time < 1 || start_time > c->ntime) { set_error("start_time out of range"); return PQMC_ERR_ARG; }
  return do_init_g(c, start_time);
}

static int check_pf_time(pqmc_chain* c, int pf_id, int time) {
  if (pf_id < 1 || pf_id > c->n_pf || time < 1 || time > c->ntime) {
    set_error("pf_id %d / time %d out of range", pf_id, time);
    return PQMC_ERR_ARG;
  }
  return PQMC_OK;
}

int pqmc_update_phonon_field(pqmc_chain* c, int pf_id, int time) {
  CHK_CHAIN(c);
  PQMC_TRY(check_pf_time(c, pf_id, time));
  if (!c->h_pf_v_exist[pf_id - 1]) {
    set_error("update_phonon_field: family %d carries no boson field", pf_id);
    return PQMC_ERR_ARG;
  }
  PQMC_TRY(launch_update(c, pf_id - 1, time));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_left_evolve_g(pqmc_chain* c, int time, int pf_id, int two_way) {
  CHK_CHAIN(c);
  PQMC_TRY(check_pf_time(c, pf_id, time));
  if (!two_way) {
    set_error("left_evolve_g supports two_way=.true. only; use pqmc_left_evolve for one-way");
    return PQMC_ERR_ARG;
  }
  PQMC_TRY(launch_wrap(c, pf_id - 1, time, true));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_right_evolve_g(pqmc_chain* c, int time, int pf_id, int two_way) {
  CHK_CHAIN(c);
  PQMC_TRY(check_pf_time(c, pf_id, time));
  if (!two_way) {
    set_error("right_evolve_g supports two_way=.true. only; use pqmc_right_evolve for one-way");
    return PQMC_ERR_ARG;
  }
  PQMC_TRY(launch_wrap(c, pf_id - 1, time, false));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

// single-family one-way propagation of a caller matrix (Ns x n columns)
static int one_family_propagate(pqmc_chain* c, int time, int pf, cplx* dX, int n, bool forward) {
  size_t smem = sizeof(cplx) * (size_t)c->ns;
  k_propagate_one<<<n, 128, smem, c->stream>>>(c->M, dX, c->ns, time - 1, pf, forward ? 1 : 0, c->expkv);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int pqmc_left_evolve(pqmc_chain* c, int time, int pf_id, double* mat, int n) {
  CHK_CHAIN(c);
  PQMC_TRY(check_pf_time(c, pf_id, time));
  if (n < 1 || n > c->ns) { set_error("n out of range"); return PQMC_ERR_ARG; }
  cplx* d;
  PQMC_CUDA(cudaMallocAsync((void**)&d, sizeof(cplx) * (size_t)c->ns * n, c->stream));
  PQMC_CUDA(cudaMemcpyAsync(d, mat, sizeof(cplx) * (size_t)c->ns * n, cudaMemcpyHostToDevice, c->stream));
  int st = one_family_propagate(c, time, pf_id - 1, d, n, true);
  if (st == PQMC_OK)
    PQMC_CUDA(cudaMemcpyAsync(mat, d, sizeof(cplx) * (size_t)c->ns * n, cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaFreeAsync(d, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return st;
}

int pqmc_right_evolve(pqmc_chain* c, int time, int pf_id, double* mat, int n) {
  CHK_CHAIN(c);
  PQMC_TRY(check_pf_time(c, pf_id, time));
  if (n < 1 || n > c->ns) { set_error("n out of range"); return PQMC_ERR_ARG; }
  // mat is (n, Ns); work on its adjoint X = mat^H (Ns, n)
  cplx *d, *x;
  PQMC_CUDA(cudaMallocAsync((void**)&d, sizeof(cplx) * (size_t)c->ns * n, c->stream));
  PQMC_CUDA(cudaMallocAsync((void**)&x, sizeof(cplx) * (size_t)c->ns * n, c->stream));
  PQMC_CUDA(cudaMemcpyAsync(d, mat, sizeof(cplx) * (size_t)c->ns * n, cudaMemcpyHostToDevice, c->stream));
  PQMC_TRY(herm_t(c->stream, n, c->ns, d, x));
  int st = one_family_propagate(c, time, pf_id - 1, x, n, false);
  PQMC_TRY(herm_t(c->stream, c->ns, n, x, d));
  if (st == PQMC_OK)
    PQMC_CUDA(cudaMemcpyAsync(mat, d, sizeof(cplx) * (size_t)c->ns * n, cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaFreeAsync(d, c->stream));
  PQMC_CUDA(cudaFreeAsync(x, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return st;
}

int pqmc_get_g_scratch(pqmc_chain* c, int time, int forward, int loop, double* err_out) {
  CHK_CHAIN(c);
  if (!c->have_g) { set_error("get_g_scratch before init_g"); return PQMC_ERR_STATE; }
  PQMC_TRY(do_g_scratch(c, time, forward != 0, loop));
  if (err_out) {
    DevScalars h;
    PQMC_CUDA(cudaMemcpy(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost));
    err_out[0] = h.err_g;
    err_out[1] = h.err_w;
  }
  return PQMC_OK;
}

int pqmc_cal_new_weight(pqmc_chain* c, double* ln_cw_out) {
  CHK_CHAIN(c);
  if (!c->have_g) { set_error("cal_new_weight before init_g"); return PQMC_ERR_STATE; }
  PQMC_TRY(do_new_weight(c));
  if (ln_cw_out) {
    DevScalars h;
    PQMC_CUDA(cudaMemcpy(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost));
    ln_cw_out[0] = h.ln_cw.x;
    ln_cw_out[1] = h.ln_cw.y;
  }
  return PQMC_OK;
}

}  // extern "C"

namespace pqmc {
// propagation of one family at one slice (used by the one-way C entry points)
__global__ void k_propagate_one(DevModel M, cplx* X, int ldx, int t, int pf, int forward,
                                const cplx* __restrict__ expkv) {
  extern __shared__ cplx col[];
  const int ns = M.ns, pd = M.pdim;
  cplx* x = X + (size_t)ldx * blockIdx.x;
  for (int r = threadIdx.x; r < ns; r += blockDim.x) col[r] = x[r];
  __syncthreads();
  const int dim = M.pf_dim[pf], npla = M.pf_npla[pf];
  for (int p = threadIdx.x; p < npla; p += blockDim.x) {
    int S[4];
    cplx v[4];
    for (int k = 0; k < dim; ++k) {
      S[k] = M.site[k + pd * (p + M.max_pla * pf)];
      v[k] = col[S[k]];
    }
    const cplx* E = expkv + M.kv_base(p, pf, t);
    for (int a = 0; a < dim; ++a) {
      cplx s = mk(0.0);
      for (int k = 0; k < dim; ++k) {
        cplx e = forward ? E[a + pd * k] : cconj(E[k + pd * a]);
        s = cfma(e, v[k], s);
      }
      col[S[a]] = s;
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < ns; r += blockDim.x) x[r] = col[r];
}
}  // namespace pqmc
