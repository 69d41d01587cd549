// adjoint.cu -- gradient of the projector log-weight
//   W(x) = Re log det(P^H B(Lt..1) P),  B(tau) = E_{n_pf}(tau) ... E_1(tau)
// with respect to every phonon field x_{b,tau}.  The value is
// cal_new_weight_T0 (src/mod_evolution.f90:359-408); the gradient is the
// Green's-function trace formula
//   dW/dx_{b,tau} = c Re Tr[E_p^-1 dE_p/dx  G_before(S_p,S_p)]
// where p is the plaquette carrying boson b in family f, G_before is the
// equal-time Green's function R'(L'R')^-1 L' positioned just before E_f(tau)
// acts (the matrix the local update at (f,tau) sees), and c = ncopy (x2 under
// TR_weight).
//
// Reverse sweep with checkpoints: one right-to-left pass gives the value
// (cal_new_weight_T0 from the trial state) and stores the orthonormal left
// factor every ngroup slices; a left-to-right pass recomputes
// G from the left checkpoint and the current right factor at each block start
// and wraps it family by family through the block (the slices between
// checkpoints are recomputed, not stored).
#include "chain.cuh"
#include "linalg.cuh"
#include "update_dev.cuh"

namespace pqmc {

// dE/dx of the closed-form propagators (get_expKV_epsocz / _epsoc /
// epsocz_block), entry (i,j); the general generator uses a central
// difference of dev_get_expkv.
__device__ cplx closed_dentry(const DevModel& M, int pf, int pla, double x, int i, int j) {
  const int pd = M.pdim, dim = M.pf_dim[pf];
  const cplx kc = M.k_coe[pf], vc = M.v_coe[pf];
  const cplx* K = M.kmat + (size_t)pd * pd * pf;
  const cplx* V = M.vmat + (size_t)pd * pd * pf;
  const cplx* BC = M.bcp + (size_t)pd * pd * (pla + (size_t)M.max_pla * pf);
  const bool cross = M.cross[pla + M.max_pla * pf] != 0;
  // norm(x) and dnorm/dx
  double norm, dnorm;
  if (M.expkv_kind == PQMC_EXPKV_EPSOCZ_BLOCK) {
    const cplx vx = cscale(vc, x);
    cplx h11 = cadd(cmul(kc, K[0 + pd * 2]), cmul(vx, V[0 + pd * 2]));
    cplx h21 = cadd(cmul(kc, K[1 + pd * 2]), cmul(vx, V[1 + pd * 2]));
    cplx d11 = cmul(vc, V[0 + pd * 2]), d21 = cmul(vc, V[1 + pd * 2]);
    double s = cabs2(h11) + cabs2(h21);
    norm = M.delt * sqrt(s);
    double ds = 2.0 * (h11.x * d11.x + h11.y * d11.y + h21.x * d21.x + h21.y * d21.y);
    dnorm = M.delt * ds / (2.0 * sqrt(s));
  } else {
    double a = cabsd(kc), b = cabsd(vc);
    double s = a * a + (b * x) * (b * x);
    norm = M.delt * sqrt(s);
    dnorm = M.delt * (b * b * x) / sqrt(s);
  }
  const double ch = cosh(norm), sh = sinh(norm);
  if (i == j) return mk(sh * dnorm);
  const int h = dim / 2;
  bool upper = (i < h && j >= h), lower = (i >= h && j < h);
  if (!upper && !lower) return mk(0.0);
  int a = upper ? i : j, b = upper ? j : i;
  if (M.expkv_kind == PQMC_EXPKV_EPSOC && !(a == 0 && b == 1)) return mk(0.0);
  cplx hab = cadd(cmul(kc, K[a + pd * b]), cmul(cscale(vc, x), V[a + pd * b]));
  cplx dh = cmul(vc, V[a + pd * b]);
  cplx sub = cscale(hab, -M.delt), dsub = cscale(dh, -M.delt);
  if (cross) {
    sub = cmul(sub, BC[a + pd * b]);
    dsub = cmul(dsub, BC[a + pd * b]);
  }
  // d/dx [sub sinh(n)/n] = dsub sinh/n + sub (cosh n - sinh/n) dn / n
  double f = sh / norm, df = (ch - f) * dnorm / norm;
  cplx e = cadd(cscale(dsub, f), cscale(sub, df));
  return upper ? e : cconj(e);
}

// Gradient of one family at one slice: grad(b, t) for the family's plaquettes.
__global__ void k_grad_family(DevModel M, int pf, int t, const cplx* __restrict__ G, const double* __restrict__ field,
                              const cplx* __restrict__ expkv_inv, double* grad, double scale) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= M.pf_npla[pf] || !M.pf_v_exist[pf]) return;
  const int dim = M.pf_dim[pf], pd = M.pdim, ns = M.ns;
  const int b = M.bf[p + M.max_pla * pf];
  const double x = field[b + (size_t)M.n_bf * t];
  int S[4];
  for (int k = 0; k < dim; ++k) S[k] = M.site[k + pd * (p + M.max_pla * pf)];
  cplx dE[16];
  if (M.expkv_kind == PQMC_EXPKV_GENERAL) {
    cplx ep[16], em[16];
    const double h = 1e-5 * (1.0 + fabs(x));
    dev_get_expkv(M, pf, p, x + h, false, ep);
    dev_get_expkv(M, pf, p, x - h, false, em);
    for (int k = 0; k < dim * dim; ++k) dE[k] = cscale(csub(ep[k], em[k]), 0.5 / h);
  } else {
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) dE[i + dim * j] = closed_dentry(M, pf, p, x, i, j);
  }
  // A = E^-1 dE (expKV_inv is E^-1), trace with G(S,S):  sum_ab A_ab G(S_b, S_a)
  const cplx* Ei = expkv_inv + M.kv_base(p, pf, t);
  cplx tr = mk(0.0);
  for (int a = 0; a < dim; ++a)
    for (int bb = 0; bb < dim; ++bb) {
      cplx aab = mk(0.0);
      for (int k = 0; k < dim; ++k) aab = cfma(Ei[a + pd * k], dE[k + dim * bb], aab);
      tr = cfma(aab, G[S[bb] + (size_t)ns * S[a]], tr);
    }
  grad[b + (size_t)M.n_bf * t] = scale * tr.x;
}

int launch_propagate(pqmc_chain* c, cplx* X, int n, int t_from, int t_to, bool forward);
int launch_wrap(pqmc_chain* c, int pf, int time, bool left);

}  // namespace pqmc

using namespace pqmc;

extern "C" int pqmc_cal_new_weight(pqmc_chain* c, double* ln_cw_out);

extern "C" int pqmc_set_field_device(pqmc_chain* c, const double* dfield) {
  if (!c || !dfield) { set_error("set_field_device: null argument"); return PQMC_ERR_ARG; }
  PQMC_CUDA(cudaMemcpyAsync(c->field, dfield, sizeof(double) * (size_t)c->n_bf * c->ntime, cudaMemcpyDeviceToDevice,
                            c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

// logw_out: host, 2 doubles (complex log-weight as cal_new_weight_T0);
// grad_dev: device, (n_bf, ntime) doubles (gradient of Re logw).
extern "C" int pqmc_logweight_grad(pqmc_chain* c, double* logw_out, double* grad_dev) {
  if (!c || !grad_dev) { set_error("logweight_grad: null argument"); return PQMC_ERR_ARG; }
  if (c->finite_t) { set_error("logweight_grad: the projector log-weight only (the chain is at finite temperature)"); return PQMC_ERR_STATE; }
  const int ns = c->ns, ne = c->nelec, nt = c->ntime, ng = c->ngroup;
  cudaStream_t s = c->stream;
  const size_t qb = sizeof(cplx) * (size_t)ns * ne;
  const int nck = nt / ng + 1;
  cplx* ck = nullptr;
  PQMC_CUDA(cudaMallocAsync((void**)&ck, qb * nck, s));
  // right-to-left pass: cal_new_weight_T0 with the orthonormal left factor
  // checkpointed every ngroup slices (one propagation for value and
  // checkpoints)
  int st = do_new_weight_ck(c, ck);
  int info = 0;
  DevScalars h;
  if (st == PQMC_OK && (cudaMemcpyAsync(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess)) {
    set_error("logweight_grad: reading the weight failed");
    st = PQMC_ERR_CUDA;
  }
  if (st == PQMC_OK) info = h.lu_info;
  if (st == PQMC_OK && info != 0) {
    set_error("logweight_grad: zero pivot %d", info);
    st = PQMC_ERR_SINGULAR;
  }
  if (st != PQMC_OK) {
    cudaFreeAsync(ck, s);
    return st;
  }
  if (logw_out) {
    logw_out[0] = h.ln_cw.x;
    logw_out[1] = h.ln_cw.y;
  }
  // forward pass: R starts as the trial state; at each block start G from the checkpoint
  PQMC_CUDA(cudaMemcpyAsync(c->rmat, c->slater_q, qb, cudaMemcpyDeviceToDevice, s));
  const double scale = (double)c->M.ncopy * (c->M.tr_weight ? 2.0 : 1.0);
  cplx* gsave = c->g;   // keep the chain's G: compute into the pair (g, g_alt) then restore
  cplx* gsave_alt = c->g_alt;
  cplx* gtmp = nullptr;
  PQMC_CUDA(cudaMallocAsync((void**)&gtmp, sizeof(cplx) * (size_t)ns * ns, s));
  PQMC_CUDA(cudaMemcpyAsync(gtmp, c->g, sizeof(cplx) * (size_t)ns * ns, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaMemsetAsync(grad_dev, 0, sizeof(double) * (size_t)c->n_bf * nt, s));
  for (int t0 = 0; t0 < nt; t0 += ng) {
    const int t1 = (t0 + ng < nt) ? t0 + ng : nt;
    // G = R (L R)^-1 L with L = ck[slot]^H, slot = t1/ng (left part covers slices > t1)... the
    // left factor that pairs with R at tau = t0 is the checkpoint at t0
    const cplx* Xl = ck + (size_t)ns * ne * (t0 / ng);
    PQMC_TRY(zgemm(s, 'C', 'N', ne, ne, ns, mk(1.0), Xl, ns, c->rmat, ns, mk(0.0), c->pbp, ne));
    PQMC_TRY(lu_factor(s, ne, c->pbp, c->ipiv, &c->sc->lu_info, c->lcol));
    PQMC_TRY(herm_t(s, ns, ne, Xl, c->lmat));
    PQMC_TRY(lu_solve(s, ne, ns, c->pbp, c->ipiv, c->lmat, ne));
    PQMC_TRY(zgemm(s, 'N', 'N', ns, ns, ne, mk(1.0), c->rmat, ns, c->lmat, ne, mk(0.0), c->g, ns));
    for (int tau = t0 + 1; tau <= t1; ++tau) {
      for (int pf = 0; pf < c->n_pf; ++pf) {
        const int npla = c->h_pf_npla[pf];
        if (npla > 0 && c->h_pf_v_exist[pf]) {
          k_grad_family<<<(npla + 63) / 64, 64, 0, s>>>(c->M, pf, tau - 1, c->g, c->field, c->expkv_inv, grad_dev, scale);
          PQMC_LAUNCHED();
        }
        PQMC_TRY(launch_wrap(c, pf, tau, true));
      }
    }
    PQMC_TRY(launch_propagate(c, c->rmat, ne, t0 + 1, t1, true));
    if (t1 < nt) PQMC_TRY(house_qr(s, ns, ne, c->rmat, c->tau, c->dtmp));
  }
  // restore the chain's Green's function
  c->g = gsave;
  c->g_alt = gsave_alt;
  PQMC_CUDA(cudaMemcpyAsync(c->g, gtmp, sizeof(cplx) * (size_t)ns * ns, cudaMemcpyDeviceToDevice, s));
  PQMC_CUDA(cudaFreeAsync(gtmp, s));
  PQMC_CUDA(cudaFreeAsync(ck, s));
  PQMC_CUDA(cudaStreamSynchronize(s));
  return PQMC_OK;
}
