// update.cu -- update_phonon_field(ppf, time) (src/mod_update.f90:13-245,
// 475-500) as one cooperative kernel per family step.
//
// Phase 0: one thread draws the family's whole ran2 stream (each proposal
//          consumes a fixed number of draws, :84 and :117).
// Phase 1: every CTA prepares some plaquettes in parallel: jump, phonon
//          action difference (:203-228), the new propagators and
//          Delta = expKV_inv(old) expKV(new) - I (:230-245).
// Phase 2: warp 0 of CTA 0 walks the plaquettes in the reference's Markov
//          order: R = I + G_SS Delta, det R, Metropolis test (:97-119).  An
//          accepted move is published as (S, T = Delta R^-1); at the next
//          grid barrier every other CTA applies it out of place,
//          G' = G + G(:,S) T (I - G)(S,:) (:146-187), while the proposer
//          scans ahead with G plus that move's correction on the block it
//          needs.  One barrier per accepted move, none per rejection.
#include <cooperative_groups.h>
#include "chain.cuh"
#include "linalg.cuh"
#include "rng.cuh"
#include "update_dev.cuh"

namespace cg = cooperative_groups;

namespace pqmc {

// Metropolis / heat-bath threshold on |det R|^2 (cal_prob, src/mod_update.f90:
// 475-500, with the weight ratio of :101-108).  The ratio's modulus is
// |det|^n with n = ncopy (x2 under TR_weight); exp(min(10,w)) >= r with
// w = dE + log|det|^n  <=>  |det|^2 >= (r e^{-dE})^{2/n}.
__device__ __forceinline__ double accept_threshold(const DevModel& M, double dE, double r) {
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

__device__ __forceinline__ float2 cf(cplx a) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ float2 fmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// FP32 4x4 determinant over six lanes (Laplace along rows 1,2) and the sum of
// the term magnitudes, used as an error scale.
__device__ void warp_det_f32(const float2* R, int lane, float2* det, float* mag) {
  float2 v = make_float2(0.f, 0.f);
  float m = 0.f;
  if (lane < 6) {
    const int J[6] = {0, 0, 0, 1, 1, 2}, K[6] = {1, 2, 3, 2, 3, 3};
    const int L[6] = {2, 1, 1, 0, 0, 0}, Mm[6] = {3, 3, 2, 3, 2, 1};
    const float sg[6] = {1.f, -1.f, 1.f, 1.f, -1.f, 1.f};
    int j = J[lane], k = K[lane], l = L[lane], mm = Mm[lane];
    float2 mi = fsub(fmul(R[0 + 4 * j], R[1 + 4 * k]), fmul(R[0 + 4 * k], R[1 + 4 * j]));
    float2 co = fsub(fmul(R[2 + 4 * l], R[3 + 4 * mm]), fmul(R[2 + 4 * mm], R[3 + 4 * l]));
    float2 t = fmul(mi, co);
    v = make_float2(sg[lane] * t.x, sg[lane] * t.y);
    m = hypotf(mi.x, mi.y) * hypotf(co.x, co.y);
  }
  for (int o = 4; o > 0; o >>= 1) {
    float vx = __shfl_down_sync(0xffffffffu, v.x, o), vy = __shfl_down_sync(0xffffffffu, v.y, o);
    float mo = __shfl_down_sync(0xffffffffu, m, o);
    if (lane + o < 8) {
      v.x += vx;
      v.y += vy;
      m += mo;
    }
  }
  det->x = __shfl_sync(0xffffffffu, v.x, 0);
  det->y = __shfl_sync(0xffffffffu, v.y, 0);
  *mag = __shfl_sync(0xffffffffu, m, 0);
}

__global__ void __launch_bounds__(256) k_update(DevModel M, DevScalars* sc, UpdCtl* ctl, PlaqPre* pre,
                                                 double* field, cplx* expkv, cplx* expkv_inv, cplx* gA,
                                                 cplx* gB, int pf, int t) {
  cg::grid_group grid = cg::this_grid();
  const int ns = M.ns, dim = M.pf_dim[pf], npla = M.pf_npla[pf], pd = M.pdim;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ cplx s_g[16], s_r[16], s_c1[16], s_tp[16], s_cof[16];
  __shared__ float2 s_rf[16], s_c1f[16], s_tpf[16];
  __shared__ int s_Sp[4];

  // ---- phase 0: the family's ran2 stream ----------------------------------
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Ran2Dev rng;
    rng.iran = sc->rng[0]; rng.jran = sc->rng[1]; rng.kran = sc->rng[2];
    rng.mran = sc->rng[3]; rng.nran = sc->rng[4];
    for (int p = 0; p < npla; ++p) {
      if (M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
        float u1 = rng.next(), u2 = rng.next();
        pre[p].xnew = (double)u1;
        pre[p].dE = (double)u2;
      } else {
        pre[p].xnew = (double)rng.ran_sysm();      // :84
      }
      pre[p].r = (double)rng.next();               // :117
    }
    sc->rng[0] = rng.iran; sc->rng[1] = rng.jran; sc->rng[2] = rng.kran;
    sc->rng[3] = rng.mran; sc->rng[4] = rng.nran;
  }
  grid.sync();

  // ---- phase 1: proposals of all plaquettes in parallel (one warp each) ----
  {
    const int wpb = blockDim.x >> 5;
    const bool closed = (M.expkv_kind != PQMC_EXPKV_GENERAL);
    for (int p = blockIdx.x * wpb + warp; p < npla; p += gridDim.x * wpb) {
      const int b = M.bf[p + M.max_pla * pf];
      double jump;
      if (M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
        double u1 = __ldcg(&pre[p].xnew), u2 = __ldcg(&pre[p].dE);
        jump = pqmc_bm_gauss_jump(M.jump, u1, u2);   // bit-identical with the oracle
      } else {
        jump = M.jump * __ldcg(&pre[p].xnew);
      }
      double xold = field[b + (size_t)M.n_bf * t];
      double xnew = xold + jump;                                  // :92
      double norm = 0.0, ch = 0.0, sh = 0.0;
      if (lane == 0) {
        double dE = -M.delt * energy_diff(M, field, b, t, jump);  // :87-88
        pre[p].dE = dE;
        pre[p].thr = accept_threshold(M, dE, __ldcg(&pre[p].r));
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
      // Delta = expKV_inv(old) * expKV(new) - I   :240-243
      const size_t base = M.kv_base(p, pf, t);
      cplx a = mk(0.0);
      for (int k = 0; k < dim; ++k) {
        cplx ekj = shfl_c(en, k + dim * j);
        if (act) a = cfma(expkv_inv[base + i + pd * k], ekj, a);
      }
      if (act) {
        if (i == j) a = csub(a, mk(1.0));
        pre[p].delta[lane] = a;
        pre[p].deltaf[lane] = cf(a);
      }
      if (lane == 0) pre[p].xnew = xnew;
    }
  }
  grid.sync();

  // ---- phase 2: sequential Metropolis scan + distributed rank-dim updates ---
  __shared__ int s_sites[4 * 512];
  __shared__ cplx s_G0[16], s_G1[16], s_G2[16], s_D[16];
  if (blockIdx.x == 0)
    for (int e = threadIdx.x; e < npla * dim && e < 4 * 512; e += blockDim.x)
      s_sites[e] = M.site[(e % dim) + pd * ((e / dim) + M.max_pla * pf)];
  __syncthreads();
  cplx* gcur = gA;
  cplx* gnext = gB;
  int prev = -1, step = 0, next = 0;
  // ln_cw += log(real(R_elec)) per accept (:142), kept as a product
  // mantissa * 2^expo and logged once at the end
  double lprod = 1.0;
  long long lexp = 0;
  long long pa = 0, na = 0;
  for (;;) {
    UpdCtl* cw = ctl + (step & 1);
    const UpdCtl* cr = ctl + ((step + 1) & 1);
    if (blockIdx.x == 0) {
      if (warp == 0) {
        const bool has_prev = step > 0;
        int found = -1;
        const int i = lane % dim, j = lane / dim;
        const bool act = lane < dim * dim;
        for (int p = next; p < npla; ++p) {
          const int* Sp = s_sites + p * dim;
          const PlaqPre* pp = pre + p;
          // one round trip: G(S,S), G(S,S') and G(S',S) of the pending move, Delta
          cplx g0 = mk(0.0), g1 = mk(0.0), g2 = mk(0.0), dl = mk(0.0);
          float2 dlf = make_float2(0.f, 0.f);
          if (act) {
            g0 = ldg_c(gcur + Sp[i] + (size_t)ns * Sp[j]);
            if (has_prev) {
              g1 = ldg_c(gcur + Sp[i] + (size_t)ns * s_Sp[j]);     // G(S_i, S'_j)
              g2 = ldg_c(gcur + s_Sp[i] + (size_t)ns * Sp[j]);     // G(S'_i, S_j)
            }
            dl = ldg_c(&pp->delta[lane]);
            dlf = pp->deltaf[lane];
          }
          const double thr = __ldcg(&pp->thr);
          if (act) {
            s_G0[lane] = g0;
            s_G1[lane] = g1;
            s_G2[lane] = g2;
            s_D[lane] = dl;
            s_rf[lane] = dlf;   // Delta in FP32 (reused below)
          }
          __syncwarp();
          int decide = 0;   // 0: needs FP64, -1 reject, +1 accept
          if (dim == 4) {
            // FP32 screen: reject early when |det R|^2 is clearly below thr
            float2 gv = cf(g0);
            if (act && has_prev) {
              float2 a = make_float2(0.f, 0.f);
              for (int m = 0; m < dim; ++m) a = fadd(a, fmul(cf(s_G1[i + dim * m]), s_tpf[m + dim * j]));
              s_c1f[lane] = a;
            }
            __syncwarp();
            if (act && has_prev) {
              float2 a = make_float2(0.f, 0.f);
              for (int l = 0; l < dim; ++l) {
                float2 v = cf(cneg(s_G2[l + dim * j]));
                if (s_Sp[l] == Sp[j]) v.x += 1.f;
                a = fadd(a, fmul(s_c1f[i + dim * l], v));
              }
              gv = fadd(gv, a);
            }
            __syncwarp();
            if (act) s_c1f[lane] = gv;
            __syncwarp();
            float2 rf = make_float2(i == j ? 1.f : 0.f, 0.f);
            if (act)
              for (int k = 0; k < dim; ++k) rf = fadd(rf, fmul(s_c1f[i + dim * k], s_rf[k + dim * j]));
            __syncwarp();
            if (act) s_rf[lane] = rf;
            __syncwarp();
            float2 df;
            float mag;
            warp_det_f32(s_rf, lane, &df, &mag);
            const double d2 = (double)df.x * df.x + (double)df.y * df.y;
            const double tol = 1e-4 * ((double)mag * mag + thr);
            if (d2 < thr - tol) decide = -1;
            else if (d2 > thr + tol) decide = 1;
          }
          if (decide < 0) {
            if (lane == 0) na++;
            continue;
          }
          // FP64 path: exact ratio for accepted moves and near-ties
          cplx gv = g0;
          if (act && has_prev) {
            cplx a = mk(0.0);
            for (int m = 0; m < dim; ++m) a = cfma(s_G1[i + dim * m], s_tp[m + dim * j], a);
            s_c1[lane] = a;
          }
          __syncwarp();
          if (act && has_prev) {
            cplx a = mk(0.0);
            for (int l = 0; l < dim; ++l) {
              cplx v = cneg(s_G2[l + dim * j]);
              if (s_Sp[l] == Sp[j]) v = cadd(v, mk(1.0));
              a = cfma(s_c1[i + dim * l], v, a);
            }
            gv = cadd(gv, a);
          }
          if (act) s_g[lane] = gv;
          __syncwarp();
          // R = I + g_h_sub * Delta    :97-100
          if (act) {
            cplx a = mk(0.0);
            for (int k = 0; k < dim; ++k) a = cfma(s_g[i + dim * k], s_D[k + dim * j], a);
            if (i == j) a = cadd(a, mk(1.0));
            s_r[lane] = a;
          }
          __syncwarp();
          cplx det;
          if (dim == 4) {
            // cofactors on 16 lanes; det = sum_j R(0,j) cof(0,j)
            cplx cof = mk(0.0);
            const int ci = lane & 3, cj = lane >> 2;
            if (lane < 16) {
              int r3[3], c3[3], n = 0;
              for (int k = 0; k < 4; ++k)
                if (k != ci) r3[n++] = k;
              n = 0;
              for (int k = 0; k < 4; ++k)
                if (k != cj) c3[n++] = k;
#define S3(a_, b_) s_r[r3[a_] + 4 * c3[b_]]
              cof = cadd(csub(cmul(S3(0, 0), csub(cmul(S3(1, 1), S3(2, 2)), cmul(S3(1, 2), S3(2, 1)))),
                              cmul(S3(0, 1), csub(cmul(S3(1, 0), S3(2, 2)), cmul(S3(1, 2), S3(2, 0))))),
                         cmul(S3(0, 2), csub(cmul(S3(1, 0), S3(2, 1)), cmul(S3(1, 1), S3(2, 0)))));
#undef S3
              if ((ci + cj) & 1) cof = cneg(cof);
              s_cof[lane] = cof;
            }
            __syncwarp();
            det = mk(0.0);
            for (int k = 0; k < 4; ++k) det = cfma(s_r[0 + 4 * k], s_cof[0 + 4 * k], det);
          } else {
            det = warp_det(dim, s_r, lane);
          }
          const int acc = (det.x * det.x + det.y * det.y) >= thr;   // :112-117
          if (!acc) {
            if (lane == 0) na++;
            continue;
          }
          // accepted :122-187
          if (lane == 0) {
            pa++;
            cplx relec = det;
            if (M.tr_weight) relec = cmul(relec, cconj(relec));
            cplx base = relec, ac = mk(1.0);
            for (int k = 0; k < M.ncopy; ++k) ac = cmul(ac, base);
            int ex;
            lprod *= frexp(ac.x, &ex);
            lexp += ex;
            double m2 = frexp(lprod, &ex);
            lprod = m2;
            lexp += ex;
            field[M.bf[p + M.max_pla * pf] + (size_t)M.n_bf * t] = __ldcg(&pp->xnew);
          }
          {
            const size_t base2 = M.kv_base(p, pf, t);
            if (lane < pd * pd) {
              int ii = lane % pd, jj = lane / pd;
              bool in = ii < dim && jj < dim;
              expkv[base2 + lane] = in ? ldg_c(&pp->enew[ii + dim * jj]) : mk(0.0);
              expkv_inv[base2 + lane] = in ? ldg_c(&pp->einv[ii + dim * jj]) : mk(0.0);
            }
          }
          if (dim == 4) {
            cplx rd = mk(0.0);
            if (lane == 0) rd = cdiv(mk(1.0), det);
            rd = shfl_c(rd, 0);
            if (lane < 16) s_c1[(lane >> 2) + 4 * (lane & 3)] = cmul(s_cof[lane], rd);   // R^-1 = adj/det
            __syncwarp();
          } else {
            if (lane < dim * dim) s_c1[lane] = s_r[lane];
            __syncwarp();
            if (lane == 0) dev_inverse_small(dim, s_c1);                     // :171
            __syncwarp();
          }
          if (act) {
            cplx a = mk(0.0);
            for (int k = 0; k < dim; ++k) a = cfma(s_D[i + dim * k], s_c1[k + dim * j], a);
            s_tp[lane] = a;                                                  // T = Delta R^-1  :173
            s_tpf[lane] = cf(a);
            cw->T[lane] = a;
          }
          if (lane < dim) {
            cw->S[lane] = Sp[lane];
            s_Sp[lane] = Sp[lane];
          }
          __syncwarp();
          found = p;
          break;
        }
        if (lane == 0) {
          cw->p = found;
          cw->dim = dim;
        }
        next = (found >= 0) ? found + 1 : npla;
      }
    } else if (prev >= 0) {
      // G' = G + G(:,S) W,  W = T (I - G)(S,:)
      __shared__ cplx s_wc[4];
      __shared__ int s_s[4];
      __shared__ cplx s_T[16];
      if (threadIdx.x < dim) s_s[threadIdx.x] = cr->S[threadIdx.x];
      if (threadIdx.x < dim * dim) s_T[threadIdx.x] = ldg_c(&cr->T[threadIdx.x]);
      __syncthreads();
      const long total = (long)ns * ns;
      const int nw = gridDim.x - 1;
      const long chunk = (total + nw - 1) / nw;
      const long e0 = (long)(blockIdx.x - 1) * chunk;
      const long e1 = (e0 + chunk < total) ? e0 + chunk : total;
      if (e0 < e1) {
        const int c0 = (int)(e0 / ns), c1 = (int)((e1 - 1) / ns);
        for (int col = c0; col <= c1; ++col) {
          if (threadIdx.x < dim) {
            const int k = threadIdx.x;
            cplx a = mk(0.0);
            for (int l = 0; l < dim; ++l) {
              cplx v = cneg(ldg_c(gcur + s_s[l] + (size_t)ns * col));
              if (s_s[l] == col) v = cadd(v, mk(1.0));
              a = cfma(s_T[k + dim * l], v, a);
            }
            s_wc[k] = a;
          }
          __syncthreads();
          long lo = (long)col * ns, hi = lo + ns;
          if (lo < e0) lo = e0;
          if (hi > e1) hi = e1;
          for (long e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            const int r = (int)(e - (long)col * ns);
            cplx a = ldg_c(gcur + e);
            for (int k = 0; k < dim; ++k) a = cfma(ldg_c(gcur + r + (size_t)ns * s_s[k]), s_wc[k], a);
            gnext[e] = a;
          }
          __syncthreads();
        }
      }
    }
    grid.sync();
    if (prev >= 0) {
      cplx* tmp = gcur;
      gcur = gnext;
      gnext = tmp;
    }
    prev = __ldcg(&cw->p);
    ++step;
    if (prev < 0) break;
  }
  if (gcur != gA) {
    const long total = (long)ns * ns;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x)
      gA[e] = ldg_c(gcur + e);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (pa > 0) {
      double l = (lprod > 0.0) ? log(lprod) + (double)lexp * 0.69314718055994530942 : log(lprod);
      sc->ln_cw = cadd(sc->ln_cw, mk(l));
    }
    sc->pos_acc += pa;
    sc->neg_acc += na;
  }
}

int update_setup(pqmc_chain* c) {
  long elems = (long)c->ns * c->ns;
  int want = 1 + (int)((elems + 1023) / 1024);
  int npla_max = 0;
  for (int n : c->h_pf_npla) npla_max = n > npla_max ? n : npla_max;
  if (want < (npla_max + 7) / 8) want = (npla_max + 7) / 8;
  if (want < 2) want = 2;
  for (int f = 0; f < c->n_pf; ++f)
    if (c->h_pf_npla[f] * c->h_pf_dim[f] > 4 * 512) {
      set_error("update kernel stages at most 2048 plaquette sites per family");
      return PQMC_ERR_ARG;
    }
  c->upd_blocks = coop_grid((const void*)k_update, 256, want);
  if (c->upd_blocks < 2) {
    set_error("update kernel needs two co-resident blocks");
    return PQMC_ERR_CUDA;
  }
  return PQMC_OK;
}

int launch_update(pqmc_chain* c, int pf, int time) {
  int t = time - 1;
  void* args[] = {&c->M, &c->sc, &c->ctl, &c->pre, &c->field, &c->expkv, &c->expkv_inv, &c->g, &c->g_alt, &pf, &t};
  PQMC_CUDA(cudaLaunchCooperativeKernel((const void*)k_update, c->upd_blocks, 256, args, 0, c->stream));
  PQMC_LAUNCHED();
  return PQMC_OK;
}

}  // namespace pqmc
