// expkv.cuh -- the plaquette propagator exp(-/+ dtau (K_coe K + V_coe x V))
// on the device, for the four generators of the procedure pointer get_expKV
// (setup_expKV, src/mod_phonon_field.f90:472-496).
#pragma once
#include "common.cuh"

// Device view of the flattened model (pqmc_model).
struct DevModel {
  int ns, nelec, ntime, ngroup, nblock, n_pf, pdim, max_pla, n_bf;
  int expkv_kind, ncopy, tr_weight, metropolis, greatest_decent, local_update, proposal_kind;
  double delt, mass, stiff, biased, jump;
  const int* pf_dim;
  const int* pf_npla;
  const int* pf_k_exist;
  const int* pf_v_exist;
  const cplx* k_coe;
  const cplx* v_coe;
  const cplx* kmat;      // (pdim,pdim,n_pf)
  const cplx* vmat;
  const int* site;       // (pdim,max_pla,n_pf)
  const int* bf;         // (max_pla,n_pf)
  const int* cross;      // (max_pla,n_pf)
  const cplx* bcp;       // (pdim,pdim,max_pla,n_pf)

  __host__ __device__ __forceinline__ size_t kv_idx(int i, int j, int pla, int pf, int t) const {
    return (size_t)i + (size_t)pdim * (j + (size_t)pdim * (pla + (size_t)max_pla * (pf + (size_t)n_pf * t)));
  }
  __host__ __device__ __forceinline__ size_t kv_base(int pla, int pf, int t) const {
    return (size_t)pdim * pdim * (pla + (size_t)max_pla * (pf + (size_t)n_pf * t));
  }
};

// Real symmetric Jacobi on the 2n x 2n embedding of a Hermitian n x n matrix
// (n <= 4); see get_expKV_general (src/mod_phonon_field.f90:497-532) and
// zexpm (src/mod_matrixlib.f90:251-289).
__device__ inline void dev_sym_jacobi(int n, double* a, double* w, double* v) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) v[i + n * j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < j; ++i) off += a[i + n * j] * a[i + n * j];
    if (off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a[p + n * q];
        if (apq == 0.0) continue;
        double theta = (a[q + n * q] - a[p + n * p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = a[k + n * p], akq = a[k + n * q];
          a[k + n * p] = c * akp - s * akq;
          a[k + n * q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = a[p + n * k], aqk = a[q + n * k];
          a[p + n * k] = c * apk - s * aqk;
          a[q + n * k] = s * apk + c * aqk;
        }
        a[p + n * q] = 0.0;
        a[q + n * p] = 0.0;
        for (int k = 0; k < n; ++k) {
          double vkp = v[k + n * p], vkq = v[k + n * q];
          v[k + n * p] = c * vkp - s * vkq;
          v[k + n * q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = a[i + n * i];
}

__device__ inline void dev_expm(int n, cplx* mat) {
  if (n == 1) {
    mat[0] = cexp_(mat[0]);
    return;
  }
  double dh = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) dh = fmax(dh, cabsd(csub(mat[i + n * j], cconj(mat[j + n * i]))));
  bool herm = dh < 1e-7;
  const int m = 2 * n;
  double s[64], v[64], w[8];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      cplx z = herm ? mat[i + n * j] : cmul(mk(0.0, 1.0), mat[i + n * j]);
      s[i + m * j] = z.x;
      s[(i + n) + m * (j + n)] = z.x;
      s[i + m * (j + n)] = -z.y;
      s[(i + n) + m * j] = z.y;
    }
  dev_sym_jacobi(m, s, w, v);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a1 = 0.0, b1 = 0.0, a2 = 0.0, b2 = 0.0;
      for (int k = 0; k < m; ++k) {
        double f1 = herm ? exp(w[k]) : cos(w[k]);
        double f2 = herm ? 0.0 : sin(w[k]);
        a1 += v[i + m * k] * f1 * v[j + m * k];
        b1 += v[(i + n) + m * k] * f1 * v[j + m * k];
        a2 += v[i + m * k] * f2 * v[j + m * k];
        b2 += v[(i + n) + m * k] * f2 * v[j + m * k];
      }
      mat[i + n * j] = herm ? mk(a1, b1) : mk(a1 + b2, b1 - a2);
    }
}

// get_expKV(out, ppf, pla, bf_value, inv): out is dim x dim, ld = dim.
__device__ inline void dev_get_expkv(const DevModel& M, int pf, int pla, double bf, bool inv, cplx* out) {
  const int dim = M.pf_dim[pf], pd = M.pdim;
  const cplx* K = M.kmat + (size_t)pd * pd * pf;
  const cplx* V = M.vmat + (size_t)pd * pd * pf;
  const cplx* BC = M.bcp + (size_t)pd * pd * (pla + (size_t)M.max_pla * pf);
  const bool cross = M.cross[pla + M.max_pla * pf] != 0;
  const cplx kc = M.k_coe[pf], vc = M.v_coe[pf];
  for (int k = 0; k < dim * dim; ++k) out[k] = mk(0.0);
  if (M.expkv_kind == PQMC_EXPKV_EPSOCZ || M.expkv_kind == PQMC_EXPKV_EPSOCZ_BLOCK) {
    // get_expKV_epsocz (src/mod_phonon_field.f90:534-569)
    cplx sub[4];
    const cplx vx = cscale(vc, bf);
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        cplx h = cadd(cmul(kc, K[i + pd * (j + 2)]), cmul(vx, V[i + pd * (j + 2)]));
        sub[i + 2 * j] = cscale(h, -M.delt);
        if (cross) sub[i + 2 * j] = cmul(sub[i + 2 * j], BC[i + pd * (j + 2)]);
      }
    double norm;
    if (M.expkv_kind == PQMC_EXPKV_EPSOCZ) {
      double a = cabsd(kc), b = cabsd(vc) * bf;
      norm = M.delt * sqrt(a * a + b * b);
    } else {
      cplx h11 = cadd(cmul(kc, K[0 + pd * 2]), cmul(vx, V[0 + pd * 2]));
      cplx h21 = cadd(cmul(kc, K[1 + pd * 2]), cmul(vx, V[1 + pd * 2]));
      double a = cabsd(h11), b = cabsd(h21);
      norm = M.delt * sqrt(a * a + b * b);
    }
    const double ch = cosh(norm), sh = sinh(norm);
    for (int i = 0; i < dim; ++i) out[i + dim * i] = mk(ch);
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        cplx s = inv ? cneg(sub[i + 2 * j]) : sub[i + 2 * j];
        cplx t = cscale(s, sh);
        out[i + dim * (j + 2)] = mk(t.x / norm, t.y / norm);
      }
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) out[(i + 2) + dim * j] = cconj(out[j + dim * (i + 2)]);
    return;
  }
  if (M.expkv_kind == PQMC_EXPKV_EPSOC) {
    // get_expKV_epsoc (src/mod_phonon_field.f90:572-604)
    double a = cabsd(kc), b = cabsd(vc) * bf;
    double norm = M.delt * sqrt(a * a + b * b);
    const double ch = cosh(norm), sh = sinh(norm);
    for (int i = 0; i < dim; ++i) out[i + dim * i] = mk(ch);
    cplx h = cadd(cmul(kc, K[0 + pd * 1]), cmul(cscale(vc, bf), V[0 + pd * 1]));
    cplx sub = cscale(h, -M.delt);
    if (cross) sub = cmul(sub, BC[0 + pd * 1]);
    cplx s = inv ? cneg(sub) : sub;
    cplx t = cscale(s, sh);
    out[0 + dim * 1] = mk(t.x / norm, t.y / norm);
    out[1 + dim * 0] = cconj(out[0 + dim * 1]);
    return;
  }
  // get_expKV_general (src/mod_phonon_field.f90:497-532)
  const bool ke = M.pf_k_exist[pf] != 0, ve = M.pf_v_exist[pf] != 0;
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) {
      cplx h = mk(0.0);
      if (ve && ke) h = cadd(cmul(kc, K[i + pd * j]), cmul(cscale(vc, bf), V[i + pd * j]));
      else if (ve) h = cmul(cscale(vc, bf), V[i + pd * j]);
      else if (ke) h = cmul(kc, K[i + pd * j]);
      if (cross) h = cmul(h, BC[i + pd * j]);
      out[i + dim * j] = cscale(h, inv ? M.delt : -M.delt);
    }
  dev_expm(dim, out);
}

// analytic determinants of zdet (src/mod_matrixlib.f90:515-590)
__device__ inline cplx dev_det_small(int n, const cplx* a) {
#define A(i, j) a[((i)-1) + n * ((j)-1)]
  if (n == 1) return A(1, 1);
  if (n == 2) return csub(cmul(A(1, 1), A(2, 2)), cmul(A(1, 2), A(2, 1)));
  if (n == 3)
    return cadd(csub(cmul(A(1, 1), csub(cmul(A(2, 2), A(3, 3)), cmul(A(2, 3), A(3, 2)))),
                     cmul(A(1, 2), csub(cmul(A(2, 1), A(3, 3)), cmul(A(2, 3), A(3, 1))))),
                cmul(A(1, 3), csub(cmul(A(2, 1), A(3, 2)), cmul(A(2, 2), A(3, 1)))));
  cplx m1 = cadd(csub(cmul(A(2, 2), csub(cmul(A(3, 3), A(4, 4)), cmul(A(3, 4), A(4, 3)))),
                      cmul(A(2, 3), csub(cmul(A(3, 2), A(4, 4)), cmul(A(3, 4), A(4, 2))))),
                 cmul(A(2, 4), csub(cmul(A(3, 2), A(4, 3)), cmul(A(3, 3), A(4, 2)))));
  cplx m2 = cadd(csub(cmul(A(2, 1), csub(cmul(A(3, 3), A(4, 4)), cmul(A(3, 4), A(4, 3)))),
                      cmul(A(2, 3), csub(cmul(A(3, 1), A(4, 4)), cmul(A(3, 4), A(4, 1))))),
                 cmul(A(2, 4), csub(cmul(A(3, 1), A(4, 3)), cmul(A(3, 3), A(4, 1)))));
  cplx m3 = cadd(csub(cmul(A(2, 1), csub(cmul(A(3, 2), A(4, 4)), cmul(A(3, 4), A(4, 2)))),
                      cmul(A(2, 2), csub(cmul(A(3, 1), A(4, 4)), cmul(A(3, 4), A(4, 1))))),
                 cmul(A(2, 4), csub(cmul(A(3, 1), A(4, 2)), cmul(A(3, 2), A(4, 1)))));
  cplx m4 = cadd(csub(cmul(A(2, 1), csub(cmul(A(3, 2), A(4, 3)), cmul(A(3, 3), A(4, 2)))),
                      cmul(A(2, 2), csub(cmul(A(3, 1), A(4, 3)), cmul(A(3, 3), A(4, 1))))),
                 cmul(A(2, 3), csub(cmul(A(3, 1), A(4, 2)), cmul(A(3, 2), A(4, 1)))));
  cplx res = cmul(A(1, 1), m1);
  res = csub(res, cmul(A(1, 2), m2));
  res = cadd(res, cmul(A(1, 3), m3));
  res = csub(res, cmul(A(1, 4), m4));
  return res;
#undef A
}

// small dense inverse by Gauss-Jordan with partial pivoting (|re|+|im|);
// zinverse for dim <= 4 (src/mod_matrixlib.f90:410-431).  Returns false on
// an exactly singular matrix.
__device__ inline bool dev_inverse_small(int n, cplx* a) {
  cplx b[16];
  int piv[4];
  for (int k = 0; k < n * n; ++k) b[k] = a[k];
  for (int i = 0; i < n; ++i) piv[i] = i;
  cplx inv[16];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) inv[i + n * j] = mk(i == j ? 1.0 : 0.0);
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double best = -1.0;
    for (int i = j; i < n; ++i) {
      double v = fabs(b[i + n * j].x) + fabs(b[i + n * j].y);
      if (v > best) { best = v; jp = i; }
    }
    if (best == 0.0) return false;
    if (jp != j)
      for (int k = 0; k < n; ++k) {
        cplx t = b[j + n * k]; b[j + n * k] = b[jp + n * k]; b[jp + n * k] = t;
        t = inv[j + n * k]; inv[j + n * k] = inv[jp + n * k]; inv[jp + n * k] = t;
      }
    cplx r = cdiv(mk(1.0), b[j + n * j]);
    for (int k = 0; k < n; ++k) { b[j + n * k] = cmul(b[j + n * k], r); inv[j + n * k] = cmul(inv[j + n * k], r); }
    for (int i = 0; i < n; ++i) {
      if (i == j) continue;
      cplx f = b[i + n * j];
      for (int k = 0; k < n; ++k) {
        b[i + n * k] = csub(b[i + n * k], cmul(f, b[j + n * k]));
        inv[i + n * k] = csub(inv[i + n * k], cmul(f, inv[j + n * k]));
      }
    }
  }
  (void)piv;
  for (int k = 0; k < n * n; ++k) a[k] = inv[k];
  return true;
}
