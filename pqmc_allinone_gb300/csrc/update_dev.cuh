// update_dev.cuh -- device helpers of the local update shared by the
// single-chain (update.cu) and batched (batch.cu) kernels.
#pragma once
#include "chain.cuh"
#include "expkv.cuh"

namespace pqmc {

__device__ __forceinline__ cplx ldg_c(const cplx* p) { return __ldcg(p); }
__device__ __forceinline__ cplx shfl_c(cplx v, int src) {
  return mk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__device__ __forceinline__ double energy_diff(const DevModel& M, const double* field, int b, int t, double jump) {
  // cal_energy_difference (src/mod_update.f90:203-228), t 0-based, periodic in time
  const int nt = M.ntime;
  double be = field[b + (size_t)M.n_bf * ((t - 1 + nt) % nt)];
  double af = field[b + (size_t)M.n_bf * ((t + 1) % nt)];
  double now = field[b + (size_t)M.n_bf * t];
  double nw = now + jump;
  double dt2 = M.delt * M.delt;
  double e1 = ((0.5 * M.mass) * ((be - now) * (be - now) + (af - now) * (af - now))) / dt2 +
              (0.5 * M.stiff) * (now * now) - M.biased * now;
  double e2 = ((0.5 * M.mass) * ((be - nw) * (be - nw) + (af - nw) * (af - nw))) / dt2 +
              (0.5 * M.stiff) * (nw * nw) - M.biased * nw;
  return e2 - e1;
}

// Entry (i,j) of the closed-form propagators (get_expKV_epsocz / _epsoc,
// src/mod_phonon_field.f90:534-604) given norm, cosh(norm), sinh(norm).
__device__ __forceinline__ cplx closed_entry(const DevModel& M, int pf, int pla, double x, bool inv, int i, int j,
                                             double norm, double ch, double sh) {
  const int pd = M.pdim, dim = M.pf_dim[pf];
  if (i == j) return mk(ch);
  const cplx* K = M.kmat + (size_t)pd * pd * pf;
  const cplx* V = M.vmat + (size_t)pd * pd * pf;
  const cplx* BC = M.bcp + (size_t)pd * pd * (pla + (size_t)M.max_pla * pf);
  const bool cross = M.cross[pla + M.max_pla * pf] != 0;
  const cplx kc = M.k_coe[pf], vx = cscale(M.v_coe[pf], x);
  const int h = dim / 2;  // off-diagonal block offset (2 for epsocz, 1 for epsoc)
  bool upper = (i < h && j >= h), lower = (i >= h && j < h);
  if (!upper && !lower) return mk(0.0);
  int a = upper ? i : j, b = upper ? j : i;   // entry (a,b) of the upper block
  if (M.expkv_kind == PQMC_EXPKV_EPSOC && !(a == 0 && b == 1)) return mk(0.0);
  cplx hab = cadd(cmul(kc, K[a + pd * b]), cmul(vx, V[a + pd * b]));
  cplx sub = cscale(hab, -M.delt);
  if (cross) sub = cmul(sub, BC[a + pd * b]);
  cplx s = inv ? cneg(sub) : sub;
  cplx t = cscale(s, sh);
  cplx e = mk(t.x / norm, t.y / norm);
  return upper ? e : cconj(e);
}

__device__ __forceinline__ double closed_norm(const DevModel& M, int pf, double x) {
  const int pd = M.pdim;
  const cplx kc = M.k_coe[pf], vc = M.v_coe[pf];
  if (M.expkv_kind == PQMC_EXPKV_EPSOCZ_BLOCK) {
    const cplx* K = M.kmat + (size_t)pd * pd * pf;
    const cplx* V = M.vmat + (size_t)pd * pd * pf;
    const cplx vx = cscale(vc, x);
    cplx h11 = cadd(cmul(kc, K[0 + pd * 2]), cmul(vx, V[0 + pd * 2]));
    cplx h21 = cadd(cmul(kc, K[1 + pd * 2]), cmul(vx, V[1 + pd * 2]));
    double a = cabsd(h11), b = cabsd(h21);
    return M.delt * sqrt(a * a + b * b);
  }
  double a = cabsd(kc), b = cabsd(vc) * x;
  return M.delt * sqrt(a * a + b * b);
}

// 4x4 determinant by Laplace expansion along rows 1,2 over six lanes;
// the sum is returned to every lane.  Smaller sizes: the reference's
// analytic forms on lane 0 (zdet, src/mod_matrixlib.f90:515-590).
__device__ inline cplx warp_det(int dim, const cplx* R, int lane) {
  cplx v = mk(0.0);
  if (dim == 4) {
    // column pairs (j,k) of rows 0,1 and the complementary pair (l,m) of rows 2,3
    const int J[6] = {0, 0, 0, 1, 1, 2}, K[6] = {1, 2, 3, 2, 3, 3};
    const int L[6] = {2, 1, 1, 0, 0, 0}, Mm[6] = {3, 3, 2, 3, 2, 1};
    const double sg[6] = {1.0, -1.0, 1.0, 1.0, -1.0, 1.0};
    if (lane < 6) {
      int j = J[lane], k = K[lane], l = L[lane], m = Mm[lane];
      cplx mi = csub(cmul(R[0 + 4 * j], R[1 + 4 * k]), cmul(R[0 + 4 * k], R[1 + 4 * j]));
      cplx co = csub(cmul(R[2 + 4 * l], R[3 + 4 * m]), cmul(R[2 + 4 * m], R[3 + 4 * l]));
      v = cscale(cmul(mi, co), sg[lane]);
    }
    for (int o = 4; o > 0; o >>= 1) {
      cplx w = mk(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
      if (lane + o < 8) v = cadd(v, w);
    }
    return shfl_c(v, 0);
  }
  if (lane == 0) v = dev_det_small(dim, R);
  return shfl_c(v, 0);
}

// inverse of a small matrix on the warp: adjugate over 16 lanes for dim 4,
// lane-0 Gauss-Jordan otherwise (zinverse, src/mod_matrixlib.f90:410-431).
// R (dim x dim) in shared memory is replaced by its inverse.
__device__ inline void warp_inverse(int dim, cplx* R, cplx det, int lane) {
  if (dim == 4) {
    cplx cof = mk(0.0);
    int i = lane & 3, j = lane >> 2;  // cofactor of entry (i,j)
    if (lane < 16) {
      int r[3], c[3], n = 0;
      for (int k = 0; k < 4; ++k)
        if (k != i) r[n++] = k;
      n = 0;
      for (int k = 0; k < 4; ++k)
        if (k != j) c[n++] = k;
#define S(a, b) R[r[a] + 4 * c[b]]
      cof = cadd(csub(cmul(S(0, 0), csub(cmul(S(1, 1), S(2, 2)), cmul(S(1, 2), S(2, 1)))),
                      cmul(S(0, 1), csub(cmul(S(1, 0), S(2, 2)), cmul(S(1, 2), S(2, 0))))),
                 cmul(S(0, 2), csub(cmul(S(1, 0), S(2, 1)), cmul(S(1, 1), S(2, 0)))));
#undef S
      if ((i + j) & 1) cof = cneg(cof);
      cof = cdiv(cof, det);
    }
    __syncwarp();
    if (lane < 16) R[j + 4 * i] = cof;  // inverse = adj / det, adj(j,i) = cof(i,j)
    __syncwarp();
    return;
  }
  if (lane == 0) dev_inverse_small(dim, R);
  __syncwarp();
}


}  // namespace pqmc
