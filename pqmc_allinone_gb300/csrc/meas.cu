// meas.cu -- equal-time measurement (ms_take_measurement,
// src/mod_meas.f90:210-544; helpers :64-208; k-space :546-566; window
// averaging :729-763) and the fused sweep driver (src/Main_PQMC.f90:81-156).
//
// One CTA per relative displacement `ind`; its threads cover the cells c1,
// each evaluating every Wick contraction of the pair (c1, c2) with
// rel(c1,c2) = ind, then a fixed-order tree reduction per observable.  The
// per-cell phonon scalars are a separate single-thread pass in cell order.
#include <string.h>
#include <vector>
#include "chain.cuh"
#include "linalg.cuh"

namespace pqmc {

struct MeasView {
  int ns, nc;
  const cplx* gh;
  const int* sites;   // (2,nc)
  const int* bfi;     // (2,nc)
  const int* xnb;
  const int* ynb;
  const int* cross;   // (2,nc)
  const int* c2_of;   // (nc,nc): c2_of[c1 + nc*ind]
  const double* field;
  int t, n_bf;
  cplx bc[2];
  double hop, ep;
};

__device__ __forceinline__ cplx GH(const MeasView& V, int i, int j) { return V.gh[i + (size_t)V.ns * j]; }
__device__ __forceinline__ cplx GG(const MeasView& V, int i, int j) {
  cplx v = cneg(V.gh[i + (size_t)V.ns * j]);
  if (i == j) v = cadd(v, mk(1.0));
  return v;
}

// cal_wick_contraction (:165-183): mat(i,j) = gh(l2,l1) gh(r2,r1) [+ gh(r2,l1) g(l2,r1)]
template <int N>
__device__ inline void wick(const MeasView& V, const int (*ls)[2], const int (*rs)[2], bool hartree, cplx* mat) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      cplx m = mk(0.0);
      m = cfma(GH(V, ls[i][1], ls[i][0]), GH(V, rs[j][1], rs[j][0]), m);
      if (!hartree) m = cfma(GH(V, rs[j][1], ls[i][0]), GG(V, ls[i][1], rs[j][0]), m);
      mat[i + N * j] = m;
    }
}

__device__ inline void spin_current(const MeasView& V, int p1, int p2, int p3, int p4, bool h, cplx* mat) {
  auto s = [&](int c, int k) { return V.sites[k + 2 * c]; };
  int ls[4][2] = {{s(p1, 0), s(p2, 1)}, {s(p1, 1), s(p2, 0)}, {s(p2, 0), s(p1, 1)}, {s(p2, 1), s(p1, 0)}};
  int rs[4][2] = {{s(p3, 0), s(p4, 1)}, {s(p3, 1), s(p4, 0)}, {s(p4, 0), s(p3, 1)}, {s(p4, 1), s(p3, 0)}};
  wick<4>(V, ls, rs, h, mat);
}

__device__ inline void spin_momentum(const MeasView& V, int p1, int p2, cplx* mat) {
  auto s = [&](int c, int k) { return V.sites[k + 2 * c]; };
  int ls[4][2] = {{s(p1, 0), s(p1, 0)}, {s(p1, 0), s(p1, 1)}, {s(p1, 1), s(p1, 0)}, {s(p1, 1), s(p1, 1)}};
  int rs[4][2] = {{s(p2, 0), s(p2, 0)}, {s(p2, 0), s(p2, 1)}, {s(p2, 1), s(p2, 0)}, {s(p2, 1), s(p2, 1)}};
  wick<4>(V, ls, rs, false, mat);
}

__device__ inline void phys_current(const MeasView& V, int p1, int p2, int p3, int p4, cplx* mat) {
  auto s = [&](int c, int k) { return V.sites[k + 2 * c]; };
  int ls[8][2] = {{s(p1, 0), s(p2, 1)}, {s(p1, 1), s(p2, 0)}, {s(p2, 0), s(p1, 1)}, {s(p2, 1), s(p1, 0)},
                  {s(p1, 0), s(p2, 0)}, {s(p1, 1), s(p2, 1)}, {s(p2, 0), s(p1, 0)}, {s(p2, 1), s(p1, 1)}};
  int rs[8][2] = {{s(p3, 0), s(p4, 1)}, {s(p3, 1), s(p4, 0)}, {s(p4, 0), s(p3, 1)}, {s(p4, 1), s(p3, 0)},
                  {s(p3, 0), s(p4, 0)}, {s(p3, 1), s(p4, 1)}, {s(p4, 0), s(p3, 0)}, {s(p4, 1), s(p3, 1)}};
  wick<8>(V, ls, rs, false, mat);
}

__device__ __forceinline__ void bphase(const MeasView& V, cplx* v, bool cross, int dir) {
  // add_boundary_phase (:199-208)
  if (!cross) return;
  cplx bc = V.bc[dir];
  v[0] = cmul(v[0], bc); v[1] = cmul(v[1], bc); v[2] = cmul(v[2], cconj(bc)); v[3] = cmul(v[3], cconj(bc));
}

template <int N>
__device__ __forceinline__ cplx contract(const cplx* vl, const cplx* m, const cplx* vr) {
  cplx tot = mk(0.0);
  for (int i = 0; i < N; ++i) {
    cplx w = mk(0.0);
    for (int j = 0; j < N; ++j) w = cfma(m[i + N * j], vr[j], w);
    tot = cfma(vl[i], w, tot);
  }
  return tot;
}

// all field observables of one cell pair, already divided by N_cell
__device__ void pair_obs(const MeasView& V, int c1, int c2, cplx* F) {
  const double N = (double)V.nc;
  const int t = V.t;
  auto X = [&](int b) { return V.field[b + (size_t)V.n_bf * t]; };
  const int c1x = V.xnb[c1], c1y = V.ynb[c1], c2x = V.xnb[c2], c2y = V.ynb[c2];
  const bool cr1[2] = {V.cross[2 * c1] != 0, V.cross[2 * c1 + 1] != 0};
  const bool cr2[2] = {V.cross[2 * c2] != 0, V.cross[2 * c2 + 1] != 0};
  const double x1x = X(V.bfi[2 * c1]), x1y = X(V.bfi[2 * c1 + 1]);
  const double x2x = X(V.bfi[2 * c2]), x2y = X(V.bfi[2 * c2 + 1]);
  F[PQMC_F_BFX_BFX] = mk((x1x * x2x) / N);
  F[PQMC_F_BFX_BFY] = mk((x1x * x2y) / N);
  F[PQMC_F_BFY_BFY] = mk((x1y * x2y) / N);
  F[PQMC_F_BFXY_BFXY] = mk((x1x * x1y * x2x * x2y) / N);
  const cplx vx[4] = {mk(-0.0, V.hop), mk(-0.0, V.hop), mk(0.0, -V.hop), mk(0.0, -V.hop)};
  const cplx vy[4] = {mk(V.hop), mk(-V.hop), mk(-V.hop), mk(V.hop)};
  cplx m[64], vl[8], vr[8];
  auto cur = [&](int f, const cplx* lv, int ld, const cplx* rv, int rd, bool quirk) {
    for (int k = 0; k < 4; ++k) { vl[k] = lv[k]; vr[k] = rv[k]; }
    bphase(V, vl, cr1[ld], ld);
    bphase(V, vr, cr2[rd], rd);
    cplx r = contract<4>(vl, m, quirk ? vl : vr);
    F[f] = mk(r.x / N, r.y / N);
  };
  spin_current(V, c1, c1x, c2, c2x, false, m);
  cur(PQMC_F_JXX_JXX, vx, 0, vx, 0, false);
  cur(PQMC_F_JXY_JXY, vy, 0, vy, 0, false);
  spin_current(V, c1, c1y, c2, c2y, false, m);
  cur(PQMC_F_JYX_JYX, vx, 1, vx, 1, false);
  cur(PQMC_F_JYY_JYY, vy, 1, vy, 1, true);     // :353 contracts with vec_l twice
  spin_current(V, c1, c1x, c2, c2y, false, m);
  cur(PQMC_F_JXX_JYX, vx, 0, vx, 1, false);
  cur(PQMC_F_JXY_JYY, vy, 0, vy, 1, false);
  spin_current(V, c1, c1x, c2, c2x, true, m);
  cur(PQMC_F_JXXH_JXXH, vx, 0, vx, 0, false);
  cur(PQMC_F_JXYH_JXYH, vy, 0, vy, 0, false);
  spin_current(V, c1, c1y, c2, c2y, true, m);
  cur(PQMC_F_JYXH_JYXH, vx, 1, vx, 1, false);
  cur(PQMC_F_JYYH_JYYH, vy, 1, vy, 1, true);   // :417
  spin_current(V, c1, c1x, c2, c2y, true, m);
  cur(PQMC_F_JXXH_JYXH, vx, 0, vx, 1, false);
  cur(PQMC_F_JXYH_JYYH, vy, 0, vy, 1, false);
  cur(PQMC_F_JXXH_JYYH, vx, 0, vy, 1, false);
  cur(PQMC_F_JXYH_JYXH, vy, 0, vx, 1, false);
  spin_momentum(V, c1, c2, m);
  {
    const cplx dn[4] = {mk(0.5), mk(0), mk(0), mk(0.5)};
    const cplx sz[4] = {mk(0.5), mk(0), mk(0), mk(-0.5)};
    const cplx sx[4] = {mk(0), mk(0.5), mk(0.5), mk(0)};
    const cplx sy[4] = {mk(0), mk(-0.0, -0.5), mk(0.0, 0.5), mk(0)};
    cplx r = contract<4>(dn, m, dn);
    F[PQMC_F_DEN_DEN] = mk(r.x / N, r.y / N);
    int s1u = V.sites[2 * c1], s1d = V.sites[2 * c1 + 1], s2u = V.sites[2 * c2], s2d = V.sites[2 * c2 + 1];
    cplx sc = csub(cmul(GH(V, s2u, s1u), GH(V, s2d, s1d)), cmul(GH(V, s2d, s1u), GH(V, s2u, s1d)));
    F[PQMC_F_SC_SC] = mk(sc.x / N, sc.y / N);
    r = contract<4>(sz, m, sz);
    F[PQMC_F_SZ_SZ] = mk(r.x / N, r.y / N);
    r = contract<4>(sx, m, sx);
    F[PQMC_F_SX_SX] = mk(r.x / N, r.y / N);
    r = contract<4>(sy, m, sy);
    F[PQMC_F_SY_SY] = mk(r.x / N, r.y / N);
  }
  auto phys = [&](int f, const cplx* cv, double xl, double xr, int dir) {
    for (int k = 0; k < 4; ++k) vl[k] = cneg(cv[k]);
    for (int k = 0; k < 4; ++k) vl[4 + k] = mk(V.ep * xl * 1.0);
    for (int k = 0; k < 4; ++k) vr[k] = vl[k];
    for (int k = 0; k < 4; ++k) vr[4 + k] = mk(V.ep * xr * 1.0);
    bphase(V, vl, cr1[dir], dir);
    bphase(V, vr, cr2[dir], dir);
    bphase(V, vl + 4, cr1[dir], dir);
    bphase(V, vr + 4, cr2[dir], dir);
    cplx r = contract<8>(vl, m, vr);
    F[f] = mk(r.x / N, r.y / N);
  };
  phys_current(V, c1, c1y, c2, c2y, m);
  phys(PQMC_F_CJYX_CJYX, vx, x1y, x2y, 1);
  phys_current(V, c1, c1x, c2, c2x, m);
  phys(PQMC_F_CJXY_CJXY, vy, x1x, x2x, 0);
}

constexpr int MEAS_THREADS = 128;

__global__ void __launch_bounds__(MEAS_THREADS) k_meas_pairs(MeasView V, cplx* acc) {
  __shared__ double red[MEAS_THREADS];
  const int ind = blockIdx.x;
  cplx part[PQMC_N_FIELD];
  for (int f = 0; f < PQMC_N_FIELD; ++f) part[f] = mk(0.0);
  cplx F[PQMC_N_FIELD];
  for (int c1 = threadIdx.x; c1 < V.nc; c1 += blockDim.x) {
    int c2 = V.c2_of[c1 + (size_t)V.nc * ind];
    pair_obs(V, c1, c2, F);
    for (int f = 0; f < PQMC_N_FIELD; ++f) part[f] = cadd(part[f], F[f]);
  }
  for (int f = 0; f < PQMC_N_FIELD; ++f) {
    for (int comp = 0; comp < 2; ++comp) {
      red[threadIdx.x] = comp ? part[f].y : part[f].x;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        cplx* dst = acc + PQMC_N_SCALAR + (size_t)f * V.nc + ind;
        if (comp) dst->y += red[0];
        else dst->x += red[0];
      }
      __syncthreads();
    }
  }
}

// BF_KE, BF_PE, BF_X per cell in cell order (:249-268)
__global__ void k_meas_scalars(MeasView V, double D, double M, double biased, double delt, cplx* acc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double N = (double)V.nc;
  const int t = V.t;
  for (int c1 = 0; c1 < V.nc; ++c1) {
    int bx = V.bfi[2 * c1], by = V.bfi[2 * c1 + 1];
    double x1x = V.field[bx + (size_t)V.n_bf * t], x1y = V.field[by + (size_t)V.n_bf * t];
    double o = (0.5 * D) * (x1x * x1x + x1y * x1y) - biased * (x1x + x1y);
    acc[PQMC_OBS_BF_KE] = cadd(acc[PQMC_OBS_BF_KE], mk(o / N));
    double d1 = x1x - V.field[bx + (size_t)V.n_bf * (t + 1)], d2 = x1y - V.field[by + (size_t)V.n_bf * (t + 1)];
    double q = 0.0 - ((0.5 * M) * (d1 * d1 + d2 * d2)) / (delt * delt);
    q = q + (1.0 / (2.0 * delt)) * 2.0;
    acc[PQMC_OBS_BF_PE] = cadd(acc[PQMC_OBS_BF_PE], mk(q / N));
    acc[PQMC_OBS_BF_X] = cadd(acc[PQMC_OBS_BF_X], mk((x1x + x1y) / N));
  }
}

// window average + ms_k_space_obs
__global__ void k_meas_finish(int nc, double div, const cplx* __restrict__ kphase, cplx* acc) {
  // divide r-space part (block 0 does it first, others wait through a second launch)
  const int f = blockIdx.x, ik = threadIdx.x + blockIdx.y * blockDim.x;
  if (ik >= nc) return;
  const cplx* r = acc + PQMC_N_SCALAR + (size_t)f * nc;
  cplx s = mk(0.0);
  for (int i = 0; i < nc; ++i) {
    cplx rv = r[i];
    rv = mk(rv.x / div, rv.y / div);
    s = cfma(kphase[ik + (size_t)nc * i], rv, s);
  }
  cplx* kd = acc + PQMC_N_SCALAR + (size_t)(PQMC_N_FIELD + f) * nc;
  kd[ik] = cadd(kd[ik], mk(s.x / (double)nc, s.y / (double)nc));
}

__global__ void k_meas_divide(int n, double div, cplx* acc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc[i] = mk(acc[i].x / div, acc[i].y / div);
}

static MeasView view(pqmc_chain* c, int time) {
  MeasView V;
  V.ns = c->ns;
  V.nc = c->n_cell;
  V.gh = c->g;
  V.sites = c->m_cell_sites;
  V.bfi = c->m_cell_bf;
  V.xnb = c->m_cell_xnb;
  V.ynb = c->m_cell_ynb;
  V.cross = c->m_cell_cross;
  V.c2_of = c->m_c2_of;
  V.field = c->field;
  V.t = time - 1;
  V.n_bf = c->n_bf;
  V.bc[0] = c->h_bc[0];
  V.bc[1] = c->h_bc[1];
  V.hop = c->hop;
  V.ep = c->ep;
  return V;
}

int do_measure(pqmc_chain* c, int time) {
  MeasView V = view(c, time);
  k_meas_scalars<<<1, 1, 0, c->stream>>>(V, c->M.stiff, c->M.mass, c->M.biased, c->M.delt, c->m_acc);
  PQMC_LAUNCHED();
  k_meas_pairs<<<c->n_cell, MEAS_THREADS, 0, c->stream>>>(V, c->m_acc);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

int do_finish_record(pqmc_chain* c, int meas_number) {
  const int nc = c->n_cell;
  double div = (double)(2 * meas_number + 1);
  dim3 g(PQMC_N_FIELD, (nc + 127) / 128);
  k_meas_finish<<<g, 128, 0, c->stream>>>(nc, div, c->m_kphase, c->m_acc);
  PQMC_LAUNCHED();
  k_meas_divide<<<8, 256, 0, c->stream>>>(PQMC_N_SCALAR + PQMC_N_FIELD * nc, div, c->m_acc);
  PQMC_LAUNCHED();
  return PQMC_OK;
}

static int record_width(const pqmc_chain* c) { return PQMC_N_SCALAR + 2 * PQMC_N_FIELD * c->n_cell; }

// the slice loop of Main_PQMC.f90:99-154 for one value of `loop`
static int sweep_one(pqmc_chain* c, int loop, int warmup, int meas_interval, int meas_number, double* records,
                     int cap, int* nrec, int tc_first = 1, int tc_last = 0) {
  const bool forward = (loop % 2) == 0;   // the first loop (loop=1) runs backward (:85)
  const int half = c->ntime / 2;
  const int W = record_width(c);
  if (tc_last <= 0) tc_last = c->ntime;
  for (int tc = tc_first; tc <= tc_last; ++tc) {
    int time;
    if (!forward) {
      time = c->ntime - tc + 1;
      for (int pf = c->n_pf - 1; pf >= 0; --pf) {
        PQMC_TRY(launch_wrap(c, pf, time, false));
        if (c->M.local_update && c->h_pf_v_exist[pf]) PQMC_TRY(launch_update(c, pf, time));
      }
    } else {
      time = tc;
      for (int pf = 0; pf < c->n_pf; ++pf) {
        if (c->M.local_update && c->h_pf_v_exist[pf]) PQMC_TRY(launch_update(c, pf, time));
        PQMC_TRY(launch_wrap(c, pf, time, true));
      }
    }
    if (tc % c->ngroup == 0) PQMC_TRY(do_g_scratch(c, forward ? time + 1 : time, forward, loop));
    if (c->have_meas && loop > warmup && ((loop - warmup) % meas_interval) == 0 && time >= half - meas_number &&
        time <= half + meas_number) {
      PQMC_TRY(do_measure(c, time));
      bool last = (forward && time == half + meas_number) || (!forward && time == half - meas_number);
      if (last) {
        PQMC_TRY(do_finish_record(c, meas_number));
        if (records && *nrec < cap)
          PQMC_CUDA(cudaMemcpyAsync(records + (size_t)2 * W * (*nrec), c->m_acc, sizeof(cplx) * W,
                                    cudaMemcpyDeviceToHost, c->stream));
        PQMC_CUDA(cudaMemsetAsync(c->m_acc, 0, sizeof(cplx) * W, c->stream));
        (*nrec)++;
      }
    }
  }
  return PQMC_OK;
}

}  // namespace pqmc

using namespace pqmc;

extern "C" {

int pqmc_set_meas_layout(pqmc_chain* c, const pqmc_meas_layout* L) {
  if (!c || !L) { set_error("null argument"); return PQMC_ERR_ARG; }
  const int nc = L->n_cell;
  for (int k = 0; k < 2 * nc; ++k)
    if (L->cell_sites[k] < 0 || L->cell_sites[k] >= c->ns || L->cell_bf[k] < 0 || L->cell_bf[k] >= c->n_bf) {
      set_error("meas layout: site/boson index out of range");
      return PQMC_ERR_ARG;
    }
  std::vector<int> c2of((size_t)nc * nc, -1);
  for (int c1 = 0; c1 < nc; ++c1)
    for (int c2 = 0; c2 < nc; ++c2) {
      int ind = L->rel_index[c1 + (size_t)nc * c2];
      if (ind < 0 || ind >= nc || c2of[c1 + (size_t)nc * ind] >= 0) {
        set_error("meas layout: relative index table is not a permutation per cell");
        return PQMC_ERR_ARG;
      }
      c2of[c1 + (size_t)nc * ind] = c2;
    }
  auto up = [&](int** d, const int32_t* h, size_t n) -> int {
    if (*d) cudaFree(*d);
    PQMC_CUDA(cudaMalloc((void**)d, sizeof(int) * n));
    PQMC_CUDA(cudaMemcpy(*d, h, sizeof(int) * n, cudaMemcpyHostToDevice));
    return PQMC_OK;
  };
  PQMC_TRY(up(&c->m_cell_sites, L->cell_sites, 2 * nc));
  PQMC_TRY(up(&c->m_cell_bf, L->cell_bf, 2 * nc));
  PQMC_TRY(up(&c->m_cell_xnb, L->cell_xnb, nc));
  PQMC_TRY(up(&c->m_cell_ynb, L->cell_ynb, nc));
  PQMC_TRY(up(&c->m_cell_cross, L->cell_cross, 2 * nc));
  PQMC_TRY(up(&c->m_c2_of, c2of.data(), (size_t)nc * nc));
  if (c->m_kphase) cudaFree(c->m_kphase);
  PQMC_CUDA(cudaMalloc((void**)&c->m_kphase, sizeof(cplx) * (size_t)nc * nc));
  PQMC_CUDA(cudaMemcpy(c->m_kphase, L->k_phase, sizeof(cplx) * (size_t)nc * nc, cudaMemcpyHostToDevice));
  c->n_cell = nc;
  const int W = record_width(c);
  if (c->m_acc) cudaFree(c->m_acc);
  PQMC_CUDA(cudaMalloc((void**)&c->m_acc, sizeof(cplx) * W));
  PQMC_CUDA(cudaMemset(c->m_acc, 0, sizeof(cplx) * W));
  c->h_bc[0] = mk(L->bc_phase[0], L->bc_phase[1]);
  c->h_bc[1] = mk(L->bc_phase[2], L->bc_phase[3]);
  c->hop = L->hop;
  c->ep = L->ep_parameter;
  c->have_meas = true;
  return PQMC_OK;
}

int pqmc_take_measurement(pqmc_chain* c, int time) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->have_meas) { set_error("no measurement layout"); return PQMC_ERR_STATE; }
  if (time < 1 || time >= c->ntime) { set_error("time out of range"); return PQMC_ERR_ARG; }
  PQMC_TRY(do_measure(c, time));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_begin_measure(pqmc_chain* c, int forward, int time, int meas_number, double* record_out, int* done) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->have_meas) { set_error("no measurement layout"); return PQMC_ERR_STATE; }
  if (time < 1 || time >= c->ntime) { set_error("time out of range"); return PQMC_ERR_ARG; }
  PQMC_TRY(do_measure(c, time));
  const int half = c->ntime / 2;
  bool last = (forward && time == half + meas_number) || (!forward && time == half - meas_number);
  if (done) *done = last ? 1 : 0;
  if (last) {
    PQMC_TRY(do_finish_record(c, meas_number));
    const int W = record_width(c);
    if (record_out)
      PQMC_CUDA(cudaMemcpyAsync(record_out, c->m_acc, sizeof(cplx) * W, cudaMemcpyDeviceToHost, c->stream));
    PQMC_CUDA(cudaMemsetAsync(c->m_acc, 0, sizeof(cplx) * W, c->stream));
  }
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_sweep(pqmc_chain* c, int first_loop, int n_sweeps, int warmup, int meas_interval, int meas_number,
               double* records, int n_records_cap, int* n_records) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->have_g) { set_error("sweep before init_g"); return PQMC_ERR_STATE; }
  if (n_sweeps < 0 || meas_interval < 1 || meas_number < 0) { set_error("bad sweep arguments"); return PQMC_ERR_ARG; }
  if (c->have_meas && (c->ntime / 2 - meas_number < 1 || c->ntime / 2 + meas_number > c->ntime - 1)) {
    set_error("measurement window ntime/2 +- %d leaves 1..ntime-1", meas_number);
    return PQMC_ERR_ARG;
  }
  int nrec = 0;
  for (int loop = first_loop; loop < first_loop + n_sweeps; ++loop) {
    // global step before the sweep (Main_PQMC.f90:87-96), once enabled
    if (c->have_global) PQMC_TRY(pqmc_global_step(c, loop, nullptr));
    PQMC_TRY(sweep_one(c, loop, warmup, meas_interval, meas_number, records, n_records_cap, &nrec));
  }
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  if (n_records) *n_records = nrec;
  return PQMC_OK;
}

int pqmc_sweep_slices(pqmc_chain* c, int loop, int first_tc, int n_slices) {
  if (!c) { set_error("null chain"); return PQMC_ERR_ARG; }
  if (!c->have_g) { set_error("sweep before init_g"); return PQMC_ERR_STATE; }
  if (first_tc < 1 || n_slices < 0 || first_tc + n_slices - 1 > c->ntime) {
    set_error("sweep_slices: slices %d..%d outside 1..%d", first_tc, first_tc + n_slices - 1, c->ntime);
    return PQMC_ERR_ARG;
  }
  if (n_slices == 0) return PQMC_OK;
  int nrec = 0;
  PQMC_TRY(sweep_one(c, loop, 1 << 30, 1, 0, nullptr, 0, &nrec, first_tc, first_tc + n_slices - 1));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

}  // extern "C"
