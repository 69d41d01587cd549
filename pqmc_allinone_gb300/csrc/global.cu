// global.cu -- global moves of the phonon field: update_global and
// generate_newfield_global (src/mod_update.f90:250-467) with the driver's
// global step (src/Main_PQMC.f90:87-96).
//
// A global move changes the field on whole time lines, so its weight needs
// the full log det of the new configuration (cal_new_weight_T0), which runs
// on the device (do_new_weight).  The field generation itself is O(n_bf *
// ntime) scalar work on a few ran2 draws per move, done here on the host
// from a host copy of the chain's ran2 state: the draws and their order
// follow the reference exactly, so the chain's random stream continues as
// it does there.
#include <cmath>
#include <vector>
#include "chain.cuh"

namespace pqmc {

// ran2_s (src/mod_ranstate.f90:171-191) on the host, the arithmetic of the
// device copy (rng.cuh) in plain IEEE single precision
struct Ran2Host {
  int32_t iran, jran, kran, mran, nran;
  explicit Ran2Host(const int32_t* w) : iran(w[0]), jran(w[1]), kran(w[2]), mran(w[3]), nran(w[4]) {}
  void store(int32_t* w) const {
    w[0] = iran; w[1] = jran; w[2] = kran; w[3] = mran; w[4] = nran;
  }
  float next() {
    int32_t rans = (int32_t)((uint32_t)iran - (uint32_t)kran);
    if (rans < 0) rans = (int32_t)((uint32_t)rans + 2147483579u);
    iran = jran;
    jran = kran;
    kran = rans;
    uint32_t n = (uint32_t)nran;
    n ^= n << 13;
    n ^= n >> 17;
    n ^= n << 5;
    nran = (int32_t)n;
    uint32_t m = (uint32_t)mran;
    const uint32_t lo = m & 65535u;
    m = ((3533u * (m >> 16) + lo) << 16) + 3533u * lo + 820265819u;
    mran = (int32_t)m;
    const int32_t r = (int32_t)(((uint32_t)nran ^ (uint32_t)kran) + (uint32_t)mran);
    const int32_t v = r < 0 ? r : ~r;
    volatile float amm = 0.99999994039535522461f / -2147483648.0f;
    volatile float fv = (float)v;
    return amm * fv;
  }
  float rands() { return next(); }                               // :229-231
  float ran_sysm() { volatile float r = next(); return r * 2.0f - 1.0f; }   // :233-236
  // irands(n) = int(r*n) with r*n in REAL(SP) (:221-226); a product that
  // rounds up to n is kept in range
  int irands(int n) {
    volatile float r = next();
    volatile float p = r * (float)n;
    const int k = (int)p;
    return k < n ? k : n - 1;
  }
};

// PI of nrtype is REAL(SP) (src/mod_nrtype.f90:42)
static const double PI_SP = (double)3.14159265358979323846f;

static inline int modi(int i, int n) { return ((i - 1) % n + n) % n + 1; }   // periodic 1..n

// generate_newfield_space (mod_update.f90:441-467): amplitude * incell(i_bf)
// * cos(K.rpos) on every cell, amplitude = 2*distance/N_cell * rands()
static void newfield_space(const pqmc_global_params* gp, Ran2Host& rng, const double* kvec,
                           const std::vector<double>& incell, std::vector<double>& jump) {
  const double distance = 2 * gp->distance / gp->n_cell;
  const double amplitude = distance * (double)rng.rands();
  const double phi = 0.0;
  for (int c = 0; c < gp->n_cell; ++c) {
    double kr = 0.0;
    for (int d = 0; d < gp->lat_dim; ++d) kr += kvec[d] * gp->cell_rpos[d + (size_t)gp->lat_dim * c];
    for (int i = 0; i < gp->bf_sets; ++i) jump[(size_t)gp->bf_sets * c + i] = incell[i] * amplitude * cos(kr + phi);
  }
}

static int generate(const pqmc_model* m, const pqmc_global_params* gp, int kind, Ran2Host& rng, double* f,
                    double* ph, int* t_first, int* t_last) {
  const int nb = m->n_bf, nt = m->ntime;
  const double D = m->stiff, M = m->mass, dt = m->delt, bias = m->biased_phonon;
  auto at = [&](int b, int t1) -> double& { return f[b + (size_t)nb * (t1 - 1)]; };   // 1-based time
  double lncw = 0.0;
  *t_first = 1;
  *t_last = nt;
  switch (kind) {
    case PQMC_GLOBAL_EXCHANGE: {   // :304-314 (no action change)
      for (int i = 0; i < gp->n_global_update; ++i) {
        const int a = rng.irands(nb), s = rng.irands(nb);
        for (int t = 1; t <= nt; ++t) std::swap(at(a, t), at(s, t));
      }
      break;
    }
    case PQMC_GLOBAL_KSPACE:
    case PQMC_GLOBAL_KSPACE_TIME: {   // :316-374
      if (gp->lat_dim != 2) { set_error("global update: k-space moves need a 2-d lattice"); return PQMC_ERR_ARG; }
      const double kvec[2] = {2 * PI_SP * 0.5, 2 * PI_SP * 0.5};
      std::vector<double> incell(gp->bf_sets), jump((size_t)nb, 0.0);
      for (int i = 0; i < gp->bf_sets; ++i) incell[i] = rng.irands(2) * 2.0 - 1.0;
      newfield_space(gp, rng, kvec, incell, jump);
      int t0 = 1, t1 = nt;
      if (kind == PQMC_GLOBAL_KSPACE_TIME) {
        t0 = rng.irands(nt / 2) + 1;
        // end_time = max(start_time + int(M/delt**2), ntime) (:326); values
        // past ntime would index beyond boson_field, so the range is clipped
        t1 = std::min(std::max(t0 + (int)(1.0 * M / (dt * dt)), nt), nt);
      }
      // the endpoint neighbours before the change (kinetic term, :339-348)
      const int tm = modi(t0 - 1, nt), tp = modi(t1 + 1, nt);
      std::vector<double> o0(nb), om(nb), o1(nb), op(nb);
      for (int b = 0; b < nb; ++b) {
        o0[b] = at(b, t0); om[b] = at(b, tm); o1[b] = at(b, t1); op[b] = at(b, tp);
      }
      double dE = 0.0;
      for (int t = t0; t <= t1; ++t)
        for (int b = 0; b < nb; ++b) {
          const double xo = at(b, t), xn = xo + jump[b];
          at(b, t) = xn;
          dE = dE + 0.5 * D * (xn * xn - xo * xo);
          dE = dE + (-bias * (xn - xo));
        }
      if (kind == PQMC_GLOBAL_KSPACE_TIME) {
        const double kin = 0.5 * (M / (dt * dt));
        for (int b = 0; b < nb; ++b) {
          const double a0 = at(b, t0) - at(b, tm), b0 = o0[b] - om[b];
          dE = dE + kin * (a0 * a0 - b0 * b0);
          const double a1 = at(b, t1) - at(b, tp), b1 = o1[b] - op[b];
          dE = dE + kin * (a1 * a1 - b1 * b1);
        }
      }
      lncw = lncw - dE * dt;
      *t_first = t0;
      *t_last = t1;
      break;
    }
    case PQMC_GLOBAL_ROTATE: {   // :376-407 (no action change is computed)
      if (gp->bf_sets != 2) { set_error("global update: rotate needs two boson fields per cell"); return PQMC_ERR_ARG; }
      const double ang = (double)rng.ran_sysm() * 0.1 * PI_SP;
      double r11 = cos(ang), r12 = -sin(ang), r21 = sin(ang), r22 = cos(ang);
      if (rng.ran_sysm() < 0.0f) {
        r12 = -r12;
        r22 = -r22;
      }
      for (int c = 0; c < gp->n_cell; ++c) {
        const int bx = 2 * c, by = 2 * c + 1;
        for (int t = 1; t <= nt; ++t) {
          const double x = at(bx, t), y = at(by, t);
          at(bx, t) = r11 * x + r12 * y;
          at(by, t) = r21 * x + r22 * y;
        }
      }
      break;
    }
    case PQMC_GLOBAL_SINGLE: {   // :408-432
      if (!gp->flip && !gp->shift) {
        set_error("global update: the single-bond move needs flip or shift");
        return PQMC_ERR_ARG;
      }
      std::vector<double> tmp(nt);
      for (int i = 0; i < gp->n_global_update; ++i) {
        const int u = rng.irands(nb);
        if (gp->flip) {
          for (int t = 1; t <= nt; ++t) tmp[t - 1] = -at(u, t);
        } else {
          const double jump = (double)rng.ran_sysm() * gp->distance;
          for (int t = 1; t <= nt; ++t) tmp[t - 1] = at(u, t) + jump;
        }
        double dE = 0.0;
        if (!gp->flip) {
          double s = 0.0;
          for (int t = 1; t <= nt; ++t) s += tmp[t - 1] * tmp[t - 1] - at(u, t) * at(u, t);
          dE = 0.5 * D * s;
        }
        double s = 0.0;
        for (int t = 1; t <= nt; ++t) s += -bias * (tmp[t - 1] - at(u, t));
        dE = dE + s;
        for (int t = 1; t <= nt; ++t) at(u, t) = tmp[t - 1];
        lncw = lncw - dE * dt;
      }
      break;
    }
    default:
      set_error("global update: unknown kind %d", kind);
      return PQMC_ERR_ARG;
  }
  *ph = lncw;
  return PQMC_OK;
}

// cal_prob (mod_update.f90:475-500): only Re w enters the probability
static double global_prob(const pqmc_model* m, double re_w) {
  const double R = exp(std::min(10.0, re_w));
  if (m->metropolis) {
    double p = std::min(1.0, R);
    if (m->greatest_decent) p = floor(p);
    return p;
  }
  return R / (1 + R);
}

}  // namespace pqmc

using namespace pqmc;

extern "C" int pqmc_init_g(pqmc_chain* c, int start_time);

extern "C" {

int pqmc_global_generate(const pqmc_model* model, const pqmc_global_params* gp, int kind, int32_t rng[5],
                         double* field, double* ph_ln_cw, int* t_first, int* t_last) {
  if (!model || !gp || !rng || !field || !ph_ln_cw || !t_first || !t_last) {
    set_error("global_generate: null argument");
    return PQMC_ERR_ARG;
  }
  if (gp->n_cell * gp->bf_sets != model->n_bf || (!gp->cell_rpos && gp->n_cell > 0)) {
    set_error("global_generate: n_cell*bf_sets (%d*%d) must equal n_bf (%d)", gp->n_cell, gp->bf_sets, model->n_bf);
    return PQMC_ERR_ARG;
  }
  Ran2Host r(rng);
  PQMC_TRY(generate(model, gp, kind, r, field, ph_ln_cw, t_first, t_last));
  r.store(rng);
  return PQMC_OK;
}

int pqmc_set_global(pqmc_chain* c, const pqmc_global_params* gp) {
  if (!c || !gp) { set_error("set_global: null argument"); return PQMC_ERR_ARG; }
  if (gp->n_cell * gp->bf_sets != c->n_bf || gp->lat_dim < 1 || !gp->cell_rpos || gp->global_update_loop < 1) {
    set_error("set_global: inconsistent parameters (n_cell*bf_sets must equal n_bf %d)", c->n_bf);
    return PQMC_ERR_ARG;
  }
  c->gp = *gp;
  c->g_rpos.assign(gp->cell_rpos, gp->cell_rpos + (size_t)gp->lat_dim * gp->n_cell);
  c->gp.cell_rpos = c->g_rpos.data();
  c->have_global = true;
  return PQMC_OK;
}

int pqmc_update_global(pqmc_chain* c, int kind, int* accepted) {
  if (!c || !accepted) { set_error("update_global: null argument"); return PQMC_ERR_ARG; }
  if (!c->have_global) { set_error("update_global: call pqmc_set_global first"); return PQMC_ERR_STATE; }
  const size_t nf = (size_t)c->n_bf * c->ntime;
  std::vector<double> old(nf), fresh;
  DevScalars h;
  PQMC_CUDA(cudaMemcpyAsync(old.data(), c->field, sizeof(double) * nf, cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaMemcpyAsync(&h, c->sc, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  const cplx ln_old = h.ln_cw;
  fresh = old;
  Ran2Host rng(h.rng);
  double ph = 0.0;
  int t0 = 1, t1 = c->ntime;
  PQMC_TRY(generate(&c->hmodel, &c->gp, kind, rng, fresh.data(), &ph, &t0, &t1));
  // the exchange branch of the reference leaves expKV as it was (:304-314);
  // here every move refreshes expKV of the slices whose field changed
  PQMC_CUDA(cudaMemcpyAsync(c->field, fresh.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, c->stream));
  PQMC_TRY(launch_init_expkv(c, t0 - 1, t1 - t0 + 1));
  PQMC_TRY(do_new_weight(c));   // synchronises the stream
  DevScalars hn;
  PQMC_CUDA(cudaMemcpyAsync(&hn, c->sc, sizeof(hn), cudaMemcpyDeviceToHost, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  const double re_w = hn.ln_cw.x + ph - ln_old.x;
  const double prob = global_prob(&c->hmodel, re_w);
  const bool acc = (double)rng.rands() < prob;
  if (acc) {
    c->g_acc += 1;
  } else {
    c->g_rej += 1;
    PQMC_CUDA(cudaMemcpyAsync(c->field, old.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, c->stream));
    PQMC_TRY(launch_init_expkv(c, t0 - 1, t1 - t0 + 1));
    hn.ln_cw = ln_old;
  }
  rng.store(hn.rng);
  PQMC_CUDA(cudaMemcpyAsync(c->sc, &hn, sizeof(hn), cudaMemcpyHostToDevice, c->stream));
  PQMC_CUDA(cudaStreamSynchronize(c->stream));
  *accepted = acc ? 1 : 0;
  return PQMC_OK;
}

int pqmc_global_step(pqmc_chain* c, int loop, int* n_accepted) {
  if (!c) { set_error("global_step: null chain"); return PQMC_ERR_ARG; }
  if (n_accepted) *n_accepted = 0;
  if (!c->have_global) return PQMC_OK;
  const bool forward = (loop % 2) == 0;
  if (forward || ((loop + 1) % c->gp.global_update_loop) != 0) return PQMC_OK;
  int n = 0, a = 0;
  PQMC_TRY(pqmc_update_global(c, PQMC_GLOBAL_KSPACE, &a));
  n += a;
  if (c->gp.rotate) {
    PQMC_TRY(pqmc_update_global(c, PQMC_GLOBAL_ROTATE, &a));
    n += a;
  }
  PQMC_TRY(pqmc_update_global(c, PQMC_GLOBAL_KSPACE_TIME, &a));
  n += a;
  if (n > 0) PQMC_TRY(pqmc_init_g(c, 1));
  if (n_accepted) *n_accepted = n;
  return PQMC_OK;
}

int pqmc_global_counters(pqmc_chain* c, int64_t* accepted, int64_t* rejected) {
  if (!c || !accepted || !rejected) { set_error("global_counters: null argument"); return PQMC_ERR_ARG; }
  *accepted = c->g_acc;
  *rejected = c->g_rej;
  return PQMC_OK;
}

}  // extern "C"
