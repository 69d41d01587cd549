// pqmc_oracle.cpp -- CPU FP64 restatement of the projector-DQMC hot path of
// LEOMMM816/PQMC_allinone.  TEST INFRASTRUCTURE ONLY: used by tests/, by
// __graft_entry__.smoke() to check the GPU results, and by bench.py's cpu_baseline leg.
// The product (pqmc_allinone_gb300) never links or calls this file.
//
// Parity status: UNPINNED against reference outputs.  The reference ships no
// tests, golden vectors or fixtures for this path, and it cannot be built here
// (it is Fortran + MPI + LAPACK and no Fortran compiler exists in this image).
// The restatement is pinned instead by the reference's own invariants:
// closed-form vs expm expKV (src/mod_phonon_field.f90:451-469), fast vs
// scratch Green's function and ln_cw (src/mod_evolution.f90:179-193), and the
// lambda=0 free-fermion projector.  Every routine below cites the reference
// lines it follows.  Dense linear algebra follows the LAPACK conventions the
// reference calls (zgeqrf/zungqr, zgelqf/zunglq, zgetrf/zgetri) in unblocked
// form; OpenBLAS itself is not linked.
//
// Compiled with -ffp-contract=off so the float/double arithmetic of the RNG
// and of the acceptance test is the same on x86-64 and aarch64.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <thread>
#include <chrono>
#include "../include/pqmc_gb300.h"
#include "../include/pqmc_boxmuller.h"

namespace {

struct cd {
  double re, im;
};
static inline cd C(double r, double i = 0.0) { return cd{r, i}; }
static inline cd operator+(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
static inline cd operator-(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
static inline cd operator-(cd a) { return cd{-a.re, -a.im}; }
static inline cd operator*(cd a, cd b) {
  return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
static inline cd operator*(double s, cd a) { return cd{s * a.re, s * a.im}; }
static inline cd operator*(cd a, double s) { return cd{a.re * s, a.im * s}; }
static inline cd operator/(cd a, double s) { return cd{a.re / s, a.im / s}; }
static inline cd conj(cd a) { return cd{a.re, -a.im}; }
static inline double cabs_(cd a) { return std::hypot(a.re, a.im); }
// Smith's algorithm, the division gfortran and LAPACK's zladiv perform
static inline cd operator/(cd a, cd b) {
  if (std::fabs(b.re) >= std::fabs(b.im)) {
    double r = b.im / b.re, den = b.re + b.im * r;
    return cd{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return cd{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
  }
}
static inline cd clog_(cd a) { return cd{std::log(cabs_(a)), std::atan2(a.im, a.re)}; }
static inline cd cexp_(cd a) {
  double e = std::exp(a.re);
  return cd{e * std::cos(a.im), e * std::sin(a.im)};
}

// ---------------------------------------------------------------------------
// ran2_s of src/mod_ranstate.f90:171-191 (NR F90 combined generator).
// amm = nearest(1.0_sp,-1.0_sp)/hgng (:59).
struct Ran2 {
  int32_t iran, jran, kran, mran, nran;
  static float amm() { return (1.0f - 5.9604644775390625e-08f) / -2147483648.0f; }
  float next() {
    uint32_t ir = (uint32_t)iran, kr = (uint32_t)kran;
    int32_t rans = (int32_t)(ir - kr);
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
    uint32_t lo = m & 65535u;
    m = ((3533u * (m >> 16) + lo) << 16) + 3533u * lo + 820265819u;
    mran = (int32_t)m;
    int32_t r = (int32_t)(((uint32_t)nran ^ (uint32_t)kran) + (uint32_t)mran);
    int32_t v = r < 0 ? r : ~r;
    volatile float fv = (float)v;  // int -> real(sp), round to nearest
    volatile float h = amm() * fv;
    return h;
  }
  float rands() { return next(); }                // :229-231
  float ran_sysm() {                              // :233-236
    volatile float r = next();
    volatile float t = r * 2.0f;
    volatile float u = t - 1.0f;
    return u;
  }
};

// ---------------------------------------------------------------------------
// small dense helpers (column-major)
static inline cd& at(std::vector<cd>& a, int ld, int i, int j) { return a[(size_t)i + (size_t)ld * j]; }

// zdet analytic forms, src/mod_matrixlib.f90:515-590 (a is n x n col-major)
static cd det_small(int n, const cd* a) {
#define A(i, j) a[((i)-1) + n * ((j)-1)]
  if (n == 1) return A(1, 1);
  if (n == 2) return A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
  if (n == 3)
    return A(1, 1) * (A(2, 2) * A(3, 3) - A(2, 3) * A(3, 2)) -
           A(1, 2) * (A(2, 1) * A(3, 3) - A(2, 3) * A(3, 1)) +
           A(1, 3) * (A(2, 1) * A(3, 2) - A(2, 2) * A(3, 1));
  cd res = A(1, 1) * (A(2, 2) * (A(3, 3) * A(4, 4) - A(3, 4) * A(4, 3)) -
                      A(2, 3) * (A(3, 2) * A(4, 4) - A(3, 4) * A(4, 2)) +
                      A(2, 4) * (A(3, 2) * A(4, 3) - A(3, 3) * A(4, 2)));
  res = res - A(1, 2) * (A(2, 1) * (A(3, 3) * A(4, 4) - A(3, 4) * A(4, 3)) -
                         A(2, 3) * (A(3, 1) * A(4, 4) - A(3, 4) * A(4, 1)) +
                         A(2, 4) * (A(3, 1) * A(4, 3) - A(3, 3) * A(4, 1)));
  res = res + A(1, 3) * (A(2, 1) * (A(3, 2) * A(4, 4) - A(3, 4) * A(4, 2)) -
                         A(2, 2) * (A(3, 1) * A(4, 4) - A(3, 4) * A(4, 1)) +
                         A(2, 4) * (A(3, 1) * A(4, 2) - A(3, 2) * A(4, 1)));
  res = res - A(1, 4) * (A(2, 1) * (A(3, 2) * A(4, 3) - A(3, 3) * A(4, 2)) -
                         A(2, 2) * (A(3, 1) * A(4, 3) - A(3, 3) * A(4, 1)) +
                         A(2, 3) * (A(3, 1) * A(4, 2) - A(3, 2) * A(4, 1)));
  return res;
#undef A
}

// LU with partial pivoting, zgetf2 semantics (izamax uses |re|+|im|).
// Returns info (0 ok, >0 first zero pivot).  a overwritten by L\U.
static int zgetrf_(int n, cd* a, int lda, int* ipiv) {
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double best = -1.0;
    for (int i = j; i < n; ++i) {
      double v = std::fabs(a[i + (size_t)lda * j].re) + std::fabs(a[i + (size_t)lda * j].im);
      if (v > best) { best = v; jp = i; }
    }
    ipiv[j] = jp;
    cd piv = a[jp + (size_t)lda * j];
    if (piv.re != 0.0 || piv.im != 0.0) {
      if (jp != j)
        for (int k = 0; k < n; ++k) std::swap(a[j + (size_t)lda * k], a[jp + (size_t)lda * k]);
      cd rec = C(1.0) / a[j + (size_t)lda * j];
      for (int i = j + 1; i < n; ++i) a[i + (size_t)lda * j] = a[i + (size_t)lda * j] * rec;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {
      cd u = a[j + (size_t)lda * k];
      for (int i = j + 1; i < n; ++i)
        a[i + (size_t)lda * k] = a[i + (size_t)lda * k] - a[i + (size_t)lda * j] * u;
    }
  }
  return info;
}

// inverse from the LU factors (solves A X = I); zinverse :410-431
static int zinverse_(int n, cd* a) {
  std::vector<cd> lu(a, a + (size_t)n * n), x((size_t)n * n, C(0));
  std::vector<int> ipiv(n);
  int info = zgetrf_(n, lu.data(), n, ipiv.data());
  if (info) return info;
  for (int c = 0; c < n; ++c) {
    std::vector<cd> b(n, C(0));
    b[c] = C(1.0);
    for (int j = 0; j < n; ++j) std::swap(b[j], b[ipiv[j]]);
    for (int j = 0; j < n; ++j)
      for (int i = j + 1; i < n; ++i) b[i] = b[i] - lu[i + (size_t)n * j] * b[j];
    for (int j = n - 1; j >= 0; --j) {
      b[j] = b[j] / lu[j + (size_t)n * j];
      for (int i = 0; i < j; ++i) b[i] = b[i] - lu[i + (size_t)n * j] * b[j];
    }
    for (int i = 0; i < n; ++i) x[i + (size_t)n * c] = b[i];
  }
  std::memcpy(a, x.data(), sizeof(cd) * (size_t)n * n);
  return 0;
}

// log(det) with the reference's product form; when the product leaves the
// double range the same quantity is taken as a sum of logs.
static cd log_det_(int n, const cd* a, int* info_out) {
  if (n <= 4) return clog_(det_small(n, a));
  std::vector<cd> b(a, a + (size_t)n * n);
  std::vector<int> ipiv(n);
  int info = zgetrf_(n, b.data(), n, ipiv.data());
  *info_out = info;
  if (info) return C(-INFINITY);
  int s = 1;
  cd d = C(1.0);
  cd ls = C(0.0);
  for (int i = 0; i < n; ++i) {
    if (ipiv[i] != i) s = -s;
    d = d * b[i + (size_t)n * i];
    ls = ls + clog_(b[i + (size_t)n * i]);
  }
  if (s < 0) { d = -d; ls = ls + C(0.0, M_PI); }
  double ad = cabs_(d);
  if (ad > 1e-290 && ad < 1e290) return clog_(d);
  return ls;
}

// zlarfg: generate an elementary reflector (LAPACK convention, beta real)
static void zlarfg_(int n, cd* alpha, cd* x, int incx, cd* tau) {
  if (n <= 0) { *tau = C(0); return; }
  double xnorm = 0.0, scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n - 1; ++i) {
    const double v[2] = {x[(size_t)i * incx].re, x[(size_t)i * incx].im};
    for (double t : v) {
      if (t != 0.0) {
        double at_ = std::fabs(t);
        if (scale < at_) { ssq = 1.0 + ssq * (scale / at_) * (scale / at_); scale = at_; }
        else ssq += (at_ / scale) * (at_ / scale);
      }
    }
  }
  xnorm = scale * std::sqrt(ssq);
  double alphr = alpha->re, alphi = alpha->im;
  if (xnorm == 0.0 && alphi == 0.0) { *tau = C(0); return; }
  double nrm = std::sqrt(alphr * alphr + alphi * alphi + xnorm * xnorm);
  {
    // dlapy3 with scaling
    double w = std::fmax(std::fabs(alphr), std::fmax(std::fabs(alphi), xnorm));
    if (w > 0.0) {
      double a1 = alphr / w, a2 = alphi / w, a3 = xnorm / w;
      nrm = w * std::sqrt(a1 * a1 + a2 * a2 + a3 * a3);
    }
  }
  double beta = alphr >= 0.0 ? -nrm : nrm;
  *tau = C((beta - alphr) / beta, -alphi / beta);
  cd s = C(1.0) / (*alpha - C(beta));
  for (int i = 0; i < n - 1; ++i) x[(size_t)i * incx] = s * x[(size_t)i * incx];
  *alpha = C(beta);
}

// Householder QR in place: a(m,n) -> Q (first n columns), r(n,n) upper.
// zqr = zgeqrf + zungqr, src/mod_matrixlib.f90:452-467 (unblocked form).
static void zqr_(int m, int n, cd* a, int lda, cd* r) {
  std::vector<cd> tau(n);
  for (int i = 0; i < n; ++i) {
    cd* col = a + (size_t)lda * i;
    zlarfg_(m - i, &col[i], &col[i + 1], 1, &tau[i]);
    if (i < n - 1) {
      cd alpha = col[i];
      col[i] = C(1.0);
      cd ct = conj(tau[i]);
      for (int j = i + 1; j < n; ++j) {
        cd* cj = a + (size_t)lda * j;
        cd w = C(0);
        for (int k = i; k < m; ++k) w = w + conj(col[k]) * cj[k];
        cd f = ct * w;
        for (int k = i; k < m; ++k) cj[k] = cj[k] - col[k] * f;
      }
      col[i] = alpha;
    }
  }
  if (r) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) r[i + (size_t)n * j] = (i <= j) ? a[i + (size_t)lda * j] : C(0);
  }
  // zung2r
  for (int i = n - 1; i >= 0; --i) {
    cd* col = a + (size_t)lda * i;
    if (i < n - 1) {
      col[i] = C(1.0);
      for (int j = i + 1; j < n; ++j) {
        cd* cj = a + (size_t)lda * j;
        cd w = C(0);
        for (int k = i; k < m; ++k) w = w + conj(col[k]) * cj[k];
        cd f = tau[i] * w;
        for (int k = i; k < m; ++k) cj[k] = cj[k] - col[k] * f;
      }
    }
    for (int k = i + 1; k < m; ++k) col[k] = (-tau[i]) * col[k];
    col[i] = C(1.0) - tau[i];
    for (int k = 0; k < i; ++k) col[k] = C(0);
  }
}

// zqdr :323-334: Q overwrites a, d = diag(R)
static void zqdr_(int m, int n, cd* a, cd* d) {
  std::vector<cd> r((size_t)n * n);
  zqr_(m, n, a, m, r.data());
  for (int i = 0; i < n; ++i) d[i] = r[i + (size_t)n * i];
}

// zlq :488-503 by the equivalent QR of a^H: a(m,n) -> Q rows, l(m,m) lower.
static void zlq_(int m, int n, cd* a, cd* l) {
  std::vector<cd> at_((size_t)n * m), r((size_t)m * m);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) at_[j + (size_t)n * i] = conj(a[i + (size_t)m * j]);
  zqr_(n, m, at_.data(), n, r.data());
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) a[i + (size_t)m * j] = conj(at_[j + (size_t)n * i]);
  if (l)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) l[i + (size_t)m * j] = conj(r[j + (size_t)m * i]);
}

// zldq :349-360
static void zldq_(int m, int n, cd* a, cd* d) {
  std::vector<cd> l((size_t)m * m);
  zlq_(m, n, a, l.data());
  for (int i = 0; i < m; ++i) d[i] = l[i + (size_t)m * i];
}

// Matrix functions of a Hermitian H (dim <= 4) through the real symmetric
// embedding S = [[Re H, -Im H], [Im H, Re H]] and cyclic Jacobi on S.  For a
// real function f, f(S) embeds f(H) the same way, whatever the eigenvalue
// degeneracy.  Stands in for zheev inside zexpm (src/mod_matrixlib.f90:
// 251-289, 374-385): exp(mat) for Hermitian mat, and for anti-Hermitian mat
// exp(-i*(i*mat)) from the eigen-decomposition of i*mat.
static void sym_jacobi_(int n, double* a, double* w, double* v) {
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
        double t = 1.0 / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
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

// zexpm :251-289 for dim <= 4
static void zexpm_(int n, cd* mat) {
  if (n == 1) { mat[0] = cexp_(mat[0]); return; }
  double dh = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) dh = std::fmax(dh, cabs_(mat[i + n * j] - conj(mat[j + n * i])));
  bool herm = dh < 1e-7;
  cd h[16];
  for (int k = 0; k < n * n; ++k) h[k] = herm ? mat[k] : C(0.0, 1.0) * mat[k];
  const int m = 2 * n;
  double s[64], v[64], w[8];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      cd z = h[i + n * j];
      s[i + m * j] = z.re;
      s[(i + n) + m * (j + n)] = z.re;
      s[i + m * (j + n)] = -z.im;
      s[(i + n) + m * j] = z.im;
    }
  sym_jacobi_(m, s, w, v);
  // f1 = exp (Hermitian) or cos (anti-Hermitian); f2 = sin (anti-Hermitian)
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a1 = 0.0, b1 = 0.0, a2 = 0.0, b2 = 0.0;
      for (int k = 0; k < m; ++k) {
        double f1 = herm ? std::exp(w[k]) : std::cos(w[k]);
        double f2 = herm ? 0.0 : std::sin(w[k]);
        a1 += v[i + m * k] * f1 * v[j + m * k];
        b1 += v[(i + n) + m * k] * f1 * v[j + m * k];
        a2 += v[i + m * k] * f2 * v[j + m * k];
        b2 += v[(i + n) + m * k] * f2 * v[j + m * k];
      }
      // herm: exp(H) = a1 + i b1;  anti: exp(-iH') = cos(H') - i sin(H')
      mat[i + n * j] = herm ? C(a1, b1) : C(a1 + b2, b1 - a2);
    }
}

// ---------------------------------------------------------------------------
struct Chain {
  // model
  int ns, nelec, ntime, ngroup, nblock, n_pf, pdim, max_pla, n_bf;
  int expkv_kind, ncopy, tr_weight, metropolis, greatest_decent, local_update, proposal_kind;
  double delt, M, D, biased, jump;
  std::vector<int> pf_dim, pf_npla, pf_k_exist, pf_v_exist;
  std::vector<cd> k_coe, v_coe, kmat, vmat, bc_phases;
  std::vector<int> pla_site_list, bf_list, boundary_crossing;
  // state
  std::vector<double> field;   // (n_bf, ntime)
  std::vector<cd> expkv, expkv_inv;  // (pdim,pdim,max_pla,n_pf,ntime)
  std::vector<cd> g_h;         // (ns,ns)
  std::vector<cd> q_string, d_string;  // (ns,nelec,nblock), (nelec,nblock)
  std::vector<cd> slater_q, slater_d;
  cd ln_cw = C(0);
  double err_fast = 0.0, err_fast_max = 1e-6;
  int64_t pos_acc = 0, neg_acc = 0;
  Ran2 rng{1, 1, 1, 1, 1};
  bool have_g = false;
  // measurement
  bool have_meas = false;
  int n_cell = 0;
  std::vector<int> cell_sites, cell_bf, cell_xnb, cell_ynb, cell_cross, rel_index;
  cd bc_phase[2];
  std::vector<cd> k_phase;
  double hop = 1.0, ep = 1.0;
  std::vector<cd> meas_acc;  // record being accumulated

  size_t kv_idx(int i, int j, int pla, int pf, int t) const {
    return (size_t)i + (size_t)pdim * (j + (size_t)pdim * (pla + (size_t)max_pla * (pf + (size_t)n_pf * t)));
  }
  int site(int k, int pla, int pf) const { return pla_site_list[k + pdim * (pla + max_pla * pf)]; }
  int bfi(int pla, int pf) const { return bf_list[pla + max_pla * pf]; }
  double& x(int b, int t) { return field[(size_t)b + (size_t)n_bf * t]; }
  cd& G(int i, int j) { return g_h[(size_t)i + (size_t)ns * j]; }
  cd* Q(int blk) { return &q_string[(size_t)ns * nelec * blk]; }
  cd* Dv(int blk) { return &d_string[(size_t)nelec * blk]; }
};

// get_expKV dispatch (setup_expKV, src/mod_phonon_field.f90:472-496);
// out is dim x dim col-major with leading dimension dim.
static void get_expkv(const Chain& c, int pf, int pla, double bf, bool inv, cd* out) {
  int dim = c.pf_dim[pf], pd = c.pdim;
  const cd* K = &c.kmat[(size_t)pd * pd * pf];
  const cd* V = &c.vmat[(size_t)pd * pd * pf];
  const cd* BC = &c.bc_phases[(size_t)pd * pd * (pf * (size_t)c.max_pla + pla)];
  bool cross = c.boundary_crossing[pla + c.max_pla * pf] != 0;
  cd kc = c.k_coe[pf], vc = c.v_coe[pf];
  for (int k = 0; k < dim * dim; ++k) out[k] = C(0);
  if (c.expkv_kind == PQMC_EXPKV_EPSOCZ || c.expkv_kind == PQMC_EXPKV_EPSOCZ_BLOCK) {
    // get_expKV_epsocz :534-569
    cd sub[4];
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        cd kk = K[i + pd * (j + 2)], vv = V[i + pd * (j + 2)];
        sub[i + 2 * j] = (-c.delt) * (kc * kk + (vc * bf) * vv);
        if (cross) sub[i + 2 * j] = sub[i + 2 * j] * BC[i + pd * (j + 2)];
      }
    double norm;
    if (c.expkv_kind == PQMC_EXPKV_EPSOCZ) {
      double a = cabs_(kc), b = cabs_(vc) * bf;
      norm = c.delt * std::sqrt(a * a + b * b);
    } else {
      cd h11 = kc * K[0 + pd * 2] + (vc * bf) * V[0 + pd * 2];
      cd h21 = kc * K[1 + pd * 2] + (vc * bf) * V[1 + pd * 2];
      double a = cabs_(h11), b = cabs_(h21);
      norm = c.delt * std::sqrt(a * a + b * b);
    }
    double ch = std::cosh(norm), sh = std::sinh(norm);
    for (int i = 0; i < dim; ++i) out[i + dim * i] = C(ch);
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        cd s = inv ? -sub[i + 2 * j] : sub[i + 2 * j];
        out[i + dim * (j + 2)] = (s * sh) / norm;
      }
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) out[(i + 2) + dim * j] = conj(out[j + dim * (i + 2)]);
    return;
  }
  if (c.expkv_kind == PQMC_EXPKV_EPSOC) {
    // get_expKV_epsoc :572-604
    double a = cabs_(kc), b = cabs_(vc) * bf;
    double norm = c.delt * std::sqrt(a * a + b * b);
    double ch = std::cosh(norm), sh = std::sinh(norm);
    for (int i = 0; i < dim; ++i) out[i + dim * i] = C(ch);
    cd sub = (-c.delt) * (kc * K[0 + pd * 1] + (vc * bf) * V[0 + pd * 1]);
    if (cross) sub = sub * BC[0 + pd * 1];
    cd s = inv ? -sub : sub;
    out[0 + dim * 1] = (s * sh) / norm;
    out[1 + dim * 0] = conj(out[0 + dim * 1]);
    return;
  }
  // get_expKV_general :497-532
  bool ke = c.pf_k_exist[pf] != 0, ve = c.pf_v_exist[pf] != 0;
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) {
      cd kk = K[i + pd * j], vv = V[i + pd * j];
      cd h = C(0);
      if (ve && ke) h = kc * kk + (vc * bf) * vv;
      else if (ve) h = (vc * bf) * vv;
      else if (ke) h = kc * kk;
      if (cross) h = h * BC[i + pd * j];
      out[i + dim * j] = (inv ? c.delt : -c.delt) * h;
    }
  zexpm_(dim, out);
}

static void store_expkv(Chain& c, int pf, int pla, int t, const cd* m, bool inv) {
  int dim = c.pf_dim[pf];
  std::vector<cd>& dst = inv ? c.expkv_inv : c.expkv;
  for (int j = 0; j < c.pdim; ++j)
    for (int i = 0; i < c.pdim; ++i)
      dst[c.kv_idx(i, j, pla, pf, t)] = (i < dim && j < dim) ? m[i + dim * j] : C(0);
}

// init_expKV for all families + set_pf_expKV_mat (:423-450, :605-636)
static void init_expkv(Chain& c) {
  cd m[16];
  for (int pf = 0; pf < c.n_pf; ++pf)
    for (int t = 0; t < c.ntime; ++t)
      for (int p = 0; p < c.pf_npla[pf]; ++p) {
        double bf = c.pf_v_exist[pf] ? c.x(c.bfi(p, pf), t) : 0.0;
        get_expkv(c, pf, p, bf, false, m);
        store_expkv(c, pf, p, t, m, false);
        get_expkv(c, pf, p, bf, true, m);
        store_expkv(c, pf, p, t, m, true);
      }
}

static inline int modi(int n, int p) {  // src/mod_matrixlib.f90:66-77
  int r = n % p;
  if (n < 0) return p + r;
  if (r == 0) return p;
  return r;
}

// cal_energy_difference, src/mod_update.f90:203-228 (time 1-based)
static double energy_difference(Chain& c, int bf, int time, double jump) {
  double be = c.x(bf, modi(time - 1, c.ntime) - 1);
  double af = c.x(bf, modi(time + 1, c.ntime) - 1);
  double now = c.x(bf, time - 1);
  double nw = now + jump;
  double dt2 = c.delt * c.delt;
  double e1 = ((0.5 * c.M) * ((be - now) * (be - now) + (af - now) * (af - now))) / dt2 +
              (0.5 * c.D) * (now * now) - c.biased * now;
  double e2 = ((0.5 * c.M) * ((be - nw) * (be - nw) + (af - nw) * (af - nw))) / dt2 +
              (0.5 * c.D) * (nw * nw) - c.biased * nw;
  return e2 - e1;
}

// cal_prob, src/mod_update.f90:475-500 (the sign-problem print is omitted)
static double cal_prob(const Chain& c, cd w) {
  double rt = std::exp(std::fmin(10.0, w.re));
  double prob;
  if (c.metropolis) {
    prob = std::fmin(1.0, rt);
    if (c.greatest_decent) prob = std::floor(prob);
  } else {
    prob = rt / (1.0 + rt);
  }
  return prob;
}

static double draw_jump(Chain& c) {
  if (c.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
    // Box-Muller on two ran2 draws (u1 in (0,1), so log is finite), with the
    // fixed-order arithmetic the CUDA kernels use (bit-identical jumps)
    double u1 = (double)c.rng.rands();
    double u2 = (double)c.rng.rands();
    return pqmc_bm_gauss_jump(c.jump, u1, u2);
  }
  return c.jump * (double)c.rng.ran_sysm();
}

// update_phonon_field(ppf,time), src/mod_update.f90:13-201 (n_local_update=1)
static void update_phonon_field(Chain& c, int pf, int time) {
  const int dim = c.pf_dim[pf], ns = c.ns, t = time - 1;
  cd gsub[16], delta[16], rmat[16], eold[16], enew[16], tmp[16];
  std::vector<cd> u((size_t)ns * dim), v((size_t)dim * ns);
  for (int p = 0; p < c.pf_npla[pf]; ++p) {
    int S[4];
    for (int k = 0; k < dim; ++k) S[k] = c.site(k, p, pf);
    int b = c.bfi(p, pf);
    double old_bf = c.x(b, t);
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) gsub[i + dim * j] = c.G(S[i], S[j]);
    double jump = draw_jump(c);                                  // :84
    cd dE = C(energy_difference(c, b, time, jump));              // :87
    dE = (-c.delt) * dE;                                         // :88
    c.x(b, t) = c.x(b, t) + jump;                                // :92
    double xnew = c.x(b, t);
    // calculate_Delta :230-245
    get_expkv(c, pf, p, xnew, false, enew);
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + c.expkv_inv[c.kv_idx(i, k, p, pf, t)] * enew[k + dim * j];
        delta[i + dim * j] = s;
      }
    for (int i = 0; i < dim; ++i) delta[i + dim * i] = delta[i + dim * i] - C(1.0);
    // R = I + g_h_sub * Delta   :97-100
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + gsub[i + dim * k] * delta[k + dim * j];
        rmat[i + dim * j] = s;
      }
    for (int i = 0; i < dim; ++i) rmat[i + dim * i] = rmat[i + dim * i] + C(1.0);
    cd r_elec = C(1.0) * det_small(dim, rmat);                  // :101
    if (c.tr_weight) r_elec = r_elec * conj(r_elec);             // :103
    {
      cd base = r_elec, acc = C(1.0);
      for (int k = 0; k < c.ncopy; ++k) acc = acc * base;        // :104
      r_elec = acc;
    }
    dE = dE + clog_(r_elec);                                     // :108
    double prob = cal_prob(c, dE);                               // :112
    double r = (double)c.rng.rands();                            // :117
    if (prob < r) {
      c.x(b, t) = c.x(b, t) - jump;                              // :119
      c.x(b, t) = old_bf;                                        // :194
      c.neg_acc++;
      continue;
    }
    // accepted :122-142
    get_expkv(c, pf, p, xnew, false, enew);
    store_expkv(c, pf, p, t, enew, false);
    get_expkv(c, pf, p, xnew, true, tmp);
    store_expkv(c, pf, p, t, tmp, true);
    c.ln_cw = c.ln_cw + C(std::log(r_elec.re));                  // :142
    c.pos_acc++;
    // final update of g :146-192
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) gsub[i + dim * j] = c.G(S[i], S[j]);
    get_expkv(c, pf, p, old_bf, true, eold);                     // :158
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + eold[i + dim * k] * c.expkv[c.kv_idx(k, j, p, pf, t)];
        delta[i + dim * j] = s;
      }
    for (int i = 0; i < dim; ++i) delta[i + dim * i] = delta[i + dim * i] - C(1.0);
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + gsub[i + dim * k] * delta[k + dim * j];
        rmat[i + dim * j] = s;
      }
    for (int i = 0; i < dim; ++i) rmat[i + dim * i] = rmat[i + dim * i] + C(1.0);
    zinverse_(dim, rmat);                                        // :171
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + delta[i + dim * k] * rmat[k + dim * j];
        tmp[i + dim * j] = s;                                    // :173
      }
    // gh_part_nd_temp = g_h(:,S) * T    :177
    for (int k = 0; k < dim; ++k)
      for (int i = 0; i < ns; ++i) {
        cd s = C(0);
        for (int l = 0; l < dim; ++l) s = s + c.G(i, S[l]) * tmp[l + dim * k];
        u[i + (size_t)ns * k] = s;
      }
    // g_part_dn = (I - g_h)(S,:)   :154-157
    for (int j = 0; j < ns; ++j)
      for (int k = 0; k < dim; ++k) v[k + (size_t)dim * j] = -c.G(S[k], j);
    for (int k = 0; k < dim; ++k) v[k + (size_t)dim * S[k]] = v[k + (size_t)dim * S[k]] + C(1.0);
    // g_h += gh_part_nd_temp * g_part_dn   :187
    for (int j = 0; j < ns; ++j) {
      cd* gc = &c.g_h[(size_t)ns * j];
      cd vv[4];
      for (int k = 0; k < dim; ++k) vv[k] = v[k + (size_t)dim * j];
      for (int i = 0; i < ns; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + u[i + (size_t)ns * k] * vv[k];
        gc[i] = gc[i] + s;
      }
    }
  }
}

// left_evolve (time 1-based, pf 0-based), src/mod_evolution.f90:236-285
static void left_evolve(Chain& c, int time, cd* mat, int n, int pf, bool two_way) {
  const int dim = c.pf_dim[pf], ns = c.ns, t = time - 1;
  for (int p = 0; p < c.pf_npla[pf]; ++p) {
    int S[4];
    for (int k = 0; k < dim; ++k) S[k] = c.site(k, p, pf);
    for (int j = 0; j < n; ++j) {
      cd b[4], o[4];
      for (int k = 0; k < dim; ++k) b[k] = mat[S[k] + (size_t)ns * j];
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + c.expkv[c.kv_idx(i, k, p, pf, t)] * b[k];
        o[i] = s;
      }
      for (int k = 0; k < dim; ++k) mat[S[k] + (size_t)ns * j] = o[k];
    }
  }
  if (!two_way) return;
  for (int p = 0; p < c.pf_npla[pf]; ++p) {
    int S[4];
    for (int k = 0; k < dim; ++k) S[k] = c.site(k, p, pf);
    for (int i = 0; i < n; ++i) {
      cd b[4], o[4];
      for (int k = 0; k < dim; ++k) b[k] = mat[i + (size_t)ns * S[k]];
      for (int j = 0; j < dim; ++j) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + b[k] * c.expkv_inv[c.kv_idx(k, j, p, pf, t)];
        o[j] = s;
      }
      for (int k = 0; k < dim; ++k) mat[i + (size_t)ns * S[k]] = o[k];
    }
  }
}

// right_evolve, src/mod_evolution.f90:287-328; mat is (n, ns)
static void right_evolve(Chain& c, int time, cd* mat, int n, int pf, bool two_way) {
  const int dim = c.pf_dim[pf], t = time - 1;
  for (int p = 0; p < c.pf_npla[pf]; ++p) {
    int S[4];
    for (int k = 0; k < dim; ++k) S[k] = c.site(k, p, pf);
    for (int i = 0; i < n; ++i) {
      cd b[4], o[4];
      for (int k = 0; k < dim; ++k) b[k] = mat[i + (size_t)n * S[k]];
      for (int j = 0; j < dim; ++j) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + b[k] * c.expkv[c.kv_idx(k, j, p, pf, t)];
        o[j] = s;
      }
      for (int k = 0; k < dim; ++k) mat[i + (size_t)n * S[k]] = o[k];
    }
  }
  if (!two_way) return;
  for (int p = 0; p < c.pf_npla[pf]; ++p) {
    int S[4];
    for (int k = 0; k < dim; ++k) S[k] = c.site(k, p, pf);
    for (int j = 0; j < c.ns; ++j) {
      cd b[4], o[4];
      for (int k = 0; k < dim; ++k) b[k] = mat[S[k] + (size_t)n * j];
      for (int i = 0; i < dim; ++i) {
        cd s = C(0);
        for (int k = 0; k < dim; ++k) s = s + c.expkv_inv[c.kv_idx(i, k, p, pf, t)] * b[k];
        o[i] = s;
      }
      for (int k = 0; k < dim; ++k) mat[S[k] + (size_t)n * j] = o[k];
    }
  }
}

static cd branch_reduce(cd z) {
  // cmplx(real(z), mod(aimag(z), 2*pi)) with pi = PI of nrtype (REAL(SP)),
  // src/mod_evolution.f90:356 and src/mod_nrtype.f90:42
  const double two_pi_sp = (double)(2.0f * 3.14159265358979323846f);
  return C(z.re, std::fmod(z.im, two_pi_sp));
}

// cal_g_and_det_T0(lmat,rmat), src/mod_evolution.f90:330-357
static int cal_g_and_det(Chain& c, const cd* lmat, const cd* rmat) {
  const int ne = c.nelec, ns = c.ns;
  std::vector<cd> pbp((size_t)ne * ne, C(0)), buf((size_t)ns * ne, C(0));
  for (int j = 0; j < ne; ++j)
    for (int k = 0; k < ns; ++k) {
      cd r = rmat[k + (size_t)ns * j];
      for (int i = 0; i < ne; ++i) pbp[i + (size_t)ne * j] = pbp[i + (size_t)ne * j] + lmat[i + (size_t)ne * k] * r;
    }
  int info = 0;
  cd lndet = log_det_(ne, pbp.data(), &info);
  if (info) return PQMC_ERR_SINGULAR;
  cd lncw = lndet;
  cd sumd = C(0);
  for (size_t k = 0; k < c.d_string.size(); ++k) sumd = sumd + clog_(c.d_string[k]);
  lncw = lncw + sumd;
  if (zinverse_(ne, pbp.data())) return PQMC_ERR_SINGULAR;
  for (int j = 0; j < ne; ++j)
    for (int k = 0; k < ne; ++k) {
      cd p = pbp[k + (size_t)ne * j];
      for (int i = 0; i < ns; ++i) buf[i + (size_t)ns * j] = buf[i + (size_t)ns * j] + rmat[i + (size_t)ns * k] * p;
    }
  std::fill(c.g_h.begin(), c.g_h.end(), C(0));
  for (int j = 0; j < ns; ++j)
    for (int k = 0; k < ne; ++k) {
      cd l = lmat[k + (size_t)ne * j];
      cd* gc = &c.g_h[(size_t)ns * j];
      const cd* bc = &buf[(size_t)ns * k];
      for (int i = 0; i < ns; ++i) gc[i] = gc[i] + bc[i] * l;
    }
  if (c.tr_weight) lncw = lncw + conj(lncw);
  lncw = lncw * (double)c.ncopy;
  c.ln_cw = branch_reduce(lncw);
  return PQMC_OK;
}

static void herm_t(int m, int n, const cd* a, cd* out) {  // out(n,m) = a(m,n)^H
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) out[j + (size_t)n * i] = conj(a[i + (size_t)m * j]);
}

// init_g_T0(start_time), src/mod_evolution.f90:46-111
static int init_g(Chain& c, int start_time) {
  const int ns = c.ns, ne = c.nelec, nb = c.nblock;
  c.ln_cw = C(0);
  std::memcpy(c.Q(0), c.slater_q.data(), sizeof(cd) * ns * ne);
  std::memcpy(c.Q(nb - 1), c.slater_q.data(), sizeof(cd) * ns * ne);
  std::memcpy(c.Dv(0), c.slater_d.data(), sizeof(cd) * ne);
  std::memcpy(c.Dv(nb - 1), c.slater_d.data(), sizeof(cd) * ne);
  int start_block = start_time / c.ngroup + 1;
  int start_by_block = (start_block - 1) * c.ngroup + 1;
  if (start_by_block > start_time) return PQMC_ERR_ARG;
  std::vector<cd> rmat(c.Q(start_block - 1), c.Q(start_block - 1) + (size_t)ns * ne);
  for (int p = start_by_block; p <= c.ntime; ++p) {
    for (int pf = 0; pf < c.n_pf; ++pf) left_evolve(c, p, rmat.data(), ne, pf, false);
    if (p % c.ngroup != 0) continue;
    int blk = (p - 1) / c.ngroup + 2;
    zqdr_(ns, ne, rmat.data(), c.Dv(blk - 1));
    std::memcpy(c.Q(blk - 1), rmat.data(), sizeof(cd) * ns * ne);
  }
  std::vector<cd> lmat((size_t)ne * ns);
  herm_t(ns, ne, c.Q(nb - 1), lmat.data());
  int st = cal_g_and_det(c, lmat.data(), rmat.data());
  c.have_g = true;
  return st;
}

// get_g_scratch_T0(time,forward,loop), src/mod_evolution.f90:113-195
static int get_g_scratch(Chain& c, int time, bool forward, int loop, double* err_out) {
  (void)loop;
  const int ns = c.ns, ne = c.nelec;
  cd lncw_fast = c.ln_cw;
  c.ln_cw = C(0);
  std::vector<cd> gfast = c.g_h;
  std::vector<cd> rmat((size_t)ns * ne), lmat((size_t)ne * ns);
  if (forward) {
    int blk = time / c.ngroup + 1;
    std::memcpy(rmat.data(), c.Q(blk - 2), sizeof(cd) * ns * ne);
    for (int p = time - c.ngroup; p <= time - 1; ++p)
      for (int pf = 0; pf < c.n_pf; ++pf) left_evolve(c, p, rmat.data(), ne, pf, false);
    zqdr_(ns, ne, rmat.data(), c.Dv(blk - 1));
    std::memcpy(c.Q(blk - 1), rmat.data(), sizeof(cd) * ns * ne);
    herm_t(ns, ne, c.Q(blk), lmat.data());
  } else {
    int blk = time / c.ngroup + 2;
    if (c.ngroup == 1) blk = blk - 1;
    herm_t(ns, ne, c.Q(blk), lmat.data());
    for (int p = time + c.ngroup - 1; p >= time; --p)
      for (int pf = c.n_pf - 1; pf >= 0; --pf) right_evolve(c, p, lmat.data(), ne, pf, false);
    zldq_(ne, ns, lmat.data(), c.Dv(blk - 1));
    herm_t(ne, ns, lmat.data(), c.Q(blk - 1));
    std::memcpy(rmat.data(), c.Q(blk - 2), sizeof(cd) * ns * ne);
  }
  int st = cal_g_and_det(c, lmat.data(), rmat.data());
  double e1 = 0.0;
  for (size_t k = 0; k < gfast.size(); ++k) e1 = std::fmax(e1, cabs_(gfast[k] - c.g_h[k]));
  c.err_fast = e1;
  if (e1 > c.err_fast_max) c.err_fast_max = e1;
  double e2 = std::fabs((c.ln_cw - lncw_fast).re);
  c.err_fast = e2;
  if (e2 > c.err_fast_max) c.err_fast_max = e2;
  if (err_out) { err_out[0] = e1; err_out[1] = e2; }
  return st;
}

// cal_new_weight_T0, src/mod_evolution.f90:359-408
static int cal_new_weight(Chain& c, cd* out) {
  const int ns = c.ns, d = c.nelec, nb = c.nblock;
  cd lndet = C(0);
  std::vector<cd> lmat((size_t)d * ns), tmat((size_t)d * d);
  herm_t(ns, d, c.Q(nb - 1), lmat.data());
  for (int i = 0; i < d; ++i) lndet = lndet + clog_(c.Dv(nb - 1)[i]);
  int flag = 0;
  for (int p = c.ntime; p >= 1; --p) {
    for (int pf = c.n_pf - 1; pf >= 0; --pf) right_evolve(c, p, lmat.data(), d, pf, false);
    flag++;
    if (flag != c.ngroup) continue;
    flag = 0;
    zlq_(d, ns, lmat.data(), tmat.data());
    for (int i = 0; i < d; ++i) lndet = lndet + clog_(tmat[i + (size_t)d * i]);
  }
  for (int i = 0; i < d; ++i) lndet = lndet + clog_(c.Dv(0)[i]);
  std::fill(tmat.begin(), tmat.end(), C(0));
  const cd* r = c.Q(0);
  for (int j = 0; j < d; ++j)
    for (int k = 0; k < ns; ++k) {
      cd rv = r[k + (size_t)ns * j];
      for (int i = 0; i < d; ++i) tmat[i + (size_t)d * j] = tmat[i + (size_t)d * j] + lmat[i + (size_t)d * k] * rv;
    }
  int info = 0;
  lndet = lndet + log_det_(d, tmat.data(), &info);
  if (info) return PQMC_ERR_SINGULAR;
  if (c.tr_weight) lndet = lndet + conj(lndet);
  cd lncw = lndet * (double)c.ncopy;
  c.ln_cw = branch_reduce(lncw);
  if (out) *out = c.ln_cw;
  return PQMC_OK;
}

// ---------------------------------------------------------------------------
// measurement, src/mod_meas.f90:64-208 (helpers) and :210-544
static int meas_width(const Chain& c) { return PQMC_N_SCALAR + 2 * PQMC_N_FIELD * c.n_cell; }

static void wick(const Chain& c, const std::vector<cd>& g, int n, const int (*ls)[2],
                 const int (*rs)[2], bool hartree_only, cd* mat) {
  auto gh = [&](int i, int j) { return c.g_h[(size_t)i + (size_t)c.ns * j]; };
  auto gg = [&](int i, int j) { return g[(size_t)i + (size_t)c.ns * j]; };
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      cd m = C(0);
      m = m + gh(ls[i][1], ls[i][0]) * gh(rs[j][1], rs[j][0]);
      if (!hartree_only) m = m + gh(rs[j][1], ls[i][0]) * gg(ls[i][1], rs[j][0]);
      mat[i + n * j] = m;
    }
}

static void spin_current(const Chain& c, const std::vector<cd>& g, int p1, int p2, int p3, int p4,
                         bool h, cd* mat) {
  auto s = [&](int cell, int k) { return c.cell_sites[k + 2 * cell]; };
  int ls[4][2] = {{s(p1, 0), s(p2, 1)}, {s(p1, 1), s(p2, 0)}, {s(p2, 0), s(p1, 1)}, {s(p2, 1), s(p1, 0)}};
  int rs[4][2] = {{s(p3, 0), s(p4, 1)}, {s(p3, 1), s(p4, 0)}, {s(p4, 0), s(p3, 1)}, {s(p4, 1), s(p3, 0)}};
  wick(c, g, 4, ls, rs, h, mat);
}

static void spin_momentum(const Chain& c, const std::vector<cd>& g, int p1, int p2, cd* mat) {
  auto s = [&](int cell, int k) { return c.cell_sites[k + 2 * cell]; };
  int ls[4][2] = {{s(p1, 0), s(p1, 0)}, {s(p1, 0), s(p1, 1)}, {s(p1, 1), s(p1, 0)}, {s(p1, 1), s(p1, 1)}};
  int rs[4][2] = {{s(p2, 0), s(p2, 0)}, {s(p2, 0), s(p2, 1)}, {s(p2, 1), s(p2, 0)}, {s(p2, 1), s(p2, 1)}};
  wick(c, g, 4, ls, rs, false, mat);
}

static void phys_current(const Chain& c, const std::vector<cd>& g, int p1, int p2, int p3, int p4,
                         cd* mat) {
  auto s = [&](int cell, int k) { return c.cell_sites[k + 2 * cell]; };
  int ls[8][2] = {{s(p1, 0), s(p2, 1)}, {s(p1, 1), s(p2, 0)}, {s(p2, 0), s(p1, 1)}, {s(p2, 1), s(p1, 0)},
                  {s(p1, 0), s(p2, 0)}, {s(p1, 1), s(p2, 1)}, {s(p2, 0), s(p1, 0)}, {s(p2, 1), s(p1, 1)}};
  int rs[8][2] = {{s(p3, 0), s(p4, 1)}, {s(p3, 1), s(p4, 0)}, {s(p4, 0), s(p3, 1)}, {s(p4, 1), s(p3, 0)},
                  {s(p3, 0), s(p4, 0)}, {s(p3, 1), s(p4, 1)}, {s(p4, 0), s(p3, 0)}, {s(p4, 1), s(p3, 1)}};
  wick(c, g, 8, ls, rs, false, mat);
}

// add_boundary_phase :199-208
static void bphase(const Chain& c, cd* v, bool cross, int dir) {
  if (!cross) return;
  cd bc = c.bc_phase[dir];
  v[0] = v[0] * bc; v[1] = v[1] * bc; v[2] = v[2] * conj(bc); v[3] = v[3] * conj(bc);
}

static cd contract(int n, const cd* vl, const cd* mat, const cd* vr) {
  // sum(vec_l * matmul(mat, vec_r))
  cd tot = C(0);
  for (int i = 0; i < n; ++i) {
    cd w = C(0);
    for (int j = 0; j < n; ++j) w = w + mat[i + n * j] * vr[j];
    tot = tot + vl[i] * w;
  }
  return tot;
}

static void take_measurement(Chain& c, int time) {
  const int ns = c.ns, nc = c.n_cell, t = time - 1;
  const double N = (double)nc;
  std::vector<cd> g((size_t)ns * ns);
  for (int j = 0; j < ns; ++j) {
    for (int i = 0; i < ns; ++i) g[i + (size_t)ns * j] = -c.g_h[i + (size_t)ns * j];
    g[j + (size_t)ns * j] = g[j + (size_t)ns * j] + C(1.0);
  }
  cd* rec = c.meas_acc.data();
  auto F = [&](int f, int ind) -> cd& { return rec[PQMC_N_SCALAR + (size_t)f * nc + ind]; };
  const cd vx[4] = {C(-0.0, c.hop), C(-0.0, c.hop), C(0.0, -c.hop), C(0.0, -c.hop)};  // -hop*[-i,-i,i,i]
  const cd vy[4] = {C(c.hop), C(-c.hop), C(-c.hop), C(c.hop)};                          // -hop*[-1,1,1,-1]
  for (int c1 = 0; c1 < nc; ++c1) {
    int b1x = c.cell_bf[0 + 2 * c1], b1y = c.cell_bf[1 + 2 * c1];
    int c1x = c.cell_xnb[c1], c1y = c.cell_ynb[c1];
    double x1x = c.x(b1x, t), x1y = c.x(b1y, t);
    {
      cd o = C(0);
      o = o + C((0.5 * c.D) * (x1x * x1x + x1y * x1y) - c.biased * (x1x + x1y));
      o = o / N;
      rec[PQMC_OBS_BF_KE] = rec[PQMC_OBS_BF_KE] + o;
      double d1 = x1x - c.x(b1x, t + 1), d2 = x1y - c.x(b1y, t + 1);
      o = C(0);
      o = o - C(((0.5 * c.M) * (d1 * d1 + d2 * d2)) / (c.delt * c.delt));
      o = o + C((1.0 / (2.0 * c.delt)) * 2.0);
      o = o / N;
      rec[PQMC_OBS_BF_PE] = rec[PQMC_OBS_BF_PE] + o;
      o = C(0);
      o = o + C((x1x + x1y) / N);
      rec[PQMC_OBS_BF_X] = rec[PQMC_OBS_BF_X] + o;
    }
    bool cr1[2] = {c.cell_cross[0 + 2 * c1] != 0, c.cell_cross[1 + 2 * c1] != 0};
    for (int c2 = 0; c2 < nc; ++c2) {
      int c2x = c.cell_xnb[c2], c2y = c.cell_ynb[c2];
      bool cr2[2] = {c.cell_cross[0 + 2 * c2] != 0, c.cell_cross[1 + 2 * c2] != 0};
      int ind = c.rel_index[c1 + nc * c2];
      int b2x = c.cell_bf[0 + 2 * c2], b2y = c.cell_bf[1 + 2 * c2];
      double x2x = c.x(b2x, t), x2y = c.x(b2y, t);
      F(PQMC_F_BFX_BFX, ind) = F(PQMC_F_BFX_BFX, ind) + C((x1x * x2x) / N);
      F(PQMC_F_BFX_BFY, ind) = F(PQMC_F_BFX_BFY, ind) + C((x1x * x2y) / N);
      F(PQMC_F_BFY_BFY, ind) = F(PQMC_F_BFY_BFY, ind) + C((x1y * x2y) / N);
      F(PQMC_F_BFXY_BFXY, ind) = F(PQMC_F_BFXY_BFXY, ind) + C((x1x * x1y * x2x * x2y) / N);
      cd m[64], vl[8], vr[8];
      // full Wick (Hartree + Fock)
      auto cur = [&](int f, const cd* lv, int ldir, const cd* rv, int rdir, bool quirk) {
        for (int k = 0; k < 4; ++k) { vl[k] = lv[k]; vr[k] = rv[k]; }
        bphase(c, vl, cr1[ldir], ldir);
        bphase(c, vr, cr2[rdir], rdir);
        F(f, ind) = F(f, ind) + contract(4, vl, m, quirk ? vl : vr) / N;
      };
      spin_current(c, g, c1, c1x, c2, c2x, false, m);
      cur(PQMC_F_JXX_JXX, vx, 0, vx, 0, false);
      cur(PQMC_F_JXY_JXY, vy, 0, vy, 0, false);
      spin_current(c, g, c1, c1y, c2, c2y, false, m);
      cur(PQMC_F_JYX_JYX, vx, 1, vx, 1, false);
      cur(PQMC_F_JYY_JYY, vy, 1, vy, 1, true);   // mod_meas.f90:353 uses vec_l twice
      spin_current(c, g, c1, c1x, c2, c2y, false, m);
      cur(PQMC_F_JXX_JYX, vx, 0, vx, 1, false);
      cur(PQMC_F_JXY_JYY, vy, 0, vy, 1, false);
      // Hartree only :378-458
      spin_current(c, g, c1, c1x, c2, c2x, true, m);
      cur(PQMC_F_JXXH_JXXH, vx, 0, vx, 0, false);
      cur(PQMC_F_JXYH_JXYH, vy, 0, vy, 0, false);
      spin_current(c, g, c1, c1y, c2, c2y, true, m);
      cur(PQMC_F_JYXH_JYXH, vx, 1, vx, 1, false);
      cur(PQMC_F_JYYH_JYYH, vy, 1, vy, 1, true);  // :417
      spin_current(c, g, c1, c1x, c2, c2y, true, m);
      cur(PQMC_F_JXXH_JYXH, vx, 0, vx, 1, false);
      cur(PQMC_F_JXYH_JYYH, vy, 0, vy, 1, false);
      cur(PQMC_F_JXXH_JYYH, vx, 0, vy, 1, false);
      cur(PQMC_F_JXYH_JYXH, vy, 0, vx, 1, false);
      // spin momentum :463-500
      spin_momentum(c, g, c1, c2, m);
      {
        const cd dn[4] = {C(0.5), C(0), C(0), C(0.5)};
        const cd sz[4] = {C(0.5), C(0), C(0), C(-0.5)};
        const cd sx[4] = {C(0), C(0.5), C(0.5), C(0)};
        const cd sy[4] = {C(0), C(-0.0, -0.5), C(0.0, 0.5), C(0)};
        F(PQMC_F_DEN_DEN, ind) = F(PQMC_F_DEN_DEN, ind) + contract(4, dn, m, dn) / N;
        int s1u = c.cell_sites[0 + 2 * c1], s1d = c.cell_sites[1 + 2 * c1];
        int s2u = c.cell_sites[0 + 2 * c2], s2d = c.cell_sites[1 + 2 * c2];
        cd sc = c.G(s2u, s1u) * c.G(s2d, s1d) - c.G(s2d, s1u) * c.G(s2u, s1d);
        F(PQMC_F_SC_SC, ind) = F(PQMC_F_SC_SC, ind) + sc / N;
        F(PQMC_F_SZ_SZ, ind) = F(PQMC_F_SZ_SZ, ind) + contract(4, sz, m, sz) / N;
        F(PQMC_F_SX_SX, ind) = F(PQMC_F_SX_SX, ind) + contract(4, sx, m, sx) / N;
        F(PQMC_F_SY_SY, ind) = F(PQMC_F_SY_SY, ind) + contract(4, sy, m, sy) / N;
      }
      // physical currents :504-536
      auto phys = [&](int f, const cd* cv, double xl, double xr, int dir) {
        for (int k = 0; k < 4; ++k) { vl[k] = (-1.0) * cv[k]; }  // hop*[..] = -(-hop*[..])
        for (int k = 0; k < 4; ++k) vl[4 + k] = C(c.ep * xl * 1.0);
        for (int k = 0; k < 4; ++k) vr[k] = vl[k];
        for (int k = 0; k < 4; ++k) vr[4 + k] = C(c.ep * xr * 1.0);
        bphase(c, vl, cr1[dir], dir);
        bphase(c, vr, cr2[dir], dir);
        bphase(c, vl + 4, cr1[dir], dir);
        bphase(c, vr + 4, cr2[dir], dir);
        F(f, ind) = F(f, ind) + contract(8, vl, m, vr) / N;
      };
      phys_current(c, g, c1, c1y, c2, c2y, m);
      phys(PQMC_F_CJYX_CJYX, vx, x1y, x2y, 1);
      phys_current(c, g, c1, c1x, c2, c2x, m);
      phys(PQMC_F_CJXY_CJXY, vy, x1x, x2x, 0);
    }
  }
}

// begin_measure's end-of-window step + ms_k_space_obs :740-743, :546-566
static void finish_record(Chain& c, int meas_number) {
  const int nc = c.n_cell;
  const double div = (double)(2 * meas_number + 1);
  cd* rec = c.meas_acc.data();
  for (int k = 0; k < PQMC_N_SCALAR + PQMC_N_FIELD * nc; ++k) rec[k] = rec[k] / div;
  for (int f = 0; f < PQMC_N_FIELD; ++f) {
    const cd* r = rec + PQMC_N_SCALAR + (size_t)f * nc;
    cd* kd = rec + PQMC_N_SCALAR + (size_t)(PQMC_N_FIELD + f) * nc;
    std::vector<cd> acc(nc, C(0));
    for (int i = 0; i < nc; ++i)
      for (int ik = 0; ik < nc; ++ik) acc[ik] = acc[ik] + c.k_phase[ik + (size_t)nc * i] * r[i];
    for (int ik = 0; ik < nc; ++ik) kd[ik] = kd[ik] + acc[ik] / (double)nc;
  }
}

}  // namespace

// ===========================================================================
// C API of the oracle (mirrors include/pqmc_gb300.h with an oracle_ prefix)
extern "C" {

typedef struct oracle_chain oracle_chain;

int oracle_create(const pqmc_model* m, oracle_chain** out) {
  if (!m || !out || m->max_dim > PQMC_MAX_DIM || m->ns <= 0 || m->nelec <= 0 || m->nelec > m->ns ||
      m->ngroup <= 0 || m->ntime <= 0)
    return PQMC_ERR_ARG;
  Chain* c = new Chain();
  c->ns = m->ns; c->nelec = m->nelec; c->ntime = m->ntime; c->ngroup = m->ngroup;
  c->nblock = m->ntime / m->ngroup + 2;
  c->n_pf = m->n_pf; c->pdim = m->max_dim; c->max_pla = m->max_pla; c->n_bf = m->n_bf;
  c->expkv_kind = m->expkv_kind; c->ncopy = m->ncopy; c->tr_weight = m->tr_weight;
  c->metropolis = m->metropolis; c->greatest_decent = m->greatest_decent;
  c->local_update = m->local_update; c->proposal_kind = m->proposal_kind;
  c->delt = m->delt; c->M = m->mass; c->D = m->stiff; c->biased = m->biased_phonon; c->jump = m->jump_distance;
  int npf = m->n_pf, pd = m->max_dim, mp = m->max_pla;
  c->pf_dim.assign(m->pf_dim, m->pf_dim + npf);
  c->pf_npla.assign(m->pf_npla, m->pf_npla + npf);
  c->pf_k_exist.assign(m->pf_k_exist, m->pf_k_exist + npf);
  c->pf_v_exist.assign(m->pf_v_exist, m->pf_v_exist + npf);
  auto cpy = [](const double* p, size_t n) {
    std::vector<cd> v(n);
    for (size_t k = 0; k < n; ++k) v[k] = C(p[2 * k], p[2 * k + 1]);
    return v;
  };
  c->k_coe = cpy(m->pf_k_coe, npf);
  c->v_coe = cpy(m->pf_v_coe, npf);
  c->kmat = cpy(m->pf_kmat, (size_t)pd * pd * npf);
  c->vmat = cpy(m->pf_vmat, (size_t)pd * pd * npf);
  c->bc_phases = cpy(m->bc_phases, (size_t)pd * pd * mp * npf);
  c->pla_site_list.assign(m->pla_site_list, m->pla_site_list + (size_t)pd * mp * npf);
  c->bf_list.assign(m->bf_list, m->bf_list + (size_t)mp * npf);
  c->boundary_crossing.assign(m->boundary_crossing, m->boundary_crossing + (size_t)mp * npf);
  c->field.assign((size_t)c->n_bf * c->ntime, 0.0);
  size_t nkv = (size_t)pd * pd * mp * npf * c->ntime;
  c->expkv.assign(nkv, C(0));
  c->expkv_inv.assign(nkv, C(0));
  c->g_h.assign((size_t)c->ns * c->ns, C(0));
  c->q_string.assign((size_t)c->ns * c->nelec * c->nblock, C(0));
  c->d_string.assign((size_t)c->nelec * c->nblock, C(1.0));
  c->slater_q.assign((size_t)c->ns * c->nelec, C(0));
  c->slater_d.assign((size_t)c->nelec, C(1.0));
  *out = reinterpret_cast<oracle_chain*>(c);
  return PQMC_OK;
}

int oracle_destroy(oracle_chain* h) { delete reinterpret_cast<Chain*>(h); return PQMC_OK; }

int oracle_set_meas_layout(oracle_chain* h, const pqmc_meas_layout* L) {
  Chain* c = reinterpret_cast<Chain*>(h);
  int nc = L->n_cell;
  c->n_cell = nc;
  c->cell_sites.assign(L->cell_sites, L->cell_sites + 2 * nc);
  c->cell_bf.assign(L->cell_bf, L->cell_bf + 2 * nc);
  c->cell_xnb.assign(L->cell_xnb, L->cell_xnb + nc);
  c->cell_ynb.assign(L->cell_ynb, L->cell_ynb + nc);
  c->cell_cross.assign(L->cell_cross, L->cell_cross + 2 * nc);
  c->rel_index.assign(L->rel_index, L->rel_index + (size_t)nc * nc);
  c->bc_phase[0] = C(L->bc_phase[0], L->bc_phase[1]);
  c->bc_phase[1] = C(L->bc_phase[2], L->bc_phase[3]);
  c->k_phase.resize((size_t)nc * nc);
  for (size_t k = 0; k < (size_t)nc * nc; ++k) c->k_phase[k] = C(L->k_phase[2 * k], L->k_phase[2 * k + 1]);
  c->hop = L->hop;
  c->ep = L->ep_parameter;
  c->meas_acc.assign(meas_width(*c), C(0));
  c->have_meas = true;
  return PQMC_OK;
}

int oracle_set_field(oracle_chain* h, const double* f) {
  Chain* c = reinterpret_cast<Chain*>(h);
  std::memcpy(c->field.data(), f, sizeof(double) * c->field.size());
  return PQMC_OK;
}
int oracle_get_field(oracle_chain* h, double* f) {
  Chain* c = reinterpret_cast<Chain*>(h);
  std::memcpy(f, c->field.data(), sizeof(double) * c->field.size());
  return PQMC_OK;
}
int oracle_set_slater(oracle_chain* h, const double* q, const double* d) {
  Chain* c = reinterpret_cast<Chain*>(h);
  std::memcpy(c->slater_q.data(), q, sizeof(cd) * c->slater_q.size());
  std::memcpy(c->slater_d.data(), d, sizeof(cd) * c->slater_d.size());
  return PQMC_OK;
}
int oracle_get_g(oracle_chain* h, double* g) {
  Chain* c = reinterpret_cast<Chain*>(h);
  std::memcpy(g, c->g_h.data(), sizeof(cd) * c->g_h.size());
  return PQMC_OK;
}
int oracle_set_g(oracle_chain* h, const double* g) {
  Chain* c = reinterpret_cast<Chain*>(h);
  std::memcpy(c->g_h.data(), g, sizeof(cd) * c->g_h.size());
  return PQMC_OK;
}
int oracle_get_state(oracle_chain* h, pqmc_state* s) {
  Chain* c = reinterpret_cast<Chain*>(h);
  s->ln_cw[0] = c->ln_cw.re; s->ln_cw[1] = c->ln_cw.im;
  s->err_fast_max = c->err_fast_max; s->err_fast = c->err_fast;
  s->positive_accept = c->pos_acc; s->negative_accept = c->neg_acc;
  s->rng[0] = c->rng.iran; s->rng[1] = c->rng.jran; s->rng[2] = c->rng.kran;
  s->rng[3] = c->rng.mran; s->rng[4] = c->rng.nran;
  s->reserved = 0;
  return PQMC_OK;
}
int oracle_set_rng(oracle_chain* h, const int32_t* r) {
  Chain* c = reinterpret_cast<Chain*>(h);
  c->rng = Ran2{r[0], r[1], r[2], r[3], r[4]};
  return PQMC_OK;
}
int oracle_get_qd(oracle_chain* h, int blk, double* q, double* d) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (blk < 1 || blk > c->nblock) return PQMC_ERR_ARG;
  if (q) std::memcpy(q, c->Q(blk - 1), sizeof(cd) * c->ns * c->nelec);
  if (d) std::memcpy(d, c->Dv(blk - 1), sizeof(cd) * c->nelec);
  return PQMC_OK;
}
int oracle_get_expkv(oracle_chain* h, double* kv, double* kvinv) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (kv) std::memcpy(kv, c->expkv.data(), sizeof(cd) * c->expkv.size());
  if (kvinv) std::memcpy(kvinv, c->expkv_inv.data(), sizeof(cd) * c->expkv_inv.size());
  return PQMC_OK;
}
// get_expKV for one plaquette (test hook for the closed-form vs expm check)
int oracle_expkv_single(oracle_chain* h, int kind, int pf, int pla, double bf, int inv, double* out) {
  Chain* c = reinterpret_cast<Chain*>(h);
  int saved = c->expkv_kind;
  c->expkv_kind = kind;
  cd m[16];
  get_expkv(*c, pf, pla, bf, inv != 0, m);
  c->expkv_kind = saved;
  int dim = c->pf_dim[pf];
  for (int k = 0; k < dim * dim; ++k) { out[2 * k] = m[k].re; out[2 * k + 1] = m[k].im; }
  return PQMC_OK;
}
int oracle_init_expkv(oracle_chain* h) { init_expkv(*reinterpret_cast<Chain*>(h)); return PQMC_OK; }
int oracle_init_g(oracle_chain* h, int start_time) { return init_g(*reinterpret_cast<Chain*>(h), start_time); }
int oracle_update_phonon_field(oracle_chain* h, int pf_id, int time) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (pf_id < 1 || pf_id > c->n_pf || time < 1 || time > c->ntime) return PQMC_ERR_ARG;
  update_phonon_field(*c, pf_id - 1, time);
  return PQMC_OK;
}
int oracle_left_evolve_g(oracle_chain* h, int time, int pf_id, int two_way) {
  Chain* c = reinterpret_cast<Chain*>(h);
  left_evolve(*c, time, c->g_h.data(), c->ns, pf_id - 1, two_way != 0);
  return PQMC_OK;
}
int oracle_right_evolve_g(oracle_chain* h, int time, int pf_id, int two_way) {
  Chain* c = reinterpret_cast<Chain*>(h);
  right_evolve(*c, time, c->g_h.data(), c->ns, pf_id - 1, two_way != 0);
  return PQMC_OK;
}
int oracle_left_evolve(oracle_chain* h, int time, int pf_id, double* mat, int n) {
  Chain* c = reinterpret_cast<Chain*>(h);
  left_evolve(*c, time, reinterpret_cast<cd*>(mat), n, pf_id - 1, false);
  return PQMC_OK;
}
int oracle_right_evolve(oracle_chain* h, int time, int pf_id, double* mat, int n) {
  Chain* c = reinterpret_cast<Chain*>(h);
  right_evolve(*c, time, reinterpret_cast<cd*>(mat), n, pf_id - 1, false);
  return PQMC_OK;
}
int oracle_get_g_scratch(oracle_chain* h, int time, int forward, int loop, double* err) {
  return get_g_scratch(*reinterpret_cast<Chain*>(h), time, forward != 0, loop, err);
}
int oracle_cal_new_weight(oracle_chain* h, double* out) {
  cd z = C(0);
  int st = cal_new_weight(*reinterpret_cast<Chain*>(h), &z);
  if (out) { out[0] = z.re; out[1] = z.im; }
  return st;
}
int oracle_take_measurement(oracle_chain* h, int time) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (!c->have_meas) return PQMC_ERR_STATE;
  take_measurement(*c, time);
  return PQMC_OK;
}
int oracle_begin_measure(oracle_chain* h, int forward, int time, int meas_number, double* out, int* done) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (!c->have_meas) return PQMC_ERR_STATE;
  take_measurement(*c, time);
  int half = c->ntime / 2;
  bool last = (forward && time == half + meas_number) || (!forward && time == half - meas_number);
  if (done) *done = last ? 1 : 0;
  if (last) {
    finish_record(*c, meas_number);
    if (out) std::memcpy(out, c->meas_acc.data(), sizeof(cd) * c->meas_acc.size());
    std::fill(c->meas_acc.begin(), c->meas_acc.end(), C(0));
  }
  return PQMC_OK;
}
int oracle_record_width(oracle_chain* h) { return meas_width(*reinterpret_cast<Chain*>(h)); }

// The sweep loop body of src/Main_PQMC.f90:81-156 (global update excluded).
// forward alternates with loop parity: the first loop (loop=1) runs backward.
// max_slices > 0 stops after that many slices (bounded CPU-baseline samples).
int oracle_sweep_ex(oracle_chain* h, int first_loop, int n_sweeps, int warmup, int meas_interval,
                    int meas_number, double* records, int cap, int* n_rec, int max_slices) {
  Chain* c = reinterpret_cast<Chain*>(h);
  if (!c->have_g) return PQMC_ERR_STATE;
  int nrec = 0, slices = 0;
  const int W = meas_width(*c);
  for (int loop = first_loop; loop < first_loop + n_sweeps; ++loop) {
    bool forward = (loop % 2) == 0;
    for (int tc = 1; tc <= c->ntime; ++tc) {
      int time;
      if (!forward) {
        time = c->ntime - tc + 1;
        for (int pf = c->n_pf - 1; pf >= 0; --pf) {
          right_evolve(*c, time, c->g_h.data(), c->ns, pf, true);
          if (c->local_update && c->pf_v_exist[pf]) update_phonon_field(*c, pf, time);
        }
      } else {
        time = tc;
        for (int pf = 0; pf < c->n_pf; ++pf) {
          if (c->local_update && c->pf_v_exist[pf]) update_phonon_field(*c, pf, time);
          left_evolve(*c, time, c->g_h.data(), c->ns, pf, true);
        }
      }
      if (tc % c->ngroup == 0) {
        int st = get_g_scratch(*c, forward ? time + 1 : time, forward, loop, nullptr);
        if (st) return st;
      }
      if (c->have_meas && loop > warmup && ((loop - warmup) % meas_interval) == 0) {
        int half = c->ntime / 2;
        if (time >= half - meas_number && time <= half + meas_number) {
          int done = 0;
          double* out = (records && nrec < cap) ? records + (size_t)2 * W * nrec : nullptr;
          oracle_begin_measure(h, forward ? 1 : 0, time, meas_number, out, &done);
          if (done) nrec++;
        }
      }
      if (max_slices > 0 && ++slices >= max_slices) { if (n_rec) *n_rec = nrec; return PQMC_OK; }
    }
  }
  if (n_rec) *n_rec = nrec;
  return PQMC_OK;
}

int oracle_sweep(oracle_chain* h, int first_loop, int n_sweeps, int warmup, int meas_interval,
                 int meas_number, double* records, int cap, int* n_rec) {
  return oracle_sweep_ex(h, first_loop, n_sweeps, warmup, meas_interval, meas_number, records, cap,
                         n_rec, 0);
}

// Runs `n` independent copies of the same prepared chain on `threads` host
// threads for `max_slices` slices each; returns wall seconds.  This is the
// CPU baseline: one chain per core as in the reference's MPI layout
// (src/Main_PQMC.f90:373-443).
double oracle_time_parallel(oracle_chain* proto, int n, int threads, int first_loop, int max_slices) {
  Chain* p = reinterpret_cast<Chain*>(proto);
  std::vector<Chain*> cs(n);
  for (int i = 0; i < n; ++i) cs[i] = new Chain(*p);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (int w = 0; w < threads; ++w)
    th.emplace_back([&, w]() {
      for (int i = w; i < n; i += threads)
        oracle_sweep_ex(reinterpret_cast<oracle_chain*>(cs[i]), first_loop, 1, 1 << 30, 1, 0, nullptr, 0,
                        nullptr, max_slices);
    });
  for (auto& t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  for (auto* c : cs) delete c;
  return std::chrono::duration<double>(t1 - t0).count();
}

// ran2 helpers (test hooks): init_rng_by_seed semantics and raw draws
void oracle_rng_seed_words(int seed, int32_t* out) {
  // ran_seed(put=seed): all five words = seed, then nonnegativity / nonzero
  // enforcement of mod_ranstate.f90:119-122
  for (int k = 0; k < 5; ++k) out[k] = seed;
  for (int k = 0; k < 3; ++k) if (out[k] < 0) out[k] = ~out[k];
  for (int k = 3; k < 5; ++k) if (out[k] == 0) out[k] = 1;
}
// the fixed-order Box-Muller pieces (log u1, cos 2 pi u2, jump of width 1)
void oracle_gauss_parts(const double* u1, const double* u2, int n, double* out) {
  for (int i = 0; i < n; ++i) {
    out[3 * i] = pqmc_bm_log(u1[i]);
    out[3 * i + 1] = pqmc_bm_cos2pi(u2[i]);
    out[3 * i + 2] = pqmc_bm_gauss_jump(1.0, u1[i], u2[i]);
  }
}

void oracle_rng_draw(int32_t* state, int n, float* out) {
  Ran2 r{state[0], state[1], state[2], state[3], state[4]};
  for (int k = 0; k < n; ++k) out[k] = r.next();
  state[0] = r.iran; state[1] = r.jran; state[2] = r.kran; state[3] = r.mran; state[4] = r.nran;
}
// dense kernels exposed for unit tests
int oracle_qdr(int m, int n, double* a, double* d) {
  zqdr_(m, n, reinterpret_cast<cd*>(a), reinterpret_cast<cd*>(d));
  return 0;
}
int oracle_ldq(int m, int n, double* a, double* d) {
  zldq_(m, n, reinterpret_cast<cd*>(a), reinterpret_cast<cd*>(d));
  return 0;
}
int oracle_det_small(int n, const double* a, double* out) {
  cd z = det_small(n, reinterpret_cast<const cd*>(a));
  out[0] = z.re; out[1] = z.im;
  return 0;
}
int oracle_inverse(int n, double* a) { return zinverse_(n, reinterpret_cast<cd*>(a)); }
int oracle_expm(int n, double* a) { zexpm_(n, reinterpret_cast<cd*>(a)); return 0; }

}  // extern "C"
