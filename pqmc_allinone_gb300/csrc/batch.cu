// batch.cu -- many independent chains in one device context (replica
// parallelism of src/Main_PQMC.f90:373-443 without MPI), advanced together
// one family step at a time.
//
// Mixed-precision family step (one launch per phase for all chains):
//   k_bdraw   ran2 stream of every chain for the step
//   k_bprep   per-plaquette proposal data (as phase 1 of k_update)
//   k_bscan   one CTA per chain walks its plaquettes in Markov order; an
//             accepted move appends a rank-dim column block to the FP32
//             delayed-update panels A (Ns x K) and B (K x Ns), so later
//             ratios see G + A B without touching G (delayed updates)
//   k_bflush  G += A B for every chain: split-BF16 tensor-core products
//             (3 bf16 terms per operand, 6 cross products) accumulated in
//             FP32, added to the FP64 G
//   k_bwrap   two-way wrap G <- A G B by the family: the FP32 correction
//             (A-I)(G B) + G (B-I) added to the FP64 G
// FP64 stays in G itself, in the 4x4 ratio / T = Delta R^-1 of accepted
// moves, and in the stabilised recompute and log-weight.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <functional>
#include <deque>
#include <string>
#include <thread>
#include <vector>
#include "chain.cuh"
#include "linalg.cuh"
#include "rng.cuh"
#include "update_dev.cuh"
#include "recompute_b.cuh"
#include "df32.cuh"
#include "tc.cuh"
#include "exact.cuh"

namespace pqmc {

struct BDesc {
  DevModel M;
  double* field;
  cplx* expkv;
  cplx* expkv_inv;
  cplx* g;       // parity 0 buffer
  cplx* g_alt;   // parity 1 buffer
  float2* A;     // (kmax, ldp): A[q*ldp + r]
  float2* B;     // (kmax, ldp): B[q*ldp + c]
  int kmax;
  int ldp;       // panel leading dimension: Ns rounded up to even (16-byte columns)
  int* err;      // batch-wide error word (PQMC_ERR_* of a device-side failure)
  PlaqPre* pre;
  DevScalars* sc;
  int* kcount;
  // TMA tensor maps over the two G buffers (double-float, Ns rows x Ns
  // columns, a row read as nrb boxes of rb columns)
  const CUtensorMap* tm_g;
  const CUtensorMap* tm_galt;
  int rb, nrb;
  int t;         // 0-based time index of the slice in progress (k_bsettime)
  unsigned long long* nflush;   // flush rounds with work (for the roofline accounting)
  // the round's accepted moves for the exact update (exact.cuh)
  int* acc_site;
  float4* acc_delta;
  // scan profile while phase timing is on: SM cycles of the chain's scan
  // CTA, accepted moves, rejected proposals
  unsigned long long* scan_prof;
};

// ---------------------------------------------------------------------------
// the ran2 draws of n_fam family steps in sweep order (family pf_first,
// then pf_first + pf_step, ...), each family's proposals into its own part
// of the proposal records; families without a local update draw nothing
__global__ void k_bdraw(const BDesc* D, int C, int pf_first, int pf_step, int n_fam) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const BDesc d = D[c];
  Ran2Dev rng;
  rng.iran = d.sc->rng[0]; rng.jran = d.sc->rng[1]; rng.kran = d.sc->rng[2];
  rng.mran = d.sc->rng[3]; rng.nran = d.sc->rng[4];
  for (int q = 0; q < n_fam; ++q) {
    const int pf = pf_first + q * pf_step;
    if (!d.M.pf_v_exist[pf]) continue;
    const int npla = d.M.pf_npla[pf];
    PlaqPre* pre = d.pre + (size_t)pf * d.M.max_pla;
    for (int p = 0; p < npla; ++p) {
      if (d.M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
        pre[p].xnew = (double)rng.next();
        pre[p].dE = (double)rng.next();
      } else {
        pre[p].xnew = (double)rng.ran_sysm();
      }
      pre[p].r = (double)rng.next();
    }
  }
  d.sc->rng[0] = rng.iran; d.sc->rng[1] = rng.jran; d.sc->rng[2] = rng.kran;
  d.sc->rng[3] = rng.mran; d.sc->rng[4] = rng.nran;
}

__device__ __forceinline__ double b_threshold(const DevModel& M, double dE, double r) {
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

// the slice every chain of a group works on; kept on the device so that one
// captured graph of a slice's launches serves every time index
__global__ void k_bsettime(BDesc* D, int C, int t) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) D[c].t = t;
}

// proposals of families pf_first .. (bpf blocks of PREP_PLA plaquettes per
// family), each into the family's part of the records.  The per-plaquette
// scalars (jump, action change, threshold, the closed-form norm and its
// cosh/sinh) are formed one plaquette per lane of warp 0, the 4x4 blocks
// (new propagators, Delta) by 16 lanes per plaquette: on GB300 every FP64
// warp instruction costs the same whatever its active lanes, so the scalar
// part is spread across lanes instead of repeated per plaquette.
constexpr int PREP_PLA = 16;
__global__ void __launch_bounds__(256) k_bprep(const BDesc* D, int pf_first, int bpf) {
  __shared__ BDesc sd;
  __shared__ double s_x[PREP_PLA], s_norm[PREP_PLA], s_ch[PREP_PLA], s_sh[PREP_PLA];
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const BDesc& d = sd;
  const int t = d.t;
  const DevModel& M = d.M;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pf = pf_first + (int)blockIdx.x / bpf;
  const int npla = M.pf_npla[pf], dim = M.pf_dim[pf], pd = M.pdim;
  const int p0 = ((int)blockIdx.x % bpf) * PREP_PLA;
  if (p0 >= npla || !M.pf_v_exist[pf]) return;
  PlaqPre* pre = d.pre + (size_t)pf * M.max_pla;
  const double* field = d.field;
  const bool closed = (M.expkv_kind != PQMC_EXPKV_GENERAL);
  // ---- scalars: one plaquette per lane ------------------------------------
  if (warp == 0 && lane < PREP_PLA && p0 + lane < npla) {
    const int p = p0 + lane;
    const int b = M.bf[p + M.max_pla * pf];
    double jump;
    if (M.proposal_kind == PQMC_PROPOSAL_GAUSSIAN) {
      double u1 = pre[p].xnew, u2 = pre[p].dE;
      jump = pqmc_bm_gauss_jump(M.jump, u1, u2);   // bit-identical with the oracle
    } else {
      jump = M.jump * pre[p].xnew;
    }
    const double xnew = field[b + (size_t)M.n_bf * t] + jump;
    const double dE = -M.delt * energy_diff(M, field, b, t, jump);
    pre[p].dE = dE;
    pre[p].thr = b_threshold(M, dE, pre[p].r);
    pre[p].xnew = xnew;
    s_x[lane] = xnew;
    if (closed) {
      const double norm = closed_norm(M, pf, xnew);
      s_norm[lane] = norm;
      s_ch[lane] = cosh(norm);
      s_sh[lane] = sinh(norm);
    } else {
      dev_get_expkv(M, pf, p, xnew, false, pre[p].enew);
      dev_get_expkv(M, pf, p, xnew, true, pre[p].einv);
    }
  }
  __syncthreads();
  // ---- 4x4 blocks: 16 lanes per plaquette, two plaquettes per warp ---------
  const int h = lane >> 4, sl = lane & 15, q = 2 * warp + h, p = p0 + q;
  const bool valid = q < PREP_PLA && p < npla;
  const int i = sl % dim, j = sl / dim;
  const bool act = valid && sl < dim * dim;
  cplx en = mk(0.0);
  if (act) {
    if (closed) {
      const double xnew = s_x[q], norm = s_norm[q], ch = s_ch[q], sh = s_sh[q];
      en = closed_entry(M, pf, p, xnew, false, i, j, norm, ch, sh);
      pre[p].enew[sl] = en;
      pre[p].einv[sl] = closed_entry(M, pf, p, xnew, true, i, j, norm, ch, sh);
    } else {
      en = pre[p].enew[sl];
    }
  }
  __syncwarp();
  // Delta = expKV_inv(old) expKV(new) - I   (mod_update.f90:240-243)
  const size_t base = valid ? M.kv_base(p, pf, t) : 0;
  cplx a = mk(0.0);
  for (int k = 0; k < dim; ++k) {
    const cplx ekj = shfl_c(en, 16 * h + k + dim * j);
    if (act) a = cadd(a, cmul(d.expkv_inv[base + i + pd * k], ekj));
  }
  if (act) {
    if (i == j) a = csub(a, mk(1.0));
    pre[p].delta[sl] = a;
    pre[p].deltaf[sl] = make_float2((float)a.x, (float)a.y);
    pre[p].deltad[sl] = dg_make(a);
  }
}

// ---------------------------------------------------------------------------
// Sequential scan with delayed updates, one CTA per chain.  The scan resumes
// at the chain's next plaquette and stops when the panels hold `kd` columns
// (the delay depth); k_bflush then folds them into G and the next round
// continues.  Ratios, R^-1 and T are FP32 (the panels are FP32); the weight
// ln_cw is accumulated in FP64.
//
// Latency design: at the start of a round (panels empty) the kernel stages
// the family's site table, the FP32 Delta and thresholds, and
// Geff(S_p,S_p) = G(S_p,S_p) for every plaquette still to come in shared
// memory.  Every warp evaluates each ratio redundantly from shared memory,
// so a rejected proposal costs no block barrier and no global access.  An
// accepted move builds its rank-dim panel block (one pass over the panels)
// and adds its contribution to the cached Geff blocks of the later
// plaquettes.
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_KSTAGE = 512;   // max delay depth (panel columns)

constexpr int SCAN_NSTAGE = 3;   // panel chunks in flight
constexpr int SCAN_RPT = 2;      // rows per thread: Ns <= SCAN_RPT * SCAN_THREADS

__host__ __device__ __forceinline__ size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }

// dynamic shared memory of k_bscan (byte offsets, 16-byte aligned pieces)
struct ScanLayout {
  size_t rows, stage, delta, geff, newA, newB, thr, site, accp, accd, total;
};
// rows first: the TMA tile destination wants a 128-byte aligned address
__host__ __device__ __forceinline__ ScanLayout scan_layout(int npla, int ns, int ldp, int qc, int kd, int rows_bytes) {
  ScanLayout L;
  size_t o = 0;
  L.rows = o;  o += (size_t)((rows_bytes + 127) & ~127);
  L.stage = o; o += al16(sizeof(float2) * (size_t)SCAN_NSTAGE * 2 * qc * ldp);
  L.delta = o; o += al16(sizeof(float2) * 16 * (size_t)npla);
  L.geff = o;  o += al16(sizeof(float2) * 16 * (size_t)npla);
  L.newA = o;  o += al16(sizeof(float2) * 4 * (size_t)ns);
  L.newB = o;  o += al16(sizeof(float2) * 4 * (size_t)ns);
  L.thr = o;   o += al16(sizeof(double) * (size_t)npla);
  L.site = o;  o += al16(sizeof(int) * 4 * (size_t)npla);
  L.accp = o;  o += al16(sizeof(int) * (size_t)kd);
  L.accd = o;  o += al16(sizeof(float2) * (size_t)kd);
  L.total = o;
  return L;
}

// thread 0: stream panel columns [c*qc, c*qc+nq) of A and B into stage c % NSTAGE
__device__ __forceinline__ void scan_issue(float2* s_stage, uint64_t* s_full, const float2* A, const float2* B,
                                           int ldp, int qc, int K, int c) {
  const int st = c % SCAN_NSTAGE, q0 = c * qc, nq = min(qc, K - q0);
  const uint32_t bytes = (uint32_t)(sizeof(float2) * (size_t)nq * ldp);
  float2* dA = s_stage + (size_t)st * 2 * qc * ldp;
  float2* dB = dA + (size_t)qc * ldp;
  mbar_arrive_tx(&s_full[st], 2 * bytes);
  bulk_g2s(dA, A + (size_t)q0 * ldp, bytes, &s_full[st]);
  bulk_g2s(dB, B + (size_t)q0 * ldp, bytes, &s_full[st]);
}

template <int DIM, int RPT>
__global__ void __launch_bounds__(SCAN_THREADS) k_bscan(const BDesc* D, int pf, int parity, int kd, int qc,
                                                         int* next_p, int exact, int prof) {
  const long long t_start = prof ? clock64() : 0;
  constexpr int NW = SCAN_THREADS / 32;
  __shared__ BDesc sd;
  __shared__ float2 s_R[NW][16];
  __shared__ float2 s_T[16];
  __shared__ float2 s_det[NW];
  __shared__ int s_dec[NW];
  __shared__ __align__(8) uint64_t s_full[SCAN_NSTAGE];
  __shared__ __align__(8) uint64_t s_rowbar;
  __shared__ int s_abort;
  extern __shared__ __align__(1024) unsigned char s_dyn[];
  if (threadIdx.x == 0) {
    sd = D[blockIdx.x];
    s_abort = 0;
    for (int k = 0; k < SCAN_NSTAGE; ++k) mbar_init(&s_full[k], 1);
    mbar_init(&s_rowbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const BDesc& d = sd;
  const DevModel& M = d.M;
  const int t = d.t;
  constexpr int dim = DIM, dd = DIM * DIM;
  const int ns = M.ns, npla = M.pf_npla[pf], pd = M.pdim, ldp = d.ldp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p0 = next_p[blockIdx.x];
  // the thread that drives the copy engine: lane 0 of the last warp when that
  // warp holds no row of G (its issue cost stays off the row workers' path)
  if (p0 >= npla) {
    if (tid == 0) *d.kcount = 0;
    return;
  }
  const int rb = d.rb, nrb = d.nrb;
  const int io = (ns <= SCAN_THREADS - 32) ? SCAN_THREADS - 32 : 0;
  const bool row_warp = warp * 32 < ns;   // holds a row of G (every warp when RPT = 2)
  // a warp with no row of G that is not the copy-engine warp
  const int inv_warp = (RPT == 1 && ns <= SCAN_THREADS - 64) ? SCAN_THREADS / 32 - 2 : -1;
  const ScanLayout L = scan_layout(npla, ns, ldp, qc, kd, 4 * nrb * rb * (int)sizeof(float4));
  float4* s_rows = reinterpret_cast<float4*>(s_dyn + L.rows);     // [dim][nrb*rb] rows of G at S
  float2* s_stage = reinterpret_cast<float2*>(s_dyn + L.stage);
  float2* s_delta = reinterpret_cast<float2*>(s_dyn + L.delta);   // [npla][16]
  float2* s_geff = reinterpret_cast<float2*>(s_dyn + L.geff);     // [npla][16]
  float2* s_newA = reinterpret_cast<float2*>(s_dyn + L.newA);     // [4][ns]
  float2* s_newB = reinterpret_cast<float2*>(s_dyn + L.newB);     // [4][ns]
  double* s_thr = reinterpret_cast<double*>(s_dyn + L.thr);
  int* s_site = reinterpret_cast<int*>(s_dyn + L.site);           // [npla][4]
  int* s_accp = reinterpret_cast<int*>(s_dyn + L.accp);
  float2* s_accd = reinterpret_cast<float2*>(s_dyn + L.accd);
  const float4* G = reinterpret_cast<const float4*>(parity ? d.g_alt : d.g);   // double-float G
  const CUtensorMap* tmG = parity ? d.tm_galt : d.tm_g;
  float2* A = d.A;
  float2* B = d.B;
  const PlaqPre* pre = d.pre + (size_t)pf * M.max_pla;
  // ---- stage the rest of the family (panels are empty: Geff = G) ----------
  for (int e = tid; e < (npla - p0) * 4; e += blockDim.x) {
    const int p = p0 + e / 4, m = e % 4;
    s_site[4 * p + m] = m < dim ? M.site[m + pd * (p + M.max_pla * pf)] : 0;
  }
  for (int p = p0 + tid; p < npla; p += blockDim.x) s_thr[p] = pre[p].thr;
  for (int e = tid; e < (npla - p0) * 16; e += blockDim.x) {
    const int p = p0 + e / 16, k = e % 16;
    if (k < dd) s_delta[16 * p + k] = pre[p].deltaf[k];
  }
  __syncthreads();
  for (int e = tid; e < (npla - p0) * 16; e += blockDim.x) {
    const int p = p0 + e / 16, k = e % 16;
    if (k < dd) s_geff[16 * p + k] = dg_f2(G[s_site[4 * p + k % dim] + (size_t)ns * s_site[4 * p + k / dim]]);
  }
  __syncthreads();
  int K = 0, n_acc = 0;
  long long na = 0;
  uint32_t phase = 0;   // bit s: parity of the next completion of stage s
  uint32_t rowphase = 0;
  int npre = 0;         // panel chunks already in flight for the next accepted move
  bool aborted = false;
  int p = p0;
  const int i = lane % dim, j = lane / dim;
  const bool act = lane < dd;
  while (p < npla && K + dim <= kd) {
    // ---- ratios of the next NW proposals, one warp each, from the cached
    //      Geff (valid for every proposal up to the first accepted one) ------
    {
      const int pw = p + warp;
      int dec = 0;
      float2 det = make_float2(0.f, 0.f);
      if (pw < npla) {
        const float2* ge = s_geff + 16 * pw;
        const float2* de = s_delta + 16 * pw;
        if (act) {
          float2 a = make_float2(i == j ? 1.f : 0.f, 0.f);
#pragma unroll
          for (int k = 0; k < dim; ++k) a = fcfma(ge[i + dim * k], de[k + dim * j], a);
          s_R[warp][lane] = a;
        }
        __syncwarp();
        det = wf_det(dim, s_R[warp], lane);
        const float dm = det.x * det.x + det.y * det.y;
        dec = ((double)dm >= s_thr[pw]) ? 1 : 0;
      }
      if (lane == 0) {
        s_dec[warp] = dec;
        s_det[warp] = det;
      }
    }
    __syncthreads();
    int wa = -1;
    for (int w = 0; w < NW && p + w < npla; ++w)
      if (s_dec[w]) { wa = w; break; }
    if (wa < 0) {   // all evaluated proposals rejected
      const int nrej = min(NW, npla - p);
      if (tid == 0) na += nrej;
      p += nrej;
      __syncthreads();   // s_dec / s_R are rewritten by the next pass
      continue;
    }
    if (tid == 0) na += wa;
    p += wa;
    // ---- accepted move p: T = Delta R^-1, by a warp without rows of G when
    //      there is one (its work then overlaps the row warps' panel loop),
    //      else by the warp that evaluated the move -------------------------
    const float2 det = s_det[wa];
    if (warp == (inv_warp >= 0 ? inv_warp : wa)) {
      wf_inverse(dim, s_R[wa], det, lane);
      if (act) {
        const float2* de = s_delta + 16 * p;
        float2 a = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < dim; ++k) a = fcfma(de[i + dim * k], s_R[wa][k + dim * j], a);
        s_T[lane] = a;
      }
      if (lane == 0) {
        s_accp[n_acc] = p;
        s_accd[n_acc] = det;
      }
    }
    ++n_acc;
    const int* S = s_site + 4 * p;
    const int nch = (K + qc - 1) / qc;
    if (tid == io) {
      // rows G(S_m, :) by the tensor engine (strided: one 16-byte element per column)
      mbar_arrive_tx(&s_rowbar, (uint32_t)(dim * nrb * rb * sizeof(float4)));
      for (int m = 0; m < dim; ++m)
        for (int bx = 0; bx < nrb; ++bx) tma_load_2d(s_rows + (size_t)(m * nrb + bx) * rb, tmG, 4 * S[m], bx * rb, &s_rowbar);
      if (nch > npre) {
        if (npre == 0) fence_proxy_async_global();   // this round's panel columns were written by generic stores
        for (int c = npre; c < nch && c < SCAN_NSTAGE; ++c) scan_issue(s_stage, s_full, A, B, ldp, qc, K, c);
      }
    }
    npre = 0;
    // rows of G at the accepted sites, loaded now and added after the panel
    // loop (their latency overlaps it)
    float4 gcol[RPT][dim];
    float2 gm[RPT][dim], bl[RPT][dim];
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int r = tid + k * SCAN_THREADS;
#pragma unroll
      for (int m = 0; m < dim; ++m) {
        gcol[k][m] = r < ns ? G[r + (size_t)ns * S[m]] : make_float4(0.f, 0.f, 0.f, 0.f);
        gm[k][m] = make_float2(0.f, 0.f);
        bl[k][m] = make_float2(0.f, 0.f);
      }
    }
    for (int c = 0; c < nch; ++c) {
      const int st = c % SCAN_NSTAGE;
      if (!mbar_wait_bounded(&s_full[st], (phase >> st) & 1u)) s_abort = 1;
      phase ^= 1u << st;
      const float2* cA = s_stage + (size_t)st * 2 * qc * ldp;
      const float2* cB = cA + (size_t)qc * ldp;
      // warps without a row of G skip the column loop: the broadcast loads
      // of the accepted sites' panel entries are its shared-memory bound
      const int nq = row_warp ? min(qc, K - c * qc) : 0;
#pragma unroll 2
      for (int qq = 0; qq < nq; ++qq) {
        float2 bs[dim], as[dim];
#pragma unroll
        for (int m = 0; m < dim; ++m) {
          bs[m] = cB[(size_t)qq * ldp + S[m]];
          as[m] = cA[(size_t)qq * ldp + S[m]];
        }
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
          const int r = tid + k * SCAN_THREADS;
          if (r < ns) {
            const float2 ar = cA[(size_t)qq * ldp + r], bc = cB[(size_t)qq * ldp + r];
#pragma unroll
            for (int m = 0; m < dim; ++m) {
              gm[k][m] = fcfma(ar, bs[m], gm[k][m]);
              bl[k][m] = fcfma(as[m], bc, bl[k][m]);
            }
          }
        }
      }
      __syncthreads();
      if (s_abort) break;
      if (tid == io && c + SCAN_NSTAGE < nch) scan_issue(s_stage, s_full, A, B, ldp, qc, K, c + SCAN_NSTAGE);
    }
    if (s_abort) {
      aborted = true;
      break;
    }
    if (nch == 0) __syncthreads();   // s_T visible
    if (!mbar_wait_bounded(&s_rowbar, rowphase)) s_abort = 1;   // checked after the next barrier
    rowphase ^= 1u;
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int r = tid + k * SCAN_THREADS;
      if (r >= ns) continue;
#pragma unroll
      for (int m = 0; m < dim; ++m) {
        gm[k][m] = fa(gm[k][m], dg_f2(gcol[k][m]));
        bl[k][m] = fa(bl[k][m], dg_f2(s_rows[(size_t)m * nrb * rb + r]));
      }
#pragma unroll
      for (int l = 0; l < dim; ++l) {
        float2 a = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 0; m < dim; ++m) a = fcfma(gm[k][m], s_T[m + dim * l], a);
        float2 bv = make_float2(-bl[k][l].x, -bl[k][l].y);
        if (r == S[l]) bv.x += 1.f;
        A[(size_t)(K + l) * ldp + r] = a;
        B[(size_t)(K + l) * ldp + r] = bv;
        s_newA[(size_t)l * ns + r] = a;
        s_newB[(size_t)l * ns + r] = bv;
      }
    }
    __syncthreads();
    if (s_abort) {
      aborted = true;
      break;
    }
    // ---- the new block's contribution to the cached Geff of later plaquettes
    for (int e = tid; e < (npla - p - 1) * dd; e += blockDim.x) {
      const int pq = p + 1 + e / dd, k = e % dd;
      const int si = s_site[4 * pq + k % dim], sj = s_site[4 * pq + k / dim];
      float2 a = s_geff[16 * pq + k];
#pragma unroll
      for (int l = 0; l < dim; ++l) a = fcfma(s_newA[(size_t)l * ns + si], s_newB[(size_t)l * ns + sj], a);
      s_geff[16 * pq + k] = a;
    }
    K += dim;
    ++p;
    __syncthreads();
    // the next accepted move of this round streams columns [0, K): start it now
    if (p < npla && K + dim <= kd) {
      npre = min((K + qc - 1) / qc, SCAN_NSTAGE);
      if (tid == io) {
        fence_proxy_async_global();
        for (int c = 0; c < npre; ++c) scan_issue(s_stage, s_full, A, B, ldp, qc, K, c);
      }
    }
  }
  // chunks started for an accepted move that did not come: drain them
  if (!aborted && npre > 0) {
    for (int c = 0; c < npre; ++c) {
      if (!mbar_wait_bounded(&s_full[c], (phase >> c) & 1u)) s_abort = 1;
      phase ^= 1u << c;
    }
    __syncthreads();
    aborted = s_abort != 0;
  }
  if (aborted) {
    // a panel chunk never arrived: give the copies still in flight a bounded
    // wait, flag the chain and stop (the host reports PQMC_ERR_TIMEOUT)
    if (tid == io) {
      for (int st = 0; st < SCAN_NSTAGE; ++st) mbar_wait_bounded(&s_full[st], (phase >> st) & 1u);
      mbar_wait_bounded(&s_rowbar, rowphase);
      d.sc->status = PQMC_ERR_TIMEOUT;
      atomicExch(d.err, PQMC_ERR_TIMEOUT);
      *d.kcount = 0;
      next_p[blockIdx.x] = npla;
    }
    return;
  }
  __syncthreads();
  // ---- bookkeeping of the round's accepted moves (field, expKV, ln_cw) -----
  for (int e = tid; e < n_acc * pd * pd; e += blockDim.x) {
    const int ja = e / (pd * pd), k = e % (pd * pd);
    const int pa_ = s_accp[ja], ii = k % pd, jj = k / pd;
    const bool in = ii < dim && jj < dim;
    const size_t base2 = M.kv_base(pa_, pf, t);
    d.expkv[base2 + k] = in ? pre[pa_].enew[ii + dim * jj] : mk(0.0);
    d.expkv_inv[base2 + k] = in ? pre[pa_].einv[ii + dim * jj] : mk(0.0);
  }
  for (int ja = tid; ja < n_acc; ja += blockDim.x) {
    const int pa_ = s_accp[ja];
    d.field[M.bf[pa_ + M.max_pla * pf] + (size_t)M.n_bf * t] = pre[pa_].xnew;
  }
  if (exact) {   // the accepted moves for the exact update: sites and Delta
    for (int e = tid; e < n_acc * dim; e += blockDim.x) d.acc_site[e] = s_site[4 * s_accp[e / dim] + e % dim];
    for (int e = tid; e < n_acc * 16; e += blockDim.x) d.acc_delta[e] = pre[s_accp[e / 16]].deltad[e % 16];
  }
  if (warp == 0) {
    // ln_cw += log prod_j Re(R_j^ncopy) (|R_j|^2 under TR_weight), as a
    // mantissa/exponent product so long rounds cannot overflow
    double mant = 1.0;
    long long ex = 0;
    for (int ja = lane; ja < n_acc; ja += 32) {
      const double dr = s_accd[ja].x, di = s_accd[ja].y;
      double rr = dr, ri = di;
      if (M.tr_weight) { rr = dr * dr + di * di; ri = 0.0; }
      double ar = 1.0, ai = 0.0;
      for (int k = 0; k < M.ncopy; ++k) {
        const double tr = ar * rr - ai * ri;
        ai = ar * ri + ai * rr;
        ar = tr;
      }
      int e2;
      mant *= frexp(ar, &e2);
      ex += e2;
      mant = frexp(mant, &e2);
      ex += e2;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double om = __shfl_down_sync(0xffffffffu, mant, o);
      const long long oe = __shfl_down_sync(0xffffffffu, ex, o);
      if (lane + o < 32) {
        int e2;
        mant = frexp(mant * om, &e2);
        ex += oe + e2;
      }
    }
    if (lane == 0) {
      *d.kcount = K;
      next_p[blockIdx.x] = p;
      if (n_acc > 0) {
        const double l = (mant > 0.0) ? log(mant) + (double)ex * 0.69314718055994530942 : log(mant);
        d.sc->ln_cw = cadd(d.sc->ln_cw, mk(l));
      }
      d.sc->pos_acc += n_acc;
      d.sc->neg_acc += na;
      if (prof) {
        atomicAdd(d.scan_prof, (unsigned long long)(clock64() - t_start));
        atomicAdd(d.scan_prof + 1, (unsigned long long)n_acc);
        atomicAdd(d.scan_prof + 2, (unsigned long long)na);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// G += A B with split-BF16 tensor-core products (mma.sync m16n8k16, FP32
// accumulators), 64x64 complex output tile per CTA, 8 warps of 16x32.
constexpr int FB_M = 64, FB_N = 64, FB_K = 16, FB_LD = 24;

__device__ __forceinline__ void split3(float x, __nv_bfloat16* o) {
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  float r1 = x - __bfloat162float(h);
  __nv_bfloat16 m = __float2bfloat16_rn(r1);
  float r2 = r1 - __bfloat162float(m);
  o[0] = h;
  o[1] = m;
  o[2] = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(256) k_bflush(const BDesc* D, int parity) {
  __shared__ BDesc sd;
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const BDesc& d = sd;
  const int K = *d.kcount;
  if (K == 0) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.nflush, 1ull);
  const int ns = d.M.ns;
  const int tiles_m = (ns + FB_M - 1) / FB_M, tiles_n = (ns + FB_N - 1) / FB_N;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  if (tn >= tiles_n) return;
  float4* G = reinterpret_cast<float4*>(parity ? d.g_alt : d.g);   // double-float G
  // As[split][comp re,im][m][k], Bs[split][comp re,im,-im][n][k]
  __shared__ __align__(16) __nv_bfloat16 As[3][2][FB_M][FB_LD];
  __shared__ __align__(16) __nv_bfloat16 Bs[3][3][FB_N][FB_LD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;   // 4 x 2 warps
  const int g = lane >> 2, tq = lane & 3;
  float acc[4][2][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 2; ++b)
      for (int e = 0; e < 4; ++e) acc[a][b][e] = 0.f;
  const int row0 = tm * FB_M, col0 = tn * FB_N;
  for (int k0 = 0; k0 < K; k0 += FB_K) {
    for (int e = tid; e < FB_M * FB_K; e += 256) {
      int r = e % FB_M, q = e / FB_M;
      float2 v = make_float2(0.f, 0.f);
      if (row0 + r < ns && k0 + q < K) v = d.A[(size_t)(k0 + q) * d.ldp + row0 + r];
      __nv_bfloat16 sp[3];
      split3(v.x, sp);
      As[0][0][r][q] = sp[0]; As[1][0][r][q] = sp[1]; As[2][0][r][q] = sp[2];
      split3(v.y, sp);
      As[0][1][r][q] = sp[0]; As[1][1][r][q] = sp[1]; As[2][1][r][q] = sp[2];
    }
    for (int e = tid; e < FB_N * FB_K; e += 256) {
      int cix = e % FB_N, q = e / FB_N;
      float2 v = make_float2(0.f, 0.f);
      if (col0 + cix < ns && k0 + q < K) v = d.B[(size_t)(k0 + q) * d.ldp + col0 + cix];
      __nv_bfloat16 sp[3];
      split3(v.x, sp);
      Bs[0][0][cix][q] = sp[0]; Bs[1][0][cix][q] = sp[1]; Bs[2][0][cix][q] = sp[2];
      split3(v.y, sp);
      Bs[0][1][cix][q] = sp[0]; Bs[1][1][cix][q] = sp[1]; Bs[2][1][cix][q] = sp[2];
      Bs[0][2][cix][q] = __hneg(sp[0]); Bs[1][2][cix][q] = __hneg(sp[1]); Bs[2][2][cix][q] = __hneg(sp[2]);
    }
    __syncthreads();
    uint32_t af[3][2][4];
    const int mr = wm * 16;
    for (int s = 0; s < 3; ++s)
      for (int cpt = 0; cpt < 2; ++cpt) {
        af[s][cpt][0] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g][2 * tq]);
        af[s][cpt][1] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g + 8][2 * tq]);
        af[s][cpt][2] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g][2 * tq + 8]);
        af[s][cpt][3] = *reinterpret_cast<const uint32_t*>(&As[s][cpt][mr + g + 8][2 * tq + 8]);
      }
    const int SA[6] = {0, 0, 1, 0, 1, 2}, SB[6] = {0, 1, 0, 2, 1, 0};
    for (int nt = 0; nt < 4; ++nt) {
      const int nc = wn * 32 + nt * 8 + g;
      for (int pr = 0; pr < 6; ++pr) {
        const int sa = SA[pr], sb = SB[pr];
        uint32_t br[2], bi[2], bni[2];
        br[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][0][nc][2 * tq]);
        br[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][0][nc][2 * tq + 8]);
        bi[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][1][nc][2 * tq]);
        bi[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][1][nc][2 * tq + 8]);
        bni[0] = *reinterpret_cast<const uint32_t*>(&Bs[sb][2][nc][2 * tq]);
        bni[1] = *reinterpret_cast<const uint32_t*>(&Bs[sb][2][nc][2 * tq + 8]);
        mma_bf16(acc[nt][0], af[sa][0], br);    // re += Ar Br
        mma_bf16(acc[nt][0], af[sa][1], bni);   // re += Ai (-Bi)
        mma_bf16(acc[nt][1], af[sa][0], bi);    // im += Ar Bi
        mma_bf16(acc[nt][1], af[sa][1], br);    // im += Ai Br
      }
    }
    __syncthreads();
  }
  float4 gv[4][4];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = row0 + wm * 16 + g + ((e >> 1) ? 8 : 0);
      const int cc = col0 + wn * 32 + nt * 8 + 2 * tq + (e & 1);
      if (r < ns && cc < ns) gv[nt][e] = G[r + (size_t)ns * cc];
    }
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = row0 + wm * 16 + g + ((e >> 1) ? 8 : 0);
      const int cc = col0 + wn * 32 + nt * 8 + 2 * tq + (e & 1);
      if (r < ns && cc < ns) G[r + (size_t)ns * cc] = dg_addf(gv[nt][e], make_float2(acc[nt][0][e], acc[nt][1][e]));
    }
}

// ---------------------------------------------------------------------------
// Rank-K flush on the 5th-generation tensor cores (tcgen05).
//
// The complex update G += A B is one real GEMM  D = A' B'^T  with
//   A' = [Ar | Ai]               (rows of G  x  2K),
//   B' = [[Br | -Bi]; [Bi | Br]] (64 re columns then 64 im columns x 2K),
// every FP32 operand split into three BF16 terms (hi, mid, lo) and the six
// products hi.hi, hi.mid, mid.hi, hi.lo, mid.mid, lo.hi accumulated into one
// FP32 accumulator in tensor memory (128 lanes x 128 columns per tile).
//
// k_bsplit writes the split operands as shared-memory tile images in the
// no-swizzle K-major core-matrix layout: a core matrix is 8 rows x 16 bytes
// (8 BF16 along K); a tile image of nrg row groups puts core (row group i8,
// K group j8) at j8 * nrg * 128 + i8 * 128 bytes, so the first k columns of
// each half of an image are one contiguous prefix.  Each image is
// 2*UM_KP BF16 wide (Ar/Br-part at k < UM_KP, Ai-part at UM_KP + k; the
// second half starts at (UM_KP/8) * nrg * 128).  Per chain: um_rtiles row
// tiles of A' and um_ctiles column tiles of B', three splits each, every
// image in a UM_IMG slot.  The images are compact: a row tile holds only
// its rows of G (the last one of an Ns that is not a multiple of 128 holds
// fewer), and a column tile with nc <= 32 columns of G holds 32 re columns
// followed by 32 im columns (ncg = 4 core groups each; rows past nc are
// never written and only reach accumulator columns that are not read), so
// the flush of a ragged tile copies and multiplies only what it needs
// (N = 16 ncg).

// three-way BF16 split of an FP32 value
__device__ __forceinline__ void split3b(float x, __nv_bfloat16* o) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(h);
  const __nv_bfloat16 m = __float2bfloat16_rn(r1);
  o[0] = h;
  o[1] = m;
  o[2] = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

__global__ void __launch_bounds__(256) k_bsplit(const BDesc* D, unsigned char* img_all) {
  const BDesc& d = D[blockIdx.y];
  const int K = *d.kcount;
  if (K == 0) return;
  const int ns = d.M.ns, ldp = d.ldp, K16 = (K + 15) & ~15;
  const int RT = um_rtiles(ns);
  unsigned char* img = img_all + um_chain_bytes(ns) * blockIdx.y;
  // work items: (group of 8 k, row of G) for A', then (group of 8 k, column
  // of G) for B', rows and columns padded to whole core matrices (R8);
  // consecutive threads take consecutive rows or columns, so the panel reads
  // coalesce, and every thread writes 16-byte core-matrix rows.  A B' item
  // writes both image rows of its column (re and im), so each panel entry is
  // read and split once; RN rounding is sign-symmetric: split(-x) = -split(x).
  const int KG = K16 / 8;
  const long R8 = (long)((ns + 7) / 8) * 8;
  const long na = R8 * KG;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < 2 * na; e += (long)gridDim.x * blockDim.x) {
    const bool isb = e >= na;
    const long e2 = isb ? e - na : e;
    const int r = (int)(e2 % R8), kg = (int)(e2 / R8);
    __align__(16) __nv_bfloat16 xs[3][8], ys[3][8];   // splits of the re and im parts at k = kg*8 + jj
    const float2* P = isb ? d.B : d.A;
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const int k = kg * 8 + jj;
      const float2 v = (r < ns && k < K) ? P[(size_t)k * ldp + r] : make_float2(0.f, 0.f);
      __nv_bfloat16 a3[3], b3[3];
      split3b(v.x, a3);
      split3b(v.y, b3);
#pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        xs[s3][jj] = a3[s3];
        ys[s3][jj] = b3[s3];
      }
    }
    if (!isb) {   // A' row: [Ar | Ai]
      const int t = r / 128, row = r % 128, nrg = um_rg(ns, t);
      unsigned char* base = img + (size_t)t * 3 * UM_IMG;
      const int o1 = um_off(row, kg * 8, nrg), o2 = um_off(row, UM_KP + kg * 8, nrg);
#pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        *reinterpret_cast<uint4*>(base + (size_t)s3 * UM_IMG + o1) = *reinterpret_cast<const uint4*>(xs[s3]);
        *reinterpret_cast<uint4*>(base + (size_t)s3 * UM_IMG + o2) = *reinterpret_cast<const uint4*>(ys[s3]);
      }
    } else {      // B' re row c: [Br | -Bi], im row 8 ncg + c: [Bi | Br]
      const int t = r / 64, c = r % 64, ncg = um_cg(ns, t), nrg = 2 * ncg;
      unsigned char* base = img + (size_t)(RT + t) * 3 * UM_IMG;
      const int o1 = um_off(c, kg * 8, nrg), o2 = um_off(c, UM_KP + kg * 8, nrg);
      const int o3 = um_off(8 * ncg + c, kg * 8, nrg), o4 = um_off(8 * ncg + c, UM_KP + kg * 8, nrg);
#pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        uint4 yn = *reinterpret_cast<const uint4*>(ys[s3]);
        yn.x ^= 0x80008000u;
        yn.y ^= 0x80008000u;
        yn.z ^= 0x80008000u;
        yn.w ^= 0x80008000u;
        unsigned char* b3 = base + (size_t)s3 * UM_IMG;
        *reinterpret_cast<uint4*>(b3 + o1) = *reinterpret_cast<const uint4*>(xs[s3]);
        *reinterpret_cast<uint4*>(b3 + o2) = yn;
        *reinterpret_cast<uint4*>(b3 + o3) = *reinterpret_cast<const uint4*>(ys[s3]);
        *reinterpret_cast<uint4*>(b3 + o4) = *reinterpret_cast<const uint4*>(xs[s3]);
      }
    }
  }
}


// one CTA per (128-row tile, 64-column tile, chain), two CTAs per SM; 8
// warps: warps w and w+4 read accumulator lanes 32(w%4).. and take column
// halves 0 and 1.  Thread 0 streams the six images through shared memory in
// their two K halves (the Ar/Br part, then the Ai part): copies of a half,
// the six split products over it, and the next half's copies once those
// products have read the buffer.  Each thread reads the first 16 of its 32
// G entries while the copies and products run, the rest after.
constexpr int UM_HALF = UM_IMG / 2;   // bytes of one K half of a tile image (16 KB)
__global__ void __launch_bounds__(256, 2) k_bflush_um(const BDesc* D, const unsigned char* img_all, int parity) {
  __shared__ BDesc sd;
  __shared__ __align__(8) uint64_t s_load[2], s_mma[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail, s_last;
  extern __shared__ __align__(1024) unsigned char um_dyn[];   // 3 A half-images, then 3 B half-images
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    sd = D[blockIdx.y];
    s_fail = 0;
    s_last = -1;
    for (int h = 0; h < 2; ++h) {
      mbar_init(&s_load[h], 1);
      mbar_init(&s_mma[h], 1);
    }
    fence_mbar_init();
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_addr(&s_taddr))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const BDesc& d = sd;
  const uint32_t taddr = s_taddr;
  const int K = *d.kcount;
  const int ns = d.M.ns, RT = um_rtiles(ns);
  const int ti = blockIdx.x % RT, tj = blockIdx.x / RT;
  const int nrg_a = um_rg(ns, ti), ncg = um_cg(ns, tj), nrg_b = 2 * ncg;
  if (K > 0) {
    if (blockIdx.x == 0 && tid == 0) atomicAdd(d.nflush, 1ull);
    const int K16 = (K + 15) & ~15;
    const unsigned char* img = img_all + um_chain_bytes(ns) * blockIdx.y;
    const uint32_t ka = (uint32_t)nrg_a * 128, kb = (uint32_t)nrg_b * 128;   // bytes per K group
    const uint32_t part_a = (uint32_t)(K16 / 8) * ka, part_b = (uint32_t)(K16 / 8) * kb;   // k < K16 of one half
    const uint32_t h2a = (uint32_t)(UM_KP / 8) * ka, h2b = (uint32_t)(UM_KP / 8) * kb;     // second half in global
    if (tid == 0) {
      // split pairs (A', B'): (0,0) (0,1) (1,0) (0,2) (1,1) (2,0), packed 2 bits each
      constexpr uint32_t PA = 0u | (0u << 2) | (1u << 4) | (0u << 6) | (1u << 8) | (2u << 10);
      constexpr uint32_t PB = 0u | (1u << 2) | (0u << 4) | (2u << 6) | (1u << 8) | (0u << 10);
      const uint32_t base = smem_addr(um_dyn), idesc = um_idesc(16u * (uint32_t)ncg);
      uint32_t acc = 0;
      for (int half = 0; half < 2 && !s_fail; ++half) {
        if (half == 1) {   // the products of half 0 have read the buffer
          if (!mbar_wait_bounded(&s_mma[0], 0)) {
            s_fail = 1;
            break;
          }
          um_fence_after();
        }
        mbar_arrive_tx(&s_load[half], 3u * (part_a + part_b));
        for (int s3 = 0; s3 < 3; ++s3) {
          const unsigned char* ga = img + ((size_t)ti * 3 + s3) * UM_IMG + half * h2a;
          const unsigned char* gb = img + ((size_t)(RT + tj) * 3 + s3) * UM_IMG + half * h2b;
          bulk_g2s(um_dyn + (size_t)s3 * UM_HALF, ga, part_a, &s_load[half]);
          bulk_g2s(um_dyn + (size_t)(3 + s3) * UM_HALF, gb, part_b, &s_load[half]);
        }
        if (!mbar_wait_bounded(&s_load[half], 0)) {
          s_fail = 1;
          mbar_wait_bounded(&s_load[half], 0);   // a second bounded wait for the copies in flight
          break;
        }
        um_fence_after();
        for (int pr = 0; pr < 6; ++pr) {
          const uint32_t sa = (PA >> (2 * pr)) & 3u, sb = (PB >> (2 * pr)) & 3u;
          for (int kk = 0; kk < K16 / 16; ++kk) {
            const uint64_t ad = um_desc(base + sa * UM_HALF + kk * 2 * ka, ka, 128);
            const uint64_t bd = um_desc(base + (3 + sb) * UM_HALF + kk * 2 * kb, kb, 128);
            um_mma(taddr, ad, bd, idesc, acc);
            acc = 1;
          }
        }
        um_commit(&s_mma[half]);   // also tracks every earlier product
        s_last = half;
      }
    }
    // epilogue: accumulator lanes (rows) 32(w%4)..+31, columns of half w/4
    // (re at TMEM column c, im at 8 ncg + c), in two chunks of 16 columns
    float4* G = reinterpret_cast<float4*>(parity ? d.g_alt : d.g);
    const int q = warp & 3, half = warp >> 2;
    const int r = ti * 128 + q * 32 + lane;
    const int col0 = tj * 64 + half * 32;
    const int ncol = min(32, ns - col0);
    float4 gv[16];
    if (r < ns) {
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < ncol) gv[c] = G[r + (size_t)ns * (col0 + c)];
    }
    __syncthreads();
    const int last = s_last;
    if (last >= 0) {
      if (!mbar_wait_bounded(&s_mma[last], 0)) s_fail = 1;   // every thread observes the last commit
      um_fence_after();
    }
    __syncthreads();
    if (!s_fail) {
      const uint32_t lane_base = (uint32_t)(q * 32) << 16;
#pragma unroll 1
      for (int ch = 0; ch < 2; ++ch) {
        const int c0 = ch * 16;
        if (ncol <= c0) break;   // warp-uniform
        if (ch == 1 && r < ns) {
#pragma unroll
          for (int c = 0; c < 16; ++c)
            if (c0 + c < ncol) gv[c] = G[r + (size_t)ns * (col0 + c0 + c)];
        }
        float re[16], im[16];
        um_ld16(taddr + lane_base + half * 32 + c0, re);
        um_ld16(taddr + lane_base + 8 * ncg + half * 32 + c0, im);
        if (r < ns) {
#pragma unroll
          for (int c = 0; c < 16; ++c)
            if (c0 + c < ncol) G[r + (size_t)ns * (col0 + c0 + c)] = dg_addf(gv[c], make_float2(re[c], im[c]));
        }
      }
    } else if (tid == 0) {
      atomicExch(d.err, PQMC_ERR_TIMEOUT);
    }
  }
  um_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(taddr) : "memory");
}

// ---------------------------------------------------------------------------
// Two-way wrap with an FP32 correction on the FP64 G (left: A=expKV, B=expKV_inv).
// Items are the family's plaquettes (DIM sites) and uncovered singletons, so
// every block of G between a row item and a column item is at most DIM x DIM
// and lives in registers.  A CTA takes WRAP_R row items x WRAP_C column items,
// one pair per thread, and first forms (A - I) of its row items and (B - I)
// of its column items once, in FP64 rounded to FP32, into shared memory
// (entry-major, so the threads of a warp read consecutive words).
constexpr int WRAP_R = 32, WRAP_C = 4;

// the wrap of one DIM x DIM block of G (rows of one cover item, columns of
// another) in double-float, in two one-sided passes: T = G B row by row,
// then G' = A T column by column, with A = I + am, B = I + bm; every entry
// starts from its identity term and takes DIM error-free products.  get(a,
// b) / put(a, b, v) read and write entry (a, b) of the block (in place);
// am(a, k), bm(k, b) read the double-float (A - I), (B - I).  The outer
// loops are not unrolled: the fully unrolled form overflowed the
// instruction cache.
template <int DIM, typename GET, typename PUT, typename AM, typename BM>
__device__ __forceinline__ void wrap2_df(int dr, int dc, GET get, PUT put, AM am, BM bm) {
#pragma unroll 1
  for (int a = 0; a < dr; ++a) {
    float4 g[DIM], t[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) g[k] = k < dc ? get(a, k) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      dfc acc = dfc_from_dg(g[b]);
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const float4 v = bm(k, b);
        acc = dfc_fms(acc, dfc{df{-g[k].x, -g[k].z}, df{-g[k].y, -g[k].w}}, dfc_from_dg(v));
      }
      t[b] = dg_from_dfc(acc);
    }
#pragma unroll
    for (int b = 0; b < DIM; ++b)
      if (b < dc) put(a, b, t[b]);
  }
#pragma unroll 1
  for (int b = 0; b < dc; ++b) {
    float4 t[DIM], o[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) t[k] = k < dr ? get(k, b) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      dfc acc = dfc_from_dg(t[a]);
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const float4 v = am(a, k);
        acc = dfc_fms(acc, dfc{df{-v.x, -v.z}, df{-v.y, -v.w}}, dfc_from_dg(t[k]));
      }
      o[a] = dg_from_dfc(acc);
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a)
      if (a < dr) put(a, b, o[a]);
  }
}

// the double-float (A - I) (row use) and (B - I) (column use) of every cover
// item of family pf at the group's slice, once per wrap and chain:
// tab[0][e][item] and tab[1][e][item], e = a + DIM b, zero for singletons
template <int DIM>
__global__ void k_wtab(const BDesc* D, int pf, int left, int n_items, const int* __restrict__ wpla,
                       const int* __restrict__ wdim, float4* tab_all) {
  const BDesc& d = D[blockIdx.y];
  const DevModel& M = d.M;
  const int t = d.t, pd = M.pdim;
  float4* tab = tab_all + (size_t)blockIdx.y * 2 * 16 * n_items;
  const int n = 2 * DIM * DIM * n_items;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int item = e % n_items, ent = (e / n_items) % (DIM * DIM), isc = e / (n_items * DIM * DIM);
    const int a = ent % DIM, b = ent / DIM;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    const int p = wpla[item], dm = wdim[item];
    if (p >= 0 && a < dm && b < dm) {
      const cplx* X = (isc ? (left ? d.expkv_inv : d.expkv) : (left ? d.expkv : d.expkv_inv)) + M.kv_base(p, pf, t);
      v = dg_make(csub(X[a + pd * b], mk(a == b ? 1.0 : 0.0)));
    }
    tab[(size_t)isc * 16 * n_items + (size_t)ent * n_items + item] = v;
  }
}

template <int DIM, int DF>
__global__ void __launch_bounds__(128, 3) k_bwrap(const BDesc* D, int pf, int left, int n_items, int parity,
                                               const int* __restrict__ wpla, const int* __restrict__ wsites,
                                               const int* __restrict__ wdim, const float4* __restrict__ tab_all) {
  __shared__ BDesc sd;
  __shared__ float4 s_am[DIM * DIM][WRAP_R];   // (A - I)(a, b) of row item lr at [a + DIM b][lr] (double-float)
  __shared__ float4 s_bm[DIM * DIM][WRAP_C];
  if (threadIdx.x == 0) sd = D[blockIdx.z];
  __syncthreads();
  const BDesc& d = sd;
  const DevModel& M = d.M;
  const int t = d.t;
  const int ns = M.ns, pd = M.pdim;
  const int ir0 = blockIdx.x * WRAP_R, ic0 = blockIdx.y * WRAP_C;
  const int lr = threadIdx.x % WRAP_R, lc = threadIdx.x / WRAP_R;
  const int ir = ir0 + lr, ic = ic0 + lc;
  const bool live = ir < n_items && ic < n_items;
  const int dr = live ? wdim[ir] : 0, dc = live ? wdim[ic] : 0;
  const float4* gin = reinterpret_cast<const float4*>(parity ? d.g_alt : d.g);   // double-float G
  float4* gout = reinterpret_cast<float4*>(parity ? d.g : d.g_alt);
  int Sr[DIM], Sc[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    Sr[k] = k < dr ? wsites[4 * ir + k] : 0;
    Sc[k] = k < dc ? wsites[4 * ic + k] : 0;
  }
  // the block of G, loaded first so that the loads are in flight while the
  // CTA forms its (A - I) and (B - I); its FP32 rounding dg_f2 is formed
  // where it is used (fewer registers)
  float4 gd[DIM][DIM];
#pragma unroll
  for (int b = 0; b < DIM; ++b)
#pragma unroll
    for (int a = 0; a < DIM; ++a)
      gd[a][b] = (a < dr && b < dc) ? gin[Sr[a] + (size_t)ns * Sc[b]] : make_float4(0.f, 0.f, 0.f, 0.f);
  // A - I and B - I formed in FP64 and rounded once; zero for singletons.
  // Consecutive threads take consecutive items of one entry.
  const float4* tab = DF ? tab_all + (size_t)blockIdx.z * 2 * 16 * n_items : nullptr;
  for (int e = threadIdx.x; e < (WRAP_R + WRAP_C) * DIM * DIM; e += blockDim.x) {
    const bool isc = e >= WRAP_R * DIM * DIM;
    const int e2 = isc ? e - WRAP_R * DIM * DIM : e;
    const int nl = isc ? WRAP_C : WRAP_R;
    const int il = e2 % nl, ent = e2 / nl, a = ent % DIM, b = ent / DIM;
    const int item = (isc ? ic0 : ir0) + il;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (DF) {   // the tables of k_wtab
      if (item < n_items) v = tab[(size_t)(isc ? 1 : 0) * 16 * n_items + (size_t)ent * n_items + item];
    } else if (item < n_items) {
      const int p = wpla[item], dm = wdim[item];
      if (p >= 0 && a < dm && b < dm) {
        const cplx* X = (isc ? (left ? d.expkv_inv : d.expkv) : (left ? d.expkv : d.expkv_inv)) + M.kv_base(p, pf, t);
        const cplx x = csub(X[a + pd * b], mk(a == b ? 1.0 : 0.0));
        v = make_float4((float)x.x, (float)x.y, 0.f, 0.f);
      }
    }
    if (isc) s_bm[ent][il] = v;
    else s_am[ent][il] = v;
  }
  __syncthreads();
  if (!live) return;
  if (DF) {
    float4 blk[DIM * DIM];   // the block, entry (a, b) at a + DIM b
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int a = 0; a < DIM; ++a) blk[a + DIM * b] = gd[a][b];
    wrap2_df<DIM>(dr, dc, [&](int a, int b) { return blk[a + DIM * b]; },
                  [&](int a, int b, float4 v) { blk[a + DIM * b] = v; },
                  [&](int a, int k) { return s_am[a + DIM * k][lr]; }, [&](int k, int b) { return s_bm[k + DIM * b][lc]; });
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int a = 0; a < DIM; ++a)
        if (a < dr && b < dc) gout[Sr[a] + (size_t)ns * Sc[b]] = blk[a + DIM * b];
    return;
  }
  // corr = (A - I) (G B) + G (B - I) = (A - I) G + (A - I) G (B - I) + G (B - I)
  float2 gb[DIM][DIM];   // G (B - I)
#pragma unroll
  for (int b = 0; b < DIM; ++b)
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      float2 s = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < DIM; ++k) s = fa(s, fm(dg_f2(gd[a][k]), hi2(s_bm[k + DIM * b][lc])));
      gb[a][b] = s;
    }
#pragma unroll
  for (int b = 0; b < DIM; ++b)
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      float2 corr = gb[a][b];
#pragma unroll
      for (int k = 0; k < DIM; ++k) corr = fa(corr, fm(hi2(s_am[a + DIM * k][lr]), fa(dg_f2(gd[k][b]), gb[k][b])));
      if (a < dr && b < dc) gout[Sr[a] + (size_t)ns * Sc[b]] = dg_addf(gd[a][b], corr);
    }
}

// Two-way wrap with whole columns of G staged in shared memory (used when
// they fit).  The family's cover items partition the sites, so a CTA that
// owns WRAPC_C column items owns every entry of their columns: it brings the
// columns in with 1-D bulk copies, forms (A - I) of every row item and
// (B - I) of its column items (FP64, rounded once), updates each block (row
// item x column item) in place with the arithmetic of k_bwrap, entry for
// entry, and writes the columns back with bulk stores.  Every entry of G is
// read and written once, in whole columns.  The number of column items per
// CTA (CI, 1 or 2) is a tile shape chosen by pqmc_batch_autotune_tiles:
// one item halves the staged columns, so more CTAs share an SM; two items
// share the row items' (A - I) table between more blocks.
constexpr int WRAPC_C_DEFAULT = 1;
constexpr size_t WRAPC_MAX_SMEM = 200 * 1024;   // dynamic shared memory of k_bwrap_cols at most
__host__ __device__ inline size_t wrapc_smem(int ns, int n_items, int dim, int ci) {
  return (size_t)ci * dim * ns * 16 + (size_t)dim * dim * (n_items + ci) * 16 + (size_t)n_items * 6 * 4;
}

template <int DIM, int DF, int WRAPC_C>
__global__ void __launch_bounds__(128, 4) k_bwrap_cols(const BDesc* D, int pf, int left, int n_items, int parity,
                                                    const int* __restrict__ wpla, const int* __restrict__ wsites,
                                                    const int* __restrict__ wdim, const float4* __restrict__ tab_all) {
  __shared__ BDesc sd;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_fail;
  extern __shared__ __align__(128) unsigned char wc_dyn[];
  const int tid = threadIdx.x;
  if (tid == 0) {
    sd = D[blockIdx.y];
    s_fail = 0;
    mbar_init(&s_bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const BDesc& d = sd;
  const DevModel& M = d.M;
  const int t = d.t;
  const int ns = M.ns, pd = M.pdim;
  const int ic0 = blockIdx.x * WRAPC_C, ncl = min(WRAPC_C, n_items - ic0);
  float4* s_col = reinterpret_cast<float4*>(wc_dyn);                              // [WRAPC_C * DIM][ns]
  float4* s_am = s_col + (size_t)WRAPC_C * DIM * ns;                              // [DIM * DIM][n_items]
  float4* s_bm = s_am + (size_t)DIM * DIM * n_items;                              // [DIM * DIM][WRAPC_C]
  int* s_pla = reinterpret_cast<int*>(s_bm + (size_t)DIM * DIM * WRAPC_C);        // cover items: plaquette,
  int* s_dim = s_pla + n_items;                                                   // dimension and
  int* s_site = s_dim + n_items;                                                  // sites (4 per item)
  const float4* gin = reinterpret_cast<const float4*>(parity ? d.g_alt : d.g);   // double-float G
  float4* gout = reinterpret_cast<float4*>(parity ? d.g : d.g_alt);
  const uint32_t cbytes = (uint32_t)ns * 16u;   // one column of G
  if (tid == 0) {
    // the sites of the column items, all loads issued before any is used
    int cdim[WRAPC_C], csite[WRAPC_C][DIM];
#pragma unroll
    for (int icl = 0; icl < WRAPC_C; ++icl) {
      cdim[icl] = icl < ncl ? wdim[ic0 + icl] : 0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) csite[icl][b] = icl < ncl ? wsites[4 * (ic0 + icl) + b] : 0;
    }
    uint32_t bytes = 0;
#pragma unroll
    for (int icl = 0; icl < WRAPC_C; ++icl) bytes += (uint32_t)cdim[icl] * cbytes;
    mbar_arrive_tx(&s_bar, bytes);
#pragma unroll
    for (int icl = 0; icl < WRAPC_C; ++icl)
#pragma unroll
      for (int b = 0; b < DIM; ++b)
        if (b < cdim[icl])
          bulk_g2s(s_col + (size_t)(icl * DIM + b) * ns, gin + (size_t)ns * csite[icl][b], cbytes, &s_bar);
  }
  for (int e = tid; e < n_items; e += blockDim.x) {
    s_pla[e] = wpla[e];
    s_dim[e] = wdim[e];
  }
  for (int e = tid; e < 4 * n_items; e += blockDim.x) s_site[e] = wsites[e];
  __syncthreads();
  // A - I of every row item and B - I of the CTA's column items, formed in
  // FP64 and rounded once (zero for singletons); consecutive threads take
  // consecutive items of one entry, four entries per thread in flight
  const int n_ent = (n_items + WRAPC_C) * DIM * DIM;
  if (DF) {   // the tables of k_wtab
    const float4* tab = tab_all + (size_t)blockIdx.y * 2 * 16 * n_items;
    for (int e = tid; e < n_ent; e += blockDim.x) {
      const bool isc = e >= n_items * DIM * DIM;
      const int e2 = isc ? e - n_items * DIM * DIM : e;
      const int nl = isc ? WRAPC_C : n_items;
      const int il = e2 % nl, ent = e2 / nl, item = isc ? ic0 + il : il;
      s_am[isc ? n_items * DIM * DIM + ent * WRAPC_C + il : ent * n_items + il] =
          item < n_items ? tab[(size_t)(isc ? 1 : 0) * 16 * n_items + (size_t)ent * n_items + item]
                         : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  for (int e0 = tid; e0 < n_ent && !DF; e0 += 4 * blockDim.x) {
    cplx x[4];
    int slot[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * blockDim.x;
      slot[u] = -1;
      x[u] = mk(0.0);
      if (e >= n_ent) continue;
      const bool isc = e >= n_items * DIM * DIM;
      const int e2 = isc ? e - n_items * DIM * DIM : e;
      const int nl = isc ? WRAPC_C : n_items;
      const int il = e2 % nl, ent = e2 / nl, a = ent % DIM, b = ent / DIM;
      const int item = isc ? ic0 + il : il;
      slot[u] = isc ? n_items * DIM * DIM + ent * WRAPC_C + il : ent * n_items + il;
      if (item < n_items) {
        const int p = s_pla[item], dm = s_dim[item];
        if (p >= 0 && a < dm && b < dm) {
          const cplx* X = (isc ? (left ? d.expkv_inv : d.expkv) : (left ? d.expkv : d.expkv_inv)) + M.kv_base(p, pf, t);
          x[u] = csub(X[a + pd * b], mk(a == b ? 1.0 : 0.0));
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)   // s_bm follows s_am contiguously
      if (slot[u] >= 0) s_am[slot[u]] = make_float4((float)x[u].x, (float)x[u].y, 0.f, 0.f);
  }
  if (!mbar_wait_bounded(&s_bar, 0)) s_fail = 1;
  __syncthreads();
  if (s_fail) {
    if (tid == 0) {   // a second bounded wait for the copies in flight
      mbar_wait_bounded(&s_bar, 0);
      atomicExch(d.err, PQMC_ERR_TIMEOUT);
    }
    return;
  }
  for (int pr = tid; pr < n_items * ncl; pr += blockDim.x) {
    const int ir = pr % n_items, icl = pr / n_items, ic = ic0 + icl;
    const int dr = s_dim[ir], dc = s_dim[ic];
    int Sr[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) Sr[k] = k < dr ? s_site[4 * ir + k] : 0;
    float4* col = s_col + (size_t)icl * DIM * ns;
    if (DF) {
      wrap2_df<DIM>(dr, dc, [&](int a, int b) { return col[(size_t)b * ns + Sr[a]]; },
                    [&](int a, int b, float4 v) { col[(size_t)b * ns + Sr[a]] = v; },
                    [&](int a, int k) { return s_am[(size_t)(a + DIM * k) * n_items + ir]; },
                    [&](int k, int b) { return s_bm[(size_t)(k + DIM * b) * WRAPC_C + icl]; });
      continue;
    }
    float4 gd[DIM][DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int a = 0; a < DIM; ++a)
        gd[a][b] = (a < dr && b < dc) ? col[(size_t)b * ns + Sr[a]] : make_float4(0.f, 0.f, 0.f, 0.f);
    // corr = (A - I) (G B) + G (B - I), as in k_bwrap
    float2 gb[DIM][DIM];   // G (B - I)
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        float2 sum = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < DIM; ++k) sum = fa(sum, fm(dg_f2(gd[a][k]), hi2(s_bm[(size_t)(k + DIM * b) * WRAPC_C + icl])));
        gb[a][b] = sum;
      }
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        float2 corr = gb[a][b];
#pragma unroll
        for (int k = 0; k < DIM; ++k)
          corr = fa(corr, fm(hi2(s_am[(size_t)(a + DIM * k) * n_items + ir]), fa(dg_f2(gd[k][b]), gb[k][b])));
        if (a < dr && b < dc) col[(size_t)b * ns + Sr[a]] = dg_addf(gd[a][b], corr);
      }
  }
  fence_proxy_async_smem();   // the updated columns visible to the bulk stores
  __syncthreads();
  if (tid == 0) {
    for (int icl = 0; icl < ncl; ++icl) {
      const int dc = s_dim[ic0 + icl];
      for (int b = 0; b < dc; ++b)
        bulk_s2g(gout + (size_t)ns * s_site[4 * (ic0 + icl) + b], s_col + (size_t)(icl * DIM + b) * ns, cbytes);
    }
    bulk_commit_wait_all();
  }
}

// G of every chain converted in place between FP64 complex (at rest) and the
// double-float float4 form the mixed sweep works on
__global__ void k_gconv(const BDesc* D, int to_df, long n, int parity) {
  cplx* G = parity ? D[blockIdx.y].g_alt : D[blockIdx.y].g;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    if (to_df) {
      const cplx v = G[e];
      reinterpret_cast<float4*>(G)[e] = dg_make(v);
    } else {
      const float4 v = reinterpret_cast<const float4*>(G)[e];
      G[e] = dg_to_d(v);
    }
  }
}

}  // namespace pqmc

// ===========================================================================
struct PhaseMark {
  int phase;
  cudaEvent_t a, b;
};

struct pqmc_batch {
  std::vector<pqmc_chain*> chains;
  // CUDA-event timers per phase of the family step (PQMC_PHASE_*)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<PhaseMark> marks;
  double phase_ms[PQMC_N_PHASES] = {};
  long long phase_n[PQMC_N_PHASES] = {};
  int precision = PQMC_PREC_FP64;
  pqmc::BDesc* d_desc = nullptr;
  std::vector<pqmc::BDesc> h_desc;
  std::vector<float2*> panels;
  std::vector<int*> kcounts;
  int parity = 0;
  int kd = 64;            // delay depth (panel columns per flush)
  int qc = 8;             // panel columns per streamed chunk of the scan
  int qc_max = 8;         // the largest chunk whose staging fits in shared memory
  // 2: exact round update (exact.cuh; delay depth <= 64), 1: tcgen05 flush of
  // the scan's FP32 panels (delay depth <= 64), 0: mma.sync flush of them
  int flush_mode = 2;
  pqmc::XDesc* d_xdesc = nullptr;   // per chain: the exact update's view
  std::vector<pqmc::XDesc> h_xdesc;
  unsigned char* d_ximg = nullptr;  // slice images of the exact update
  unsigned char* d_acc = nullptr;   // accepted-move records of every chain
  int wrap_df_mode = -1;            // double-float wraps: -1 with the exact update, 0 never, 1 always
  float4* d_wtab = nullptr;         // per chain: the wrap's double-float (A - I), (B - I) tables
  // kernels launched at the device's highest stream priority (bit 0: the
  // scan, bit 1: the split and flush); slice graphs then use node priorities
  int prio_mask = 3, prio_hi = 0;
  unsigned char* d_img = nullptr;   // split operand tile images of the tcgen05 flush
  CUtensorMap* d_tmaps = nullptr;   // per chain: maps of its two G buffers
  int rb = 0, nrb = 0;              // row box of the maps (columns) and boxes per row
  std::vector<cplx*> tm_buf;        // per chain x 2: the buffer each map describes
  int* d_err = nullptr;   // device error word shared by all chains
  int* d_next = nullptr;  // per chain: next plaquette of the current family step
  cudaStream_t stream = nullptr;   // the stream of group 0, the batch's public stream
  // chain groups: each group has its own stream and recompute workspace, so
  // one group's latency-bound scan overlaps the other's flush and recompute
  static constexpr int MAX_GROUPS = 16;
  int n_groups = 1;
  int g_first[MAX_GROUPS] = {}, g_count[MAX_GROUPS] = {};
  cudaStream_t g_stream[MAX_GROUPS] = {};
  pqmc::BatchRecompute rec[MAX_GROUPS];
  cudaEvent_t ev_fork = nullptr, ev_join[MAX_GROUPS] = {};
  // uneven batch (mixed precision, chains of more than one geometry): one
  // homogeneous batch per geometry class; `chains` then borrows their chains
  std::vector<pqmc_batch*> parts;
  std::vector<int> part_of, index_in_part;
  // slice graphs (pqmc_batch_set_graphs): captured family steps of one slice
  struct SliceGraph {
    int key[6];   // group, forward, parity, delay depth, flush engine, chunk
    cudaGraphExec_t exec;
    int kernels;  // kernel nodes per replay
  };
  bool graphs = false;
  std::vector<char> wrap_cols;   // per family: the most column items per k_bwrap_cols CTA whose columns fit (0: k_bwrap)
  int wrap_ci = 1;               // wrap tile: column items per k_bwrap_cols CTA (1, 2), 0 for the gather form k_bwrap
  int xflush_ct = 64;            // flush of the exact round update: 64 (k_xgemm<1>) or 32 (k_xflush2) columns per
                                 // CTA, or 2 / 1 (k_xflushp: ranges of Z tiles per row tile)
  std::deque<SliceGraph> gcache;
  // proposal records of every family per chain (n_pf x max_pla); when the
  // families' bosons are disjoint, a slice's draws and proposals of all
  // families are formed in one launch each at the start of the slice
  std::vector<pqmc::PlaqPre*> pre_all;
  bool slice_prep = false;
  pqmc::DevScalars* h_states = nullptr;   // pinned staging of pqmc_batch_states
  unsigned long long* d_nflush = nullptr;  // per chain: flush rounds with work
  unsigned long long* d_scanprof = nullptr;  // per chain: scan cycles, accepted moves, rejected proposals
  // equal-time measurement inside batched sweeps (ms_begin_measure semantics)
  int meas_on = 0, meas_warmup = 0, meas_interval = 1, meas_number = 0;
  std::vector<std::vector<double>> records;   // finished records per chain
};

using namespace pqmc;

extern "C" int pqmc_create(const pqmc_model* model, pqmc_chain** out);
extern "C" int pqmc_destroy(pqmc_chain* c);
extern "C" int pqmc_sweep(pqmc_chain* c, int first_loop, int n_sweeps, int warmup, int meas_interval,
                          int meas_number, double* records, int n_records_cap, int* n_records);
extern "C" int pqmc_sweep_slices(pqmc_chain* c, int loop, int first_tc, int n_slices);
extern "C" int pqmc_init_g(pqmc_chain* c, int start_time);

static cudaEvent_t ev_take(pqmc_batch* b) {
  if (!b->ev_pool.empty()) {
    cudaEvent_t e = b->ev_pool.back();
    b->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// open a timed phase on the batch stream (no-op unless timing is on)
static cudaEvent_t phase_begin(pqmc_batch* b) {
  if (!b->timing) return nullptr;
  cudaEvent_t e = ev_take(b);
  if (e) cudaEventRecord(e, b->stream);
  return e;
}

static void phase_end(pqmc_batch* b, int phase, cudaEvent_t a) {
  if (!b->timing || !a) return;
  cudaEvent_t e = ev_take(b);
  if (!e) return;
  cudaEventRecord(e, b->stream);
  b->marks.push_back(PhaseMark{phase, a, e});
}

// after a stream synchronisation: fold the recorded pairs into the totals
static int phase_resolve(pqmc_batch* b) {
  for (auto& m : b->marks) {
    float ms = 0.f;
    PQMC_CUDA(cudaEventElapsedTime(&ms, m.a, m.b));
    b->phase_ms[m.phase] += ms;
    b->phase_n[m.phase] += 1;
    b->ev_pool.push_back(m.a);
    b->ev_pool.push_back(m.b);
  }
  b->marks.clear();
  return PQMC_OK;
}

static int batch_refresh(pqmc_batch* b) {
  // current G of every chain is c->g; rebuild descriptors, parity 0
  for (size_t i = 0; i < b->chains.size(); ++i) {
    b->h_desc[i].g = b->chains[i]->g;
    b->h_desc[i].g_alt = b->chains[i]->g_alt;
    if (b->d_tmaps) {
      const bool same = b->tm_buf[2 * i] == b->chains[i]->g;
      b->h_desc[i].tm_g = b->d_tmaps + 2 * i + (same ? 0 : 1);
      b->h_desc[i].tm_galt = b->d_tmaps + 2 * i + (same ? 1 : 0);
    }
  }
  b->parity = 0;
  PQMC_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), sizeof(BDesc) * b->h_desc.size(), cudaMemcpyHostToDevice,
                            b->stream));
  if (b->d_xdesc) {
    for (size_t i = 0; i < b->chains.size(); ++i) {
      b->h_xdesc[i].g = reinterpret_cast<float4*>(b->chains[i]->g);
      b->h_xdesc[i].g_alt = reinterpret_cast<float4*>(b->chains[i]->g_alt);
    }
    PQMC_CUDA(cudaMemcpyAsync(b->d_xdesc, b->h_xdesc.data(), sizeof(XDesc) * b->h_xdesc.size(),
                              cudaMemcpyHostToDevice, b->stream));
  }
  return PQMC_OK;
}

static int batch_sync_parity(pqmc_batch* b) {
  // make c->g the current buffer of every chain
  if (b->parity) {
    for (auto* c : b->chains) {
      cplx* t = c->g;
      c->g = c->g_alt;
      c->g_alt = t;
    }
  }
  return batch_refresh(b);
}

// phase timers follow group 0 only (groups overlap on the device)
static cudaEvent_t gphase_begin(pqmc_batch* b, int g) { return g == 0 ? phase_begin(b) : nullptr; }
static void gphase_end(pqmc_batch* b, int g, int phase, cudaEvent_t a) {
  if (g == 0) phase_end(b, phase, a);
}

// the dynamic shared-memory limit of every k_bwrap_cols variant of one
// family dimension and column-item count
template <int DM>
static cudaError_t raise_wrapc_dm(int ci, int sm) {
  cudaError_t e = ci == 1 ? raise_dyn_smem(k_bwrap_cols<DM, 0, 1>, sm) : raise_dyn_smem(k_bwrap_cols<DM, 0, 2>, sm);
  if (e != cudaSuccess) return e;
  return ci == 1 ? raise_dyn_smem(k_bwrap_cols<DM, 1, 1>, sm) : raise_dyn_smem(k_bwrap_cols<DM, 1, 2>, sm);
}
static cudaError_t raise_wrapc(int dim, int ci, int sm) {
  switch (dim) {
    case 1: return raise_wrapc_dm<1>(ci, sm);
    case 2: return raise_wrapc_dm<2>(ci, sm);
    case 3: return raise_wrapc_dm<3>(ci, sm);
    default: return raise_wrapc_dm<4>(ci, sm);
  }
}

// two-way wrap of group g's chains by family pf at the group's slice (the
// caller flips the parity)
static int bwrap(pqmc_batch* b, int g, int pf, bool left, int parity) {
  pqmc_chain* c0 = b->chains[0];
  const WrapItems& w = c0->wrap[pf];
  const int C = b->g_count[g];
  const BDesc* D = b->d_desc + b->g_first[g];
  cudaStream_t st = b->g_stream[g];
  const int l = left ? 1 : 0;
  // double-float wrap with the exact round update; PQMC_WRAP_DF=0 keeps the
  // FP32 correction there too, PQMC_WRAP_DF=1 uses double-float with every
  // flush mode
  const bool df = b->d_wtab && (b->wrap_df_mode == 1 || (b->wrap_df_mode < 0 && b->flush_mode == 2));
  cudaEvent_t tw = gphase_begin(b, g);
  float4* tab = df ? b->d_wtab + (size_t)b->g_first[g] * 2 * 16 * w.n_items : nullptr;
  if (df) {
    const int n = 2 * 16 * w.n_items;
    const dim3 gt((unsigned)((n + 255) / 256), (unsigned)C);
    switch (c0->h_pf_dim[pf]) {
      case 1: k_wtab<1><<<gt, 256, 0, st>>>(D, pf, l, w.n_items, w.d_pla, w.d_dim, tab); break;
      case 2: k_wtab<2><<<gt, 256, 0, st>>>(D, pf, l, w.n_items, w.d_pla, w.d_dim, tab); break;
      case 3: k_wtab<3><<<gt, 256, 0, st>>>(D, pf, l, w.n_items, w.d_pla, w.d_dim, tab); break;
      default: k_wtab<4><<<gt, 256, 0, st>>>(D, pf, l, w.n_items, w.d_pla, w.d_dim, tab); break;
    }
    PQMC_LAUNCHED();
  }
  const int ci = pf < (int)b->wrap_cols.size() ? std::min(b->wrap_ci, (int)b->wrap_cols[pf]) : 0;
  if (ci > 0) {   // columns staged, ci column items per CTA
    const dim3 gc((unsigned)((w.n_items + ci - 1) / ci), (unsigned)C);
    const size_t sm = wrapc_smem(c0->ns, w.n_items, c0->h_pf_dim[pf], ci);
#define PQMC_WC(DM, F)                                                                                          \
  do {                                                                                                          \
    if (ci == 1)                                                                                                \
      k_bwrap_cols<DM, F, 1><<<gc, 128, sm, st>>>(D, pf, l, w.n_items, parity, w.d_pla, w.d_sites, w.d_dim, tab); \
    else                                                                                                        \
      k_bwrap_cols<DM, F, 2><<<gc, 128, sm, st>>>(D, pf, l, w.n_items, parity, w.d_pla, w.d_sites, w.d_dim, tab); \
  } while (0)
    switch (c0->h_pf_dim[pf] + (df ? 4 : 0)) {
      case 1: PQMC_WC(1, 0); break;
      case 2: PQMC_WC(2, 0); break;
      case 3: PQMC_WC(3, 0); break;
      case 4: PQMC_WC(4, 0); break;
      case 5: PQMC_WC(1, 1); break;
      case 6: PQMC_WC(2, 1); break;
      case 7: PQMC_WC(3, 1); break;
      default: PQMC_WC(4, 1); break;
    }
#undef PQMC_WC
    PQMC_LAUNCHED();
    gphase_end(b, g, PQMC_PHASE_WRAP, tw);
    return PQMC_OK;
  }
  const dim3 grid((unsigned)((w.n_items + WRAP_R - 1) / WRAP_R), (unsigned)((w.n_items + WRAP_C - 1) / WRAP_C),
                  (unsigned)C);
#define PQMC_WG(DM, F) \
  k_bwrap<DM, F><<<grid, 128, 0, st>>>(D, pf, l, w.n_items, parity, w.d_pla, w.d_sites, w.d_dim, tab)
  switch (c0->h_pf_dim[pf] + (df ? 4 : 0)) {
    case 1: PQMC_WG(1, 0); break;
    case 2: PQMC_WG(2, 0); break;
    case 3: PQMC_WG(3, 0); break;
    case 4: PQMC_WG(4, 0); break;
    case 5: PQMC_WG(1, 1); break;
    case 6: PQMC_WG(2, 1); break;
    case 7: PQMC_WG(3, 1); break;
    default: PQMC_WG(4, 1); break;
  }
#undef PQMC_WG
  PQMC_LAUNCHED();
  gphase_end(b, g, PQMC_PHASE_WRAP, tw);
  return PQMC_OK;
}

// update_phonon_field of family pf for group g's chains at the group's slice
// draws and proposals of n_fam families from pf_first (step pf_step in the
// draw order) for group g
static int bprepare(pqmc_batch* b, int g, int pf_first, int pf_step, int n_fam) {
  const int C = b->g_count[g];
  const BDesc* Dg = b->d_desc + b->g_first[g];
  cudaStream_t st = b->g_stream[g];
  pqmc_chain* c0 = b->chains[0];
  const int bpf = (c0->max_pla + PREP_PLA - 1) / PREP_PLA;
  const int lo = pf_step > 0 ? pf_first : pf_first + (n_fam - 1) * pf_step;
  cudaEvent_t tp = gphase_begin(b, g);
  k_bdraw<<<(C + 63) / 64, 64, 0, st>>>(Dg, C, pf_first, pf_step, n_fam);
  PQMC_LAUNCHED();
  k_bprep<<<dim3(bpf * n_fam, C), 256, 0, st>>>(Dg, lo, bpf);
  PQMC_LAUNCHED();
  gphase_end(b, g, PQMC_PHASE_PREP, tp);
  return PQMC_OK;
}

static int bupdate(pqmc_batch* b, int g, int pf, int parity) {
  const int C = b->g_count[g], c_first = b->g_first[g];
  const BDesc* Dg = b->d_desc + c_first;
  int* next = b->d_next + c_first;
  cudaStream_t st = b->g_stream[g];
  pqmc_chain* c0 = b->chains[0];
  const int npla = c0->h_pf_npla[pf], dim = c0->h_pf_dim[pf];
  if (!b->slice_prep) PQMC_TRY(bprepare(b, g, pf, 1, 1));
  PQMC_CUDA(cudaMemsetAsync(next, 0, sizeof(int) * C, st));
  const bool exact = b->flush_mode == 2 && b->d_xdesc;
  const int kd = std::max(dim, std::min(std::min(b->kd, b->h_desc[0].kmax), exact ? UM_KP : SCAN_KSTAGE));
  // enough rounds for the worst case (every proposal accepted)
  const int rounds = (npla * dim + (kd / dim) * dim - 1) / ((kd / dim) * dim);
  const int tiles = ((c0->ns + FB_M - 1) / FB_M) * ((c0->ns + FB_N - 1) / FB_N);
  const int ns = c0->ns;
  unsigned char* img = b->d_img ? b->d_img + um_chain_bytes(ns) * c_first : nullptr;
  for (int r = 0; r < rounds; ++r) {
    const BDesc& h0 = b->h_desc[0];
    const size_t smem = scan_layout(npla, ns, h0.ldp, b->qc, kd, 4 * h0.nrb * h0.rb * (int)sizeof(float4)).total;
    cudaEvent_t ts = gphase_begin(b, g);
    const bool one = ns <= SCAN_THREADS;
#define PQMC_SCAN(DM, R)                                                                                         \
  PQMC_CUDA(launch_at(k_bscan<DM, R>, dim3(C), dim3(SCAN_THREADS), smem, st, (b->prio_mask & 1) != 0, b->prio_hi, Dg, \
                      pf, parity, kd, b->qc, next, exact ? 1 : 0, b->timing ? 1 : 0))
    switch (dim) {
      case 1: if (one) PQMC_SCAN(1, 1); else PQMC_SCAN(1, 2); break;
      case 2: if (one) PQMC_SCAN(2, 1); else PQMC_SCAN(2, 2); break;
      case 3: if (one) PQMC_SCAN(3, 1); else PQMC_SCAN(3, 2); break;
      default: if (one) PQMC_SCAN(4, 1); else PQMC_SCAN(4, 2); break;
    }
#undef PQMC_SCAN
    PQMC_LAUNCHED();
    gphase_end(b, g, PQMC_PHASE_SCAN, ts);
    if (b->flush_mode == 1 && img && kd <= UM_KP) {
      const long items = 2L * ((ns + 7) / 8 * 8) * (((kd + 15) & ~15) / 8);
      cudaEvent_t tsp = gphase_begin(b, g);
      PQMC_CUDA(launch_at(k_bsplit, dim3((unsigned)std::min<long>((items + 255) / 256, 256), C), dim3(256), 0, st,
                          (b->prio_mask & 2) != 0, b->prio_hi, Dg, img));
      PQMC_LAUNCHED();
      gphase_end(b, g, PQMC_PHASE_SPLIT, tsp);
    }
    if (exact) {   // double-float core and operand slices (timed as the split phase)
      cudaEvent_t tsp = gphase_begin(b, g);
      PQMC_TRY(exact_core(b->d_xdesc + c_first, C, ns, dim, parity, b->xflush_ct, st, (b->prio_mask & 2) != 0,
                          b->prio_hi));
      gphase_end(b, g, PQMC_PHASE_SPLIT, tsp);
    }
    cudaEvent_t tf = gphase_begin(b, g);
    if (exact) {
      PQMC_TRY(exact_products(b->d_xdesc + c_first, C, ns, parity, b->xflush_ct, st, (b->prio_mask & 2) != 0,
                              b->prio_hi));
    } else if (b->flush_mode == 1 && img && kd <= UM_KP) {
      PQMC_CUDA(launch_at(k_bflush_um, dim3(um_rtiles(ns) * um_ctiles(ns), C), dim3(256), (size_t)(6 * UM_HALF), st,
                          (b->prio_mask & 2) != 0, b->prio_hi, Dg, (const unsigned char*)img, parity));
      PQMC_LAUNCHED();
    } else {
      k_bflush<<<dim3(tiles, C), 256, 0, st>>>(Dg, parity);
      PQMC_LAUNCHED();
    }
    gphase_end(b, g, PQMC_PHASE_FLUSH, tf);
  }
  return PQMC_OK;
}

// the family steps of one slice for group g (Main_PQMC.f90:99-154: forward,
// update then wrap per family; backward, wrap then update in reverse family
// order), starting at `parity`; one parity flip per family
static int slice_ops(pqmc_batch* b, int g, bool forward, int parity) {
  pqmc_chain* c0 = b->chains[0];
  const bool upd = c0->M.local_update != 0;
  if (upd && b->slice_prep) PQMC_TRY(bprepare(b, g, forward ? 0 : c0->n_pf - 1, forward ? 1 : -1, c0->n_pf));
  if (!forward) {
    for (int pf = c0->n_pf - 1; pf >= 0; --pf) {
      PQMC_TRY(bwrap(b, g, pf, false, parity));
      parity ^= 1;
      if (upd && c0->h_pf_v_exist[pf]) PQMC_TRY(bupdate(b, g, pf, parity));
    }
  } else {
    for (int pf = 0; pf < c0->n_pf; ++pf) {
      if (upd && c0->h_pf_v_exist[pf]) PQMC_TRY(bupdate(b, g, pf, parity));
      PQMC_TRY(bwrap(b, g, pf, true, parity));
      parity ^= 1;
    }
  }
  return PQMC_OK;
}

// the executable graph of slice_ops(g, forward, parity) under the current
// delay depth, flush engine and chunk size, captured on first use.  Nothing
// a slice launches depends on its time index (read from the descriptors), so
// one graph serves every slice of that direction and parity.
static int slice_graph(pqmc_batch* b, int g, bool forward, int parity, pqmc_batch::SliceGraph** out) {
  const int key[6] = {g, forward ? 1 : 0, parity, b->kd, b->flush_mode, b->qc};
  for (auto& e : b->gcache)
    if (std::equal(key, key + 6, e.key)) {
      *out = &e;
      return PQMC_OK;
    }
  cudaStream_t st = b->g_stream[g];
  const int64_t n0 = g_launches.load();
  PQMC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = slice_ops(b, g, forward, parity);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &graph);
  const int n_kernels = (int)(g_launches.load() - n0);
  count_launch(-n_kernels);   // counted again at every replay
  if (rc != PQMC_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) {
    set_error("slice graph capture: %s", cudaGetErrorString(ec));
    return PQMC_ERR_CUDA;
  }
  pqmc_batch::SliceGraph e{};
  std::copy(key, key + 6, e.key);
  e.kernels = n_kernels;
  const cudaError_t ei =
      cudaGraphInstantiate(&e.exec, graph, b->prio_mask ? (unsigned long long)cudaGraphInstantiateFlagUseNodePriority : 0ull);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    set_error("slice graph instantiate: %s", cudaGetErrorString(ei));
    return PQMC_ERR_CUDA;
  }
  b->gcache.push_back(e);
  *out = &b->gcache.back();
  return PQMC_OK;
}

static void drop_graphs(pqmc_batch* b) {
  for (auto& e : b->gcache) cudaGraphExecDestroy(e.exec);
  b->gcache.clear();
}

// one slice of group g at 1-based `time`: its time index goes to the
// descriptors, then the family steps run as a graph replay or as launches
static int group_slice(pqmc_batch* b, int g, bool forward, int time, int parity) {
  cudaStream_t st = b->g_stream[g];
  const int C = b->g_count[g];
  k_bsettime<<<(C + 127) / 128, 128, 0, st>>>(b->d_desc + b->g_first[g], C, time - 1);
  PQMC_LAUNCHED();
  if (b->graphs && !b->timing) {
    pqmc_batch::SliceGraph* e = nullptr;
    PQMC_TRY(slice_graph(b, g, forward, parity, &e));
    PQMC_CUDA(cudaGraphLaunch(e->exec, st));
    count_launch(e->kernels);
    return PQMC_OK;
  }
  return slice_ops(b, g, forward, parity);
}

// stabilised recompute of group g (the caller flips the parity)
static int bscratch(pqmc_batch* b, int g, int time, bool forward, int parity) {
  cudaEvent_t tr = gphase_begin(b, g);
  PQMC_TRY(b->rec[g].scratch(time, forward, parity));
  gphase_end(b, g, PQMC_PHASE_RECOMPUTE, tr);
  return PQMC_OK;
}

// every group stream waits for the work queued on the batch stream so far
static int groups_fork(pqmc_batch* b) {
  if (b->n_groups < 2) return PQMC_OK;
  PQMC_CUDA(cudaEventRecord(b->ev_fork, b->stream));
  for (int g = 1; g < b->n_groups; ++g) PQMC_CUDA(cudaStreamWaitEvent(b->g_stream[g], b->ev_fork, 0));
  return PQMC_OK;
}
// the batch stream waits for every group stream
static int groups_join(pqmc_batch* b) {
  for (int g = 1; g < b->n_groups; ++g) {
    PQMC_CUDA(cudaEventRecord(b->ev_join[g], b->g_stream[g]));
    PQMC_CUDA(cudaStreamWaitEvent(b->stream, b->ev_join[g], 0));
  }
  return PQMC_OK;
}

// ms_begin_measure for every chain at `time` (src/mod_meas.f90:729-763): the
// groups join, the current G goes back to FP64 for the measurement kernels of
// each chain, and returns to double-float afterwards
static int batch_measure(pqmc_batch* b, int time, bool forward) {
  pqmc_chain* c0 = b->chains[0];
  const int half = c0->ntime / 2, mn = b->meas_number;
  PQMC_TRY(groups_join(b));
  const long ng2 = (long)c0->ns * c0->ns;
  const dim3 cgrid((unsigned)std::min<long>((ng2 + 255) / 256, 64), (unsigned)b->chains.size());
  k_gconv<<<cgrid, 256, 0, b->stream>>>(b->d_desc, 0, ng2, b->parity);
  PQMC_LAUNCHED();
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  const bool last = (forward && time == half + mn) || (!forward && time == half - mn);
  for (size_t i = 0; i < b->chains.size(); ++i) {
    pqmc_chain* c = b->chains[i];
    if (!c->have_meas) continue;
    cplx* gsave = c->g;
    c->g = b->parity ? c->g_alt : c->g;
    int st = do_measure(c, time);
    if (st == PQMC_OK && last) {
      const int W = PQMC_N_SCALAR + 2 * PQMC_N_FIELD * c->n_cell;
      st = do_finish_record(c, mn);
      if (st == PQMC_OK) {
        std::vector<double>& rec = b->records[i];
        const size_t at = rec.size();
        rec.resize(at + 2 * (size_t)W);
        if (cudaMemcpyAsync(rec.data() + at, c->m_acc, sizeof(cplx) * W, cudaMemcpyDeviceToHost, c->stream) !=
                cudaSuccess ||
            cudaMemsetAsync(c->m_acc, 0, sizeof(cplx) * W, c->stream) != cudaSuccess)
          st = PQMC_ERR_CUDA;
      }
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && st == PQMC_OK) st = PQMC_ERR_CUDA;
    c->g = gsave;
    if (st != PQMC_OK) {
      set_error("batch measurement failed on chain %zu", i);
      return st;
    }
  }
  k_gconv<<<cgrid, 256, 0, b->stream>>>(b->d_desc, 1, ng2, b->parity);
  PQMC_LAUNCHED();
  return groups_fork(b);
}

// An FP64 batch runs the single-chain path of every chain; the chains are
// independent (own buffers, own stream), so worker threads drive them
// concurrently and their kernels overlap on the device.  The first failure
// is reported with its message on the calling thread.
static int fp64_each(pqmc_batch* b, const std::function<int(pqmc_chain*)>& fn) {
  const int n = (int)b->chains.size();
  int nw = 8;
  if (const char* env = getenv("PQMC_BATCH_THREADS")) nw = atoi(env);
  nw = std::max(1, std::min(nw, n));
  if (nw == 1) {
    for (auto* c : b->chains) PQMC_TRY(fn(c));
    return PQMC_OK;
  }
  std::atomic<int> next{0}, status{PQMC_OK};
  std::string msg;
  std::atomic_flag have_msg = ATOMIC_FLAG_INIT;
  auto work = [&]() {
    for (int i = next++; i < n && status.load() == PQMC_OK; i = next++) {
      const int st = fn(b->chains[i]);
      if (st != PQMC_OK) {
        int ok = PQMC_OK;
        if (status.compare_exchange_strong(ok, st) && !have_msg.test_and_set()) msg = pqmc_last_error();
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < nw; ++t) pool.emplace_back(work);
  for (auto& t : pool) t.join();
  if (status.load() != PQMC_OK) set_error("%s", msg.c_str());
  return status.load();
}

// geometry of a mixed batch: chains of one class share every launch shape
static bool same_geometry(const pqmc_model* a, const pqmc_model* b) {
  if (a->ns != b->ns || a->nelec != b->nelec || a->ntime != b->ntime || a->ngroup != b->ngroup ||
      a->n_pf != b->n_pf || a->max_dim != b->max_dim || a->max_pla != b->max_pla || a->n_bf != b->n_bf ||
      a->local_update != b->local_update)
    return false;
  for (int f = 0; f < a->n_pf; ++f)
    if (a->pf_dim[f] != b->pf_dim[f] || a->pf_npla[f] != b->pf_npla[f] || a->pf_v_exist[f] != b->pf_v_exist[f])
      return false;
  return true;
}

extern "C" int pqmc_batch_destroy(pqmc_batch* b);
extern "C" int pqmc_batch_create(const pqmc_model* const* models, int n_chains, int precision, pqmc_batch** out);

// an uneven mixed batch: one homogeneous batch per geometry class, each with
// its own streams, chain groups, delay depth and graphs
static int create_uneven(const pqmc_model* const* models, int n_chains, const std::vector<int>& cls, int n_cls,
                         pqmc_batch** out) {
  pqmc_batch* b = new pqmc_batch();
  b->precision = PQMC_PREC_MIXED;
  b->part_of.assign(n_chains, 0);
  b->index_in_part.assign(n_chains, 0);
  for (int k = 0; k < n_cls; ++k) {
    std::vector<const pqmc_model*> sub;
    for (int i = 0; i < n_chains; ++i)
      if (cls[i] == k) {
        b->part_of[i] = k;
        b->index_in_part[i] = (int)sub.size();
        sub.push_back(models[i]);
      }
    pqmc_batch* part = nullptr;
    const int st = pqmc_batch_create(sub.data(), (int)sub.size(), PQMC_PREC_MIXED, &part);
    if (st != PQMC_OK) {
      pqmc_batch_destroy(b);
      return st;
    }
    b->parts.push_back(part);
  }
  for (int i = 0; i < n_chains; ++i) b->chains.push_back(b->parts[b->part_of[i]]->chains[b->index_in_part[i]]);
  PQMC_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  PQMC_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  int groups = 0;
  for (auto* p : b->parts) groups += p->n_groups;
  b->n_groups = groups;
  b->kd = b->parts[0]->kd;
  b->flush_mode = b->parts[0]->flush_mode;
  b->graphs = b->parts[0]->graphs;
  *out = b;
  return PQMC_OK;
}

extern "C" {

int pqmc_batch_create(const pqmc_model* const* models, int n_chains, int precision, pqmc_batch** out) {
  if (!models || !out || n_chains < 1) { set_error("batch_create: bad arguments"); return PQMC_ERR_ARG; }
  if (precision != PQMC_PREC_FP64 && precision != PQMC_PREC_MIXED) {
    set_error("batch_create: unknown precision %d", precision);
    return PQMC_ERR_ARG;
  }
  if (precision == PQMC_PREC_MIXED) {
    // chains of more than one geometry: one class per geometry
    std::vector<int> cls(n_chains, -1);
    std::vector<int> rep;   // first chain of each class
    for (int i = 0; i < n_chains; ++i) {
      if (!models[i]) { set_error("batch_create: null model %d", i); return PQMC_ERR_ARG; }
      for (size_t k = 0; k < rep.size() && cls[i] < 0; ++k)
        if (same_geometry(models[i], models[rep[k]])) cls[i] = (int)k;
      if (cls[i] < 0) {
        cls[i] = (int)rep.size();
        rep.push_back(i);
      }
    }
    if (rep.size() > 1) return create_uneven(models, n_chains, cls, (int)rep.size(), out);
  }
  pqmc_batch* b = new pqmc_batch();
  b->precision = precision;
  b->graphs = precision == PQMC_PREC_MIXED;   // slice graphs on by default
  for (int i = 0; i < n_chains; ++i) {
    pqmc_chain* c = nullptr;
    int st = pqmc_create(models[i], &c);
    if (st != PQMC_OK) {
      for (auto* x : b->chains) pqmc_destroy(x);
      delete b;
      return st;
    }
    c->in_batch = true;
    b->chains.push_back(c);
  }
  pqmc_chain* c0 = b->chains[0];
  if (precision == PQMC_PREC_MIXED) {
    for (auto* c : b->chains)
      if (c->ns != c0->ns || c->n_pf != c0->n_pf || c->ntime != c0->ntime || c->ngroup != c0->ngroup ||
          c->h_pf_npla != c0->h_pf_npla || c->h_pf_dim != c0->h_pf_dim) {
        set_error("batch_create: mixed-precision batches need chains of one geometry");
        pqmc_batch_destroy(b);
        return PQMC_ERR_ARG;
      }
  }
  if (precision == PQMC_PREC_MIXED) {
    // a slice's proposals can all be formed at its start when no boson is
    // shared by two families (a family's moves then change nothing the
    // other families' proposals read)
    bool disjoint = true;
    for (int i = 0; i < n_chains && disjoint; ++i) {
      const pqmc_model* m = models[i];
      std::vector<int> owner(m->n_bf, -1);
      for (int f = 0; f < m->n_pf && disjoint; ++f)
        for (int q = 0; q < m->pf_npla[f]; ++q) {
          const int bf = m->bf_list[q + m->max_pla * f];
          if (bf < 0 || bf >= m->n_bf) continue;
          if (owner[bf] >= 0 && owner[bf] != f) { disjoint = false; break; }
          owner[bf] = f;
        }
    }
    b->slice_prep = disjoint;
  }
  PQMC_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  int kmax = 0;
  for (int f = 0; f < c0->n_pf; ++f) kmax = std::max(kmax, c0->h_pf_npla[f] * c0->h_pf_dim[f]);
  if (kmax > SCAN_KSTAGE) {
    set_error("batch_create: family too large for the staged panels");
    pqmc_batch_destroy(b);
    return PQMC_ERR_ARG;
  }
  const int ldp = (c0->ns + 1) & ~1;
  if (precision == PQMC_PREC_MIXED) {
    if (c0->ns > SCAN_RPT * SCAN_THREADS) {
      set_error("batch_create: mixed precision supports Ns <= %d", SCAN_RPT * SCAN_THREADS);
      pqmc_batch_destroy(b);
      return PQMC_ERR_ARG;
    }
    int max_pla = 0, dev = 0, optin = 0;
    for (int f = 0; f < c0->n_pf; ++f) max_pla = std::max(max_pla, c0->h_pf_npla[f]);
    PQMC_CUDA(cudaGetDevice(&dev));
    PQMC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t stat = 4096;   // static shared memory of k_bscan (descriptor, per-warp R and T, barriers)
    // rows of G by TMA boxes of rb columns (rb a multiple of 8: 128-byte aligned boxes)
    const int nrb = (c0->ns + 255) / 256;
    const int rb = (((c0->ns + nrb - 1) / nrb) + 7) & ~7;
    const int rows_bytes = 4 * nrb * rb * (int)sizeof(float4);
    int qc = 8;
    while (qc > 1 && scan_layout(max_pla, c0->ns, ldp, qc, SCAN_KSTAGE, rows_bytes).total + stat > (size_t)optin) --qc;
    const size_t need = scan_layout(max_pla, c0->ns, ldp, qc, SCAN_KSTAGE, rows_bytes).total;
    if (need + stat > (size_t)optin) {
      set_error("batch_create: scan staging needs %zu bytes of shared memory, the device offers %d", need + stat,
                optin);
      pqmc_batch_destroy(b);
      return PQMC_ERR_ARG;
    }
    b->qc = qc;
    b->qc_max = qc;
    // tensor maps over every chain's two G buffers (double-float: 4 FP32 per element)
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      set_error("batch_create: cuTensorMapEncodeTiled unavailable");
      pqmc_batch_destroy(b);
      return PQMC_ERR_CUDA;
    }
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    std::vector<CUtensorMap> maps(2 * (size_t)n_chains);
    b->tm_buf.resize(2 * (size_t)n_chains);
    for (int i = 0; i < n_chains; ++i)
      for (int k = 0; k < 2; ++k) {
        cplx* buf = k == 0 ? b->chains[i]->g : b->chains[i]->g_alt;
        b->tm_buf[2 * i + k] = buf;
        const cuuint64_t dims[2] = {4ull * (cuuint64_t)c0->ns, (cuuint64_t)c0->ns};
        const cuuint64_t strides[1] = {16ull * (cuuint64_t)c0->ns};
        const cuuint32_t box[2] = {4u, (cuuint32_t)rb};
        const cuuint32_t estr[2] = {1u, 1u};
        const CUresult r = encode(&maps[2 * i + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)buf, dims, strides, box,
                                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
          set_error("batch_create: cuTensorMapEncodeTiled failed (%d)", (int)r);
          pqmc_batch_destroy(b);
          return PQMC_ERR_CUDA;
        }
      }
    PQMC_CUDA(cudaMalloc((void**)&b->d_tmaps, sizeof(CUtensorMap) * maps.size()));
    PQMC_CUDA(cudaMemcpy(b->d_tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
    b->rb = rb;
    b->nrb = nrb;
#define PQMC_SMEM(DM, R) PQMC_CUDA(raise_dyn_smem(k_bscan<DM, R>, (int)need))
    PQMC_SMEM(1, 1); PQMC_SMEM(2, 1); PQMC_SMEM(3, 1); PQMC_SMEM(4, 1);
    PQMC_SMEM(1, 2); PQMC_SMEM(2, 2); PQMC_SMEM(3, 2); PQMC_SMEM(4, 2);
#undef PQMC_SMEM
  }
  PQMC_CUDA(cudaMalloc((void**)&b->d_err, sizeof(int)));
  PQMC_CUDA(cudaMemset(b->d_err, 0, sizeof(int)));
  if (precision == PQMC_PREC_MIXED) {
    // tcgen05 flush: split operand images (zero outside the rows and columns of G)
    const size_t ib = um_chain_bytes(c0->ns) * (size_t)n_chains;
    PQMC_CUDA(cudaMalloc((void**)&b->d_img, ib));
    PQMC_CUDA(cudaMemset(b->d_img, 0, ib));
    PQMC_CUDA(raise_dyn_smem(k_bflush_um, 6 * UM_HALF));
    // wrap with whole columns staged in shared memory where they fit
    // (PQMC_WRAP_COLS=0 keeps the gather form)
    {
      // the family step's chain of kernels (scan, split, flush) ahead of
      // the other groups' wraps and recompute GEMMs when SMs free up: a
      // group's scan is one CTA per chain on its sequential path
      // (PQMC_PRIORITY=0 launches everything at the default priority)
      const char* penv = getenv("PQMC_PRIORITY");
      b->prio_mask = penv ? atoi(penv) & 3 : 3;
      int lo = 0, hi = 0;
      PQMC_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      b->prio_hi = hi;
    }
    const char* denv = getenv("PQMC_WRAP_DF");
    b->wrap_df_mode = denv ? (atoi(denv) != 0 ? 1 : 0) : -1;
    const char* wenv = getenv("PQMC_WRAP_COLS");
    const bool wc_on = !(wenv && atoi(wenv) == 0);
    b->wrap_cols.assign(c0->n_pf, 0);
    b->wrap_ci = wc_on ? WRAPC_C_DEFAULT : 0;
    for (int f = 0; f < c0->n_pf && wc_on; ++f) {
      const int dim = c0->h_pf_dim[f];
      if (dim < 1 || dim > 4) continue;
      for (int ci = 1; ci <= 2; ++ci) {   // the staged tiles whose columns fit
        const size_t sm = wrapc_smem(c0->ns, c0->wrap[f].n_items, dim, ci);
        if (sm > WRAPC_MAX_SMEM) break;
        PQMC_CUDA(raise_wrapc(dim, ci, (int)sm));
        b->wrap_cols[f] = (char)ci;
      }
    }
  }
  b->h_desc.resize(n_chains);
  for (int i = 0; i < n_chains; ++i) {
    pqmc_chain* c = b->chains[i];
    BDesc& h = b->h_desc[i];
    memset(&h, 0, sizeof(h));
    h.M = c->M;
    h.field = c->field;
    h.expkv = c->expkv;
    h.expkv_inv = c->expkv_inv;
    h.g = c->g;
    h.g_alt = c->g_alt;
    h.kmax = kmax;
    h.ldp = ldp;
    h.rb = b->rb;
    h.nrb = b->nrb;
    h.err = b->d_err;
    h.pre = c->pre;
    if (precision == PQMC_PREC_MIXED) {
      PlaqPre* pa = nullptr;
      PQMC_CUDA(cudaMalloc((void**)&pa, sizeof(PlaqPre) * (size_t)c->n_pf * c->max_pla));
      b->pre_all.push_back(pa);
      h.pre = pa;
    }
    h.sc = c->sc;
    float2* pan = nullptr;
    int* kc = nullptr;
    if (precision == PQMC_PREC_MIXED) {
      PQMC_CUDA(cudaMalloc((void**)&pan, sizeof(float2) * (size_t)2 * kmax * ldp));
      PQMC_CUDA(cudaMalloc((void**)&kc, sizeof(int)));
      h.A = pan;
      h.B = pan + (size_t)kmax * ldp;
      h.kcount = kc;
    }
    b->panels.push_back(pan);
    b->kcounts.push_back(kc);
  }
  PQMC_CUDA(cudaMalloc((void**)&b->d_nflush, sizeof(unsigned long long) * n_chains));
  PQMC_CUDA(cudaMemset(b->d_nflush, 0, sizeof(unsigned long long) * n_chains));
  for (int i = 0; i < n_chains; ++i) b->h_desc[i].nflush = b->d_nflush + i;
  PQMC_CUDA(cudaMalloc((void**)&b->d_scanprof, sizeof(unsigned long long) * 3 * n_chains));
  PQMC_CUDA(cudaMemset(b->d_scanprof, 0, sizeof(unsigned long long) * 3 * n_chains));
  for (int i = 0; i < n_chains; ++i) b->h_desc[i].scan_prof = b->d_scanprof + 3 * i;
  if (precision == PQMC_PREC_MIXED) {
    // the exact round update: accepted-move records and slice images per
    // chain (images zero outside the rows and columns of G)
    PQMC_TRY(exact_setup());
    const size_t acc_b = (size_t)UM_KP * (sizeof(int) + 16 * sizeof(float4)) +
                         (size_t)UM_KP * UM_KP * (sizeof(float4) + sizeof(float2));
    const size_t xib = oz_chain_bytes(c0->ns);
    PQMC_CUDA(cudaMalloc((void**)&b->d_acc, acc_b * n_chains));
    PQMC_CUDA(cudaMalloc((void**)&b->d_ximg, xib * n_chains));
    PQMC_CUDA(cudaMemset(b->d_ximg, 0, xib * n_chains));
    b->h_xdesc.resize(n_chains);
    for (int i = 0; i < n_chains; ++i) {
      pqmc_chain* c = b->chains[i];
      BDesc& h = b->h_desc[i];
      unsigned char* a = b->d_acc + acc_b * i;   // float4 parts first (alignment)
      h.acc_delta = reinterpret_cast<float4*>(a);
      float4* wdf = h.acc_delta + (size_t)UM_KP * 16;
      float2* v0 = reinterpret_cast<float2*>(wdf + (size_t)UM_KP * UM_KP);
      h.acc_site = reinterpret_cast<int*>(v0 + (size_t)UM_KP * UM_KP);
      XDesc& x = b->h_xdesc[i];
      memset(&x, 0, sizeof(x));
      x.g = reinterpret_cast<float4*>(c->g);
      x.g_alt = reinterpret_cast<float4*>(c->g_alt);
      x.ns = c->ns;
      x.ncopy = c->M.ncopy;
      x.tr_weight = c->M.tr_weight;
      x.kmax = UM_KP;
      x.kcount = h.kcount;
      x.acc_site = h.acc_site;
      x.acc_delta = h.acc_delta;
      x.wdf = wdf;
      x.v0 = v0;
      x.img = b->d_ximg + xib * i;
      x.sc = c->sc;
      x.err = b->d_err;
      x.nflush = b->d_nflush + i;
    }
    int max_items = 0;
    for (int f = 0; f < c0->n_pf; ++f) max_items = std::max(max_items, c0->wrap[f].n_items);
    PQMC_CUDA(cudaMalloc((void**)&b->d_wtab, sizeof(float4) * 2 * 16 * (size_t)max_items * n_chains));
    PQMC_CUDA(cudaMalloc((void**)&b->d_xdesc, sizeof(XDesc) * n_chains));
    PQMC_CUDA(cudaMemcpy(b->d_xdesc, b->h_xdesc.data(), sizeof(XDesc) * n_chains, cudaMemcpyHostToDevice));
  }
  PQMC_CUDA(cudaMalloc((void**)&b->d_desc, sizeof(BDesc) * n_chains));
  PQMC_CUDA(cudaMalloc((void**)&b->d_next, sizeof(int) * n_chains));
  // chain groups: PQMC_BATCH_GROUPS (1..16) when set, else one per 8 chains
  // (at most 8)
  {
    int ng = precision == PQMC_PREC_MIXED ? std::min(n_chains / 8, 8) : 1;
    const char* env = getenv("PQMC_BATCH_GROUPS");
    if (env && precision == PQMC_PREC_MIXED) ng = atoi(env);
    ng = std::max(1, std::min(std::min(ng, (int)pqmc_batch::MAX_GROUPS), n_chains));
    b->n_groups = ng;
  }
  b->g_stream[0] = b->stream;
  for (int g = 0, first = 0; g < b->n_groups; ++g) {
    const int cnt = (n_chains - first) / (b->n_groups - g);
    b->g_first[g] = first;
    b->g_count[g] = cnt;
    first += cnt;
    if (g > 0) PQMC_CUDA(cudaStreamCreateWithFlags(&b->g_stream[g], cudaStreamNonBlocking));
    PQMC_CUDA(cudaEventCreateWithFlags(&b->ev_join[g], cudaEventDisableTiming));
  }
  PQMC_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  if (precision == PQMC_PREC_MIXED)
    for (int g = 0; g < b->n_groups; ++g) {
      std::vector<pqmc_chain*> sub(b->chains.begin() + b->g_first[g],
                                   b->chains.begin() + b->g_first[g] + b->g_count[g]);
      PQMC_TRY(b->rec[g].setup(sub, b->g_stream[g]));
      b->rec[g].err = b->d_err;
    }
  PQMC_TRY(batch_refresh(b));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  *out = b;
  return PQMC_OK;
}

int pqmc_batch_destroy(pqmc_batch* b) {
  if (!b) return PQMC_OK;
  if (!b->parts.empty() || !b->part_of.empty()) {
    for (auto* p : b->parts) pqmc_batch_destroy(p);   // the chains belong to the classes
    b->parts.clear();
    b->chains.clear();
  }
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& m : b->marks) {
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  for (auto e : b->ev_pool) cudaEventDestroy(e);
  drop_graphs(b);
  for (auto* c : b->chains) pqmc_destroy(c);
  for (auto* p : b->panels)
    if (p) cudaFree(p);
  for (auto* k : b->kcounts)
    if (k) cudaFree(k);
  for (auto* pa : b->pre_all)
    if (pa) cudaFree(pa);
  if (b->h_states) cudaFreeHost(b->h_states);
  if (b->d_nflush) cudaFree(b->d_nflush);
  if (b->d_scanprof) cudaFree(b->d_scanprof);
  if (b->d_desc) cudaFree(b->d_desc);
  if (b->d_next) cudaFree(b->d_next);
  if (b->d_err) cudaFree(b->d_err);
  if (b->d_img) cudaFree(b->d_img);
  if (b->d_xdesc) cudaFree(b->d_xdesc);
  if (b->d_wtab) cudaFree(b->d_wtab);
  if (b->d_ximg) cudaFree(b->d_ximg);
  if (b->d_acc) cudaFree(b->d_acc);
  if (b->d_tmaps) cudaFree(b->d_tmaps);
  for (int g = 1; g < pqmc_batch::MAX_GROUPS; ++g)
    if (b->g_stream[g]) {
      cudaStreamSynchronize(b->g_stream[g]);
      cudaStreamDestroy(b->g_stream[g]);
    }
  for (int g = 0; g < pqmc_batch::MAX_GROUPS; ++g)
    if (b->ev_join[g]) cudaEventDestroy(b->ev_join[g]);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PQMC_OK;
}

int pqmc_batch_set_flush(pqmc_batch* b, int mode) {
  if (!b || mode < 0 || mode > 2) {
    set_error("batch_set_flush: mode 0 (mma.sync), 1 (tcgen05) or 2 (exact round update)");
    return PQMC_ERR_ARG;
  }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_flush(p, mode));
  b->flush_mode = mode;
  return PQMC_OK;
}

int pqmc_batch_set_wrap_tile(pqmc_batch* b, int ci) {
  if (!b || ci < 0 || ci > 2) {
    set_error("batch_set_wrap_tile: 0 (gathered blocks), 1 or 2 (column items per CTA)");
    return PQMC_ERR_ARG;
  }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_wrap_tile(p, ci));
  if (b->wrap_ci != ci) {   // the slice graphs hold the old wrap launches
    PQMC_CUDA(cudaStreamSynchronize(b->stream));
    drop_graphs(b);
  }
  b->wrap_ci = ci;
  return PQMC_OK;
}

int pqmc_batch_get_wrap_tile(pqmc_batch* b, int* ci) {
  if (!b || !ci) { set_error("null argument"); return PQMC_ERR_ARG; }
  *ci = b->parts.empty() ? b->wrap_ci : b->parts[0]->wrap_ci;
  return PQMC_OK;
}

int pqmc_batch_set_flush_tile(pqmc_batch* b, int ct) {
  if (!b || (ct != 32 && ct != 64 && ct != 1 && ct != 2)) {
    set_error("batch_set_flush_tile: 64 or 32 columns per CTA, or the pipeline with 1 or 2 CTAs per row tile");
    return PQMC_ERR_ARG;
  }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_flush_tile(p, ct));
  if (b->xflush_ct != ct) {   // the slice graphs hold the old launches
    PQMC_CUDA(cudaStreamSynchronize(b->stream));
    drop_graphs(b);
  }
  b->xflush_ct = ct;
  return PQMC_OK;
}

int pqmc_batch_get_flush_tile(pqmc_batch* b, int* ct) {
  if (!b || !ct) { set_error("null argument"); return PQMC_ERR_ARG; }
  *ct = b->parts.empty() ? b->xflush_ct : b->parts[0]->xflush_ct;
  return PQMC_OK;
}

int pqmc_batch_set_gemm_engine(pqmc_batch* b, int engine) {
  if (!b || (engine != 0 && engine != 1)) {
    set_error("batch_set_gemm_engine: 0 (double-float, FP32 pipe) or 1 (Ozaki, tensor cores)");
    return PQMC_ERR_ARG;
  }
  if (b->precision != PQMC_PREC_MIXED) {
    set_error("batch_set_gemm_engine: mixed batches only (the FP64 batch recomputes with its chains' own path)");
    return PQMC_ERR_ARG;
  }
  if (!b->parts.empty()) {   // the classes hold the recomputes
    for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_gemm_engine(p, engine));
    return PQMC_OK;
  }
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  for (int g = 0; g < b->n_groups; ++g) PQMC_TRY(b->rec[g].set_engine(engine));
  return PQMC_OK;
}

int pqmc_batch_get_gemm_engine(pqmc_batch* b, int* engine) {
  if (!b || !engine) { set_error("null argument"); return PQMC_ERR_ARG; }
  *engine = b->parts.empty() ? b->rec[0].engine : b->parts[0]->rec[0].engine;
  return PQMC_OK;
}

int pqmc_batch_set_scan_chunk(pqmc_batch* b, int qc) {
  if (!b || qc < 1) {
    set_error("batch_set_scan_chunk: a chunk of at least one panel column");
    return PQMC_ERR_ARG;
  }
  if (!b->parts.empty()) {
    for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_scan_chunk(p, qc));
    return PQMC_OK;
  }
  if (qc > b->qc_max) {
    set_error("batch_set_scan_chunk: %d panel columns per chunk do not fit in shared memory (at most %d)", qc,
              b->qc_max);
    return PQMC_ERR_ARG;
  }
  if (b->qc != qc) {   // the slice graphs hold the old launches
    PQMC_CUDA(cudaStreamSynchronize(b->stream));
    drop_graphs(b);
  }
  b->qc = qc;
  return PQMC_OK;
}

int pqmc_batch_get_scan_chunk(pqmc_batch* b, int* qc, int* qc_max) {
  if (!b || !qc) { set_error("null argument"); return PQMC_ERR_ARG; }
  const pqmc_batch* p = b->parts.empty() ? b : b->parts[0];
  *qc = p->qc;
  if (qc_max) *qc_max = p->qc_max;
  return PQMC_OK;
}

// candidates of pqmc_batch_autotune_tiles, in ms_out order
static const int TILE_WRAP[3] = {0, 1, 2};
static const int TILE_FLUSH[4] = {64, 32, 2, 1};
// the scan chunks tried: the largest that fits, about three quarters and half of it
static inline int tile_qc(int qc_max, int i) { return i == 0 ? qc_max : i == 1 ? (3 * qc_max + 3) / 4 : (qc_max + 1) / 2; }
constexpr int TILE_N = 10;   // entries of ms_out: 3 wrap, 4 flush, 3 scan-chunk slots

int pqmc_batch_autotune_tiles(pqmc_batch* b, int loop, int first_tc, int n_slices, int* best, double* ms_out) {
  if (!b || n_slices < 1 || !best) { set_error("batch_autotune_tiles: bad arguments"); return PQMC_ERR_ARG; }
  if (b->precision != PQMC_PREC_MIXED) { set_error("batch_autotune_tiles: mixed batches only"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {   // every class tunes its own tiles; ms_out sums the classes
    double part_ms[TILE_N];
    if (ms_out)
      for (int i = 0; i < TILE_N; ++i) ms_out[i] = 0.0;
    for (size_t k = 0; k < b->parts.size(); ++k) {
      int bk[3] = {0, 0, 0};
      PQMC_TRY(pqmc_batch_autotune_tiles(b->parts[k], loop, first_tc, n_slices, bk, part_ms));
      if (k == 0)
        for (int i = 0; i < 3; ++i) best[i] = bk[i];
      if (ms_out)
        for (int i = 0; i < TILE_N; ++i)
          ms_out[i] = (ms_out[i] < 0.0 || part_ms[i] < 0.0) ? -1.0 : ms_out[i] + part_ms[i];
    }
    return PQMC_OK;
  }
  const int nt = b->chains[0]->ntime;
  int max_ci = 0;
  for (char v : b->wrap_cols) max_ci = std::max(max_ci, (int)v);
  cudaEvent_t e0, e1;
  PQMC_CUDA(cudaEventCreate(&e0));
  PQMC_CUDA(cudaEventCreate(&e1));
  const bool graphs = b->graphs;
  b->graphs = false;   // plain launches for every candidate, as in pqmc_batch_autotune
  int lp = loop, tc = first_tc, st = PQMC_OK;
  auto time_slices = [&](double* out) {
    const int n = std::min(n_slices, nt - tc + 1);
    cudaEventRecord(e0, b->stream);
    st = pqmc_batch_sweep_slices(b, lp, tc, n);
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *out = ms / n;
    tc += n;
    if (tc > nt) { tc = 1; ++lp; }
  };
  // the wrap tile, then the exact round update's flush tile at the best wrap
  double best_ms = 1e300;
  int best_ci = b->wrap_ci;
  // every candidate slot runs its n_slices, so that every class of an uneven
  // batch ends on the same slice: a shape that does not fit runs them at the
  // best shape so far and reports -1
  for (int i = 0; i < 3 && st == PQMC_OK; ++i) {
    double v = -1.0;
    const bool fits = TILE_WRAP[i] <= max_ci;
    b->wrap_ci = fits ? TILE_WRAP[i] : best_ci;
    time_slices(&v);
    if (fits && v < best_ms) { best_ms = v; best_ci = TILE_WRAP[i]; }
    if (ms_out) ms_out[i] = fits ? v : -1.0;
  }
  b->wrap_ci = best_ci;
  best_ms = 1e300;
  int best_ct = b->xflush_ct;
  for (int i = 0; i < 4 && st == PQMC_OK; ++i) {
    double v = -1.0;
    if (b->flush_mode == 2) {
      b->xflush_ct = TILE_FLUSH[i];
      time_slices(&v);
      if (v < best_ms) { best_ms = v; best_ct = TILE_FLUSH[i]; }
    }
    if (ms_out) ms_out[3 + i] = v;
  }
  b->xflush_ct = best_ct;
  // the scan's panel chunk at the best wrap and flush tiles
  best_ms = 1e300;
  int best_qc = b->qc;
  for (int i = 0; i < 3 && st == PQMC_OK; ++i) {
    double v = -1.0;
    b->qc = tile_qc(b->qc_max, i);
    time_slices(&v);
    if (v < best_ms) { best_ms = v; best_qc = b->qc; }
    if (ms_out) ms_out[7 + i] = v;
  }
  b->qc = best_qc;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->graphs = graphs;
  if (st != PQMC_OK) return st;
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  drop_graphs(b);
  best[0] = best_ci;
  best[1] = best_ct;
  best[2] = best_qc;
  return PQMC_OK;
}

int pqmc_batch_set_graphs(pqmc_batch* b, int enable) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  if (enable && b->precision != PQMC_PREC_MIXED) {
    set_error("batch_set_graphs: slice graphs belong to mixed-precision batches");
    return PQMC_ERR_ARG;
  }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_graphs(p, enable));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  b->graphs = enable != 0;
  if (!b->graphs) drop_graphs(b);
  return PQMC_OK;
}

int pqmc_batch_graph_count(pqmc_batch* b, int* n) {
  if (!b || !n) { set_error("batch_graph_count: null argument"); return PQMC_ERR_ARG; }
  int total = (int)b->gcache.size();
  for (auto* p : b->parts) {
    int k = 0;
    PQMC_TRY(pqmc_batch_graph_count(p, &k));
    total += k;
  }
  *n = total;
  return PQMC_OK;
}

int pqmc_batch_set_delay(pqmc_batch* b, int kd) {
  if (!b || kd < 1 || kd > SCAN_KSTAGE) { set_error("batch_set_delay: depth must be in 1..%d", SCAN_KSTAGE); return PQMC_ERR_ARG; }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_delay(p, kd));
  b->kd = kd;
  return PQMC_OK;
}

int pqmc_batch_init(pqmc_batch* b) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {
    for (auto* p : b->parts) PQMC_TRY(pqmc_batch_init(p));
    return PQMC_OK;
  }
  for (auto* c : b->chains) PQMC_TRY(launch_init_expkv(c, 0, c->ntime));
  for (auto* c : b->chains) PQMC_CUDA(cudaStreamSynchronize(c->stream));
  pqmc_chain* c0 = b->chains[0];
  if (b->precision == PQMC_PREC_FP64 || c0->ntime % c0->ngroup != 0)
    return fp64_each(b, [](pqmc_chain* c) { return pqmc_init_g(c, 1); });
  for (int g = 0; g < b->n_groups; ++g) PQMC_TRY(b->rec[g].init_g());
  for (auto* c : b->chains) c->have_g = true;
  return batch_refresh(b);
}

int pqmc_batch_set_timing(pqmc_batch* b, int enable) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_timing(p, enable));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  PQMC_TRY(phase_resolve(b));
  b->timing = enable != 0;
  for (int k = 0; k < PQMC_N_PHASES; ++k) {
    b->phase_ms[k] = 0.0;
    b->phase_n[k] = 0;
  }
  if (b->d_nflush) PQMC_CUDA(cudaMemset(b->d_nflush, 0, sizeof(unsigned long long) * b->chains.size()));
  if (b->d_scanprof)
    PQMC_CUDA(cudaMemset(b->d_scanprof, 0, sizeof(unsigned long long) * 3 * b->chains.size()));
  return PQMC_OK;
}

int pqmc_batch_scan_profile(pqmc_batch* b, long long* out) {
  if (!b || !out) { set_error("batch_scan_profile: null argument"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {
    for (size_t k = 0; k < b->parts.size(); ++k) {
      std::vector<long long> pr(3 * b->parts[k]->chains.size());
      PQMC_TRY(pqmc_batch_scan_profile(b->parts[k], pr.data()));
      for (size_t i = 0; i < b->chains.size(); ++i)
        if (b->part_of[i] == (int)k)
          for (int q = 0; q < 3; ++q) out[3 * i + q] = pr[3 * b->index_in_part[i] + q];
    }
    return PQMC_OK;
  }
  const size_t n = b->chains.size();
  std::vector<unsigned long long> h(3 * n, 0ull);
  if (b->d_scanprof) {
    PQMC_CUDA(cudaStreamSynchronize(b->stream));
    for (int g = 1; g < b->n_groups; ++g) PQMC_CUDA(cudaStreamSynchronize(b->g_stream[g]));
    PQMC_CUDA(cudaMemcpy(h.data(), b->d_scanprof, sizeof(unsigned long long) * 3 * n, cudaMemcpyDeviceToHost));
  }
  for (size_t i = 0; i < 3 * n; ++i) out[i] = (long long)h[i];
  return PQMC_OK;
}

int pqmc_batch_flush_rounds(pqmc_batch* b, long long* rounds) {
  if (!b || !rounds) { set_error("batch_flush_rounds: null argument"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {
    for (size_t k = 0; k < b->parts.size(); ++k) {
      std::vector<long long> pr(b->parts[k]->chains.size());
      PQMC_TRY(pqmc_batch_flush_rounds(b->parts[k], pr.data()));
      for (size_t i = 0; i < b->chains.size(); ++i)
        if (b->part_of[i] == (int)k) rounds[i] = pr[b->index_in_part[i]];
    }
    return PQMC_OK;
  }
  const size_t n = b->chains.size();
  if (!b->d_nflush) {
    for (size_t i = 0; i < n; ++i) rounds[i] = 0;
    return PQMC_OK;
  }
  std::vector<unsigned long long> h(n);
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  for (int g = 1; g < b->n_groups; ++g) PQMC_CUDA(cudaStreamSynchronize(b->g_stream[g]));
  PQMC_CUDA(cudaMemcpy(h.data(), b->d_nflush, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n; ++i) rounds[i] = (long long)h[i];
  return PQMC_OK;
}

int pqmc_batch_get_timing(pqmc_batch* b, double* ms, long long* launches) {
  if (!b || !ms || !launches) { set_error("batch_get_timing: null argument"); return PQMC_ERR_ARG; }
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  PQMC_TRY(phase_resolve(b));
  for (int k = 0; k < PQMC_N_PHASES; ++k) {
    ms[k] = b->phase_ms[k];
    launches[k] = b->phase_n[k];
  }
  // an uneven batch: the sum over its classes (which overlap on the device)
  for (auto* p : b->parts) {
    double pm[PQMC_N_PHASES];
    long long pn[PQMC_N_PHASES];
    PQMC_TRY(pqmc_batch_get_timing(p, pm, pn));
    for (int k = 0; k < PQMC_N_PHASES; ++k) {
      ms[k] += pm[k];
      launches[k] += pn[k];
    }
  }
  return PQMC_OK;
}

int pqmc_batch_info(pqmc_batch* b, int* info) {
  if (!b || !info) { set_error("batch_info: null argument"); return PQMC_ERR_ARG; }
  info[0] = (int)b->chains.size();
  info[1] = b->n_groups;
  info[2] = b->kd;
  info[3] = b->flush_mode;
  info[4] = b->precision;
  return PQMC_OK;
}

int pqmc_batch_field_slices(pqmc_batch* b, int first_time, int n_times, double* host, int to_device) {
  if (!b || !host || first_time < 1 || n_times < 1) { set_error("batch_field_slices: bad arguments"); return PQMC_ERR_ARG; }
  // every chain's copy (and expKV refresh) is queued on its own stream
  // first; one wait per stream at the end
  size_t off = 0;
  for (auto* c : b->chains) {
    const int n = std::min(n_times, c->ntime - first_time + 1);
    if (n <= 0) continue;
    double* dev = c->field + (size_t)c->n_bf * (first_time - 1);
    const size_t bytes = sizeof(double) * (size_t)c->n_bf * n;
    if (to_device) {
      PQMC_CUDA(cudaMemcpyAsync(dev, host + off, bytes, cudaMemcpyHostToDevice, c->stream));
      PQMC_TRY(launch_init_expkv(c, first_time - 1, n));
    } else {
      PQMC_CUDA(cudaMemcpyAsync(host + off, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    }
    off += (size_t)c->n_bf * n;
  }
  for (auto* c : b->chains) PQMC_CUDA(cudaStreamSynchronize(c->stream));
  return PQMC_OK;
}

int pqmc_batch_states(pqmc_batch* b, pqmc_state* out) {
  if (!b || !out) { set_error("batch_states: null argument"); return PQMC_ERR_ARG; }
  const size_t n = b->chains.size();
  if (!b->h_states) PQMC_CUDA(cudaMallocHost((void**)&b->h_states, sizeof(DevScalars) * n));
  for (size_t i = 0; i < n; ++i)
    PQMC_CUDA(cudaMemcpyAsync(b->h_states + i, b->chains[i]->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost,
                              b->chains[i]->stream));
  for (auto* c : b->chains) PQMC_CUDA(cudaStreamSynchronize(c->stream));
  for (size_t i = 0; i < n; ++i) {
    const DevScalars& h = b->h_states[i];
    pqmc_state& o = out[i];
    o.ln_cw[0] = h.ln_cw.x;
    o.ln_cw[1] = h.ln_cw.y;
    o.err_fast_max = h.err_fast_max;
    o.err_fast = h.err_fast;
    o.err_g = h.err_g;
    o.err_g_rel_max = h.err_g_rel_max;
    o.positive_accept = h.pos_acc;
    o.negative_accept = h.neg_acc;
    for (int k = 0; k < 5; ++k) o.rng[k] = h.rng[k];
    o.reserved = 0;
  }
  return PQMC_OK;
}

int pqmc_batch_classes(pqmc_batch* b, int* n) {
  if (!b || !n) { set_error("batch_classes: null argument"); return PQMC_ERR_ARG; }
  *n = b->parts.empty() ? 1 : (int)b->parts.size();
  return PQMC_OK;
}

int pqmc_batch_class_info(pqmc_batch* b, int k, int* info) {
  if (!b || !info) { set_error("batch_class_info: null argument"); return PQMC_ERR_ARG; }
  const int n = b->parts.empty() ? 1 : (int)b->parts.size();
  if (k < 0 || k >= n) { set_error("batch_class_info: class %d of %d", k, n); return PQMC_ERR_ARG; }
  pqmc_batch* p = b->parts.empty() ? b : b->parts[k];
  info[0] = (int)p->chains.size();
  info[1] = p->chains[0]->ns;
  info[2] = p->chains[0]->ntime;
  info[3] = p->kd;
  info[4] = p->flush_mode;
  info[5] = p->n_groups;
  return PQMC_OK;
}

int pqmc_batch_stream(pqmc_batch* b, void** stream) {
  if (!b || !stream) { set_error("batch_stream: null argument"); return PQMC_ERR_ARG; }
  *stream = (void*)b->stream;
  return PQMC_OK;
}

int pqmc_batch_autotune(pqmc_batch* b, int loop, int first_tc, int n_slices, const int* candidates, int n_candidates,
                        int* best, double* ms_out) {
  if (!b || !candidates || n_candidates < 1 || n_slices < 1 || !best) {
    set_error("batch_autotune: bad arguments");
    return PQMC_ERR_ARG;
  }
  if (b->precision != PQMC_PREC_MIXED) { set_error("batch_autotune: mixed batches only"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {
    // every class tunes its own depth; ms_out sums the classes' ms per slice
    std::vector<double> part_ms(n_candidates);
    if (ms_out)
      for (int i = 0; i < n_candidates; ++i) ms_out[i] = 0.0;
    for (size_t k = 0; k < b->parts.size(); ++k) {
      int bk = 0;
      PQMC_TRY(pqmc_batch_autotune(b->parts[k], loop, first_tc, n_slices, candidates, n_candidates, &bk,
                                   part_ms.data()));
      if (k == 0) *best = bk;
      if (ms_out)
        for (int i = 0; i < n_candidates; ++i) ms_out[i] += part_ms[i];
    }
    b->kd = *best;
    b->flush_mode = b->parts[0]->flush_mode;
    return PQMC_OK;
  }
  pqmc_chain* c0 = b->chains[0];
  const int nt = c0->ntime;
  cudaEvent_t e0, e1;
  PQMC_CUDA(cudaEventCreate(&e0));
  PQMC_CUDA(cudaEventCreate(&e1));
  double best_ms = 1e300;
  int best_kd = b->kd;
  int lp = loop, tc = first_tc;
  int st = PQMC_OK;
  // candidates are timed with plain launches (a first capture would bias
  // the comparison); the graphs of the chosen depth are captured afterwards
  const bool graphs = b->graphs;
  b->graphs = false;
  for (int i = 0; i < n_candidates && st == PQMC_OK; ++i) {
    const int kd = candidates[i];
    if (kd < 1 || kd > SCAN_KSTAGE) { st = PQMC_ERR_ARG; set_error("batch_autotune: depth %d out of range", kd); break; }
    if (b->flush_mode == 2 && kd > UM_KP) {   // the exact update takes at most UM_KP columns
      if (ms_out) ms_out[i] = -1.0;
      continue;
    }
    b->kd = kd;
    const int n = std::min(n_slices, nt - tc + 1);
    cudaEventRecord(e0, b->stream);
    st = pqmc_batch_sweep_slices(b, lp, tc, n);
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per_slice = ms / n;
    if (ms_out) ms_out[i] = per_slice;
    if (per_slice < best_ms) { best_ms = per_slice; best_kd = kd; }
    tc += n;
    if (tc > nt) { tc = 1; ++lp; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->graphs = graphs;
  if (st != PQMC_OK) return st;
  b->kd = best_kd;
  if (b->flush_mode != 2) b->flush_mode = best_kd <= UM_KP ? 1 : 0;
  *best = best_kd;
  return PQMC_OK;
}

int pqmc_batch_set_measure(pqmc_batch* b, int warmup, int meas_interval, int meas_number) {
  if (!b || meas_interval < 1 || meas_number < 0) { set_error("batch_set_measure: bad arguments"); return PQMC_ERR_ARG; }
  if (!b->parts.empty()) {
    for (auto* p : b->parts) PQMC_TRY(pqmc_batch_set_measure(p, warmup, meas_interval, meas_number));
    b->meas_on = 1;
    return PQMC_OK;
  }
  pqmc_chain* c0 = b->chains[0];
  if (c0->ntime / 2 - meas_number < 1 || c0->ntime / 2 + meas_number > c0->ntime - 1) {
    set_error("measurement window ntime/2 +- %d leaves 1..ntime-1", meas_number);
    return PQMC_ERR_ARG;
  }
  for (auto* c : b->chains)
    if (!c->have_meas) { set_error("batch_set_measure: a chain has no measurement layout"); return PQMC_ERR_STATE; }
  b->meas_on = 1;
  b->meas_warmup = warmup;
  b->meas_interval = meas_interval;
  b->meas_number = meas_number;
  b->records.assign(b->chains.size(), std::vector<double>());
  return PQMC_OK;
}

int pqmc_batch_records(pqmc_batch* b, int i, double* out, int cap, int* n) {
  if (!b || i < 0 || i >= (int)b->chains.size() || !n || (cap > 0 && !out)) {
    set_error("batch_records: bad arguments");
    return PQMC_ERR_ARG;
  }
  if (!b->parts.empty()) return pqmc_batch_records(b->parts[b->part_of[i]], b->index_in_part[i], out, cap, n);
  if (i >= (int)b->records.size()) { *n = 0; return PQMC_OK; }
  pqmc_chain* c = b->chains[i];
  const size_t w = 2 * (size_t)(PQMC_N_SCALAR + 2 * PQMC_N_FIELD * c->n_cell);
  std::vector<double>& rec = b->records[i];
  const int have = (int)(rec.size() / w), take = std::min(have, cap);
  if (take > 0) memcpy(out, rec.data(), sizeof(double) * w * take);
  rec.erase(rec.begin(), rec.begin() + (size_t)take * w);
  *n = take;
  return PQMC_OK;
}

int pqmc_batch_chain(pqmc_batch* b, int i, pqmc_chain** chain) {
  if (!b || !chain || i < 0 || i >= (int)b->chains.size()) { set_error("batch_chain: bad index"); return PQMC_ERR_ARG; }
  *chain = b->chains[i];
  return PQMC_OK;
}

// ---- a mixed sweep in three parts, so that the classes of an uneven batch
// can interleave their slices on their own streams -------------------------
static int mixed_begin(pqmc_batch* b, int first_tc, int n_slices) {
  pqmc_chain* c0 = b->chains[0];
  if (first_tc + n_slices - 1 > c0->ntime) {
    set_error("batch_sweep_slices: slices %d..%d outside 1..%d", first_tc, first_tc + n_slices - 1, c0->ntime);
    return PQMC_ERR_ARG;
  }
  // every chain finished its own previous work on its stream
  for (auto* c : b->chains) PQMC_CUDA(cudaStreamSynchronize(c->stream));
  PQMC_TRY(batch_refresh(b));
  const long ng2 = (long)c0->ns * c0->ns;
  const dim3 cgrid((unsigned)std::min<long>((ng2 + 255) / 256, 64), (unsigned)b->chains.size());
  k_gconv<<<cgrid, 256, 0, b->stream>>>(b->d_desc, 1, ng2, 0);
  PQMC_LAUNCHED();
  // fork: the other groups' streams start after the work queued so far
  return groups_fork(b);
}

// slice tc of sweep `loop` for every group, the recompute that closes a
// block of ngroup slices, and the measurement window
static int mixed_slice(pqmc_batch* b, int loop, int tc) {
  pqmc_chain* c0 = b->chains[0];
  const int NG = b->n_groups;
  const bool forward = (loop % 2) == 0;
  const int time = forward ? tc : c0->ntime - tc + 1;
  for (int g = 0; g < NG; ++g) PQMC_TRY(group_slice(b, g, forward, time, b->parity));
  b->parity ^= (c0->n_pf & 1);
  if (tc % c0->ngroup == 0) {
    for (int g = 0; g < NG; ++g) PQMC_TRY(bscratch(b, g, forward ? time + 1 : time, forward, b->parity));
    b->parity ^= 1;
  }
  const int half = c0->ntime / 2;
  if (b->meas_on && loop > b->meas_warmup && ((loop - b->meas_warmup) % b->meas_interval) == 0 &&
      time >= half - b->meas_number && time <= half + b->meas_number)
    PQMC_TRY(batch_measure(b, time, forward));
  return PQMC_OK;
}

// join, then G back to FP64 in the current buffer of every chain; returns
// after the batch's work is done
static int mixed_end(pqmc_batch* b) {
  pqmc_chain* c0 = b->chains[0];
  PQMC_TRY(groups_join(b));
  PQMC_TRY(batch_sync_parity(b));
  const long ng2 = (long)c0->ns * c0->ns;
  const dim3 cgrid((unsigned)std::min<long>((ng2 + 255) / 256, 64), (unsigned)b->chains.size());
  k_gconv<<<cgrid, 256, 0, b->stream>>>(b->d_desc, 0, ng2, 0);
  PQMC_LAUNCHED();
  int err = 0;
  PQMC_CUDA(cudaMemcpyAsync(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  PQMC_CUDA(cudaStreamSynchronize(b->stream));
  PQMC_TRY(phase_resolve(b));
  if (err != 0) {
    set_error("batch sweep: a device-side wait gave up (panel stream of the scan)");
    return err;
  }
  return PQMC_OK;
}

// the classes of an uneven batch advance together: class k runs n[k] slices
// from first_tc, its slices spread evenly over the call so that every class
// keeps work queued until the end
static int classes_run(pqmc_batch* b, int loop, int first_tc, const std::vector<int>& n) {
  const size_t P = b->parts.size();
  PQMC_CUDA(cudaEventRecord(b->ev_fork, b->stream));
  int S = 0;
  for (size_t k = 0; k < P; ++k) {
    if (n[k] <= 0) continue;
    PQMC_CUDA(cudaStreamWaitEvent(b->parts[k]->stream, b->ev_fork, 0));
    PQMC_TRY(mixed_begin(b->parts[k], first_tc, n[k]));
    S = std::max(S, n[k]);
  }
  std::vector<int> done(P, 0);
  for (int step = 1; step <= S; ++step)
    for (size_t k = 0; k < P; ++k) {
      const int target = (int)(((long)step * n[k] + S - 1) / S);
      while (done[k] < target) PQMC_TRY(mixed_slice(b->parts[k], loop, first_tc + done[k]++));
    }
  int st = PQMC_OK;
  for (size_t k = 0; k < P; ++k) {
    if (n[k] <= 0) continue;
    const int sk = mixed_end(b->parts[k]);
    if (st == PQMC_OK) st = sk;
  }
  return st;
}

int pqmc_batch_sweep_slices(pqmc_batch* b, int loop, int first_tc, int n_slices) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  for (auto* c : b->chains)
    if (!c->have_g) { set_error("batch_sweep before init_g"); return PQMC_ERR_STATE; }
  if (first_tc < 1 || n_slices < 0) { set_error("batch_sweep_slices: bad slice range"); return PQMC_ERR_ARG; }
  if (b->precision == PQMC_PREC_FP64)
    return fp64_each(b, [&](pqmc_chain* c) {
      const int n = std::min(n_slices, c->ntime - first_tc + 1);
      return n > 0 ? pqmc_sweep_slices(c, loop, first_tc, n) : PQMC_OK;
    });
  if (!b->parts.empty()) {
    // uneven batch: each class takes the slices that exist in its sweep
    std::vector<int> n(b->parts.size());
    for (size_t k = 0; k < n.size(); ++k) n[k] = std::min(n_slices, b->parts[k]->chains[0]->ntime - first_tc + 1);
    return classes_run(b, loop, first_tc, n);
  }
  PQMC_TRY(mixed_begin(b, first_tc, n_slices));
  for (int tc = first_tc; tc < first_tc + n_slices; ++tc) PQMC_TRY(mixed_slice(b, loop, tc));
  return mixed_end(b);
}

int pqmc_batch_sweep(pqmc_batch* b, int loop) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  for (auto* c : b->chains)
    if (!c->have_g) { set_error("batch_sweep before init_g"); return PQMC_ERR_STATE; }
  // the driver's global step of every chain with global moves enabled
  // (Main_PQMC.f90:87-96) before the batched sweep; the chains' steps are
  // independent and run from worker threads
  bool any_global = false;
  for (auto* c : b->chains) any_global = any_global || c->have_global;
  if (any_global)
    PQMC_TRY(fp64_each(b, [&](pqmc_chain* c) { return c->have_global ? pqmc_global_step(c, loop, nullptr) : PQMC_OK; }));
  if (b->precision == PQMC_PREC_FP64)
    return fp64_each(b, [&](pqmc_chain* c) { return pqmc_sweep(c, loop, 1, 1 << 30, 1, 0, nullptr, 0, nullptr); });
  if (!b->parts.empty()) {
    // one whole sweep of every chain, each class over its own ntime slices
    std::vector<int> n(b->parts.size());
    for (size_t k = 0; k < n.size(); ++k) n[k] = b->parts[k]->chains[0]->ntime;
    return classes_run(b, loop, 1, n);
  }
  return pqmc_batch_sweep_slices(b, loop, 1, b->chains[0]->ntime);
}

}  // extern "C"
