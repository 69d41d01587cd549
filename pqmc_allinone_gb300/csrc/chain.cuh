// chain.cuh -- device state of one Markov chain and the launchers shared by
// the single-chain C-ABI (chain.cu) and the batched driver (batch.cu).
#pragma once
#include <vector>
#include "common.cuh"
#include "expkv.cuh"

namespace pqmc {

// Scalars the reference keeps as module globals (src/input.f90:7,53,72) plus
// the ran2 state (src/mod_ranstate.f90:15).
struct DevScalars {
  cplx ln_cw;
  cplx logdet;          // scratch for cal_g_and_det
  cplx sumlogd;
  double err_fast;
  double err_fast_max;
  double err_g;
  double err_w;
  double err_g_rel;       // ||G_fast - G_scratch||_F / ||G_scratch||_F at the last recompute
  double err_g_rel_max;   // largest err_g_rel so far
  long long pos_acc;
  long long neg_acc;
  int rng[5];
  int lu_info;
  int status;
  int pad;
};

// Control record the proposer publishes at every grid barrier of the update
// kernel: the accepted plaquette and T = Delta R^-1 of its rank-dim update.
struct UpdCtl {
  int p;
  int dim;
  int S[4];
  cplx T[16];
};

// Per-plaquette proposal data of one family step, computed in parallel
// before the sequential Metropolis scan (every proposal consumes a fixed
// number of ran2 draws, so jumps, energies and propagators do not depend on
// earlier accepts).
struct PlaqPre {
  cplx delta[16];   // Delta = expKV_inv(old) expKV(new) - I
  cplx enew[16];    // expKV(new)
  cplx einv[16];    // expKV_inv(new)
  float2 deltaf[16];// Delta rounded to FP32 for the fast test
  float4 deltad[16];// Delta in double-float {re_hi, im_hi, re_lo, im_lo} (mixed batch)
  double dE;        // -dtau * (E_new - E_old)
  double xnew;
  double r;         // acceptance draw rands()
  double thr;       // accept iff |det R|^2 >= thr (the Metropolis test of cal_prob)
};

struct FtState;           // finite-temperature strings (finite_t.cu)

struct WrapItems {        // cover of all sites by one family: plaquettes + singletons
  int n_items;
  int* d_pla;             // (n_items) plaquette index or -1
  int* d_sites;           // (4*n_items)
  int* d_dim;             // (n_items)
};

}  // namespace pqmc

struct pqmc_chain {
  ::DevModel M;                     // device pointers
  // host copies of the sizes / tables
  int ns, nelec, ntime, ngroup, nblock, n_pf, pdim, max_pla, n_bf;
  std::vector<int> h_pf_dim, h_pf_npla, h_pf_v_exist;
  // device buffers
  void* d_model_blob = nullptr;
  double* field = nullptr;          // (n_bf, ntime)
  cplx* expkv = nullptr;            // (pdim,pdim,max_pla,n_pf,ntime)
  cplx* expkv_inv = nullptr;
  cplx* g = nullptr;                // current g_h (Ns,Ns)
  cplx* g_alt = nullptr;            // ping-pong partner
  cplx* q_string = nullptr;         // (Ns,nelec,nblock)
  cplx* d_string = nullptr;         // (nelec,nblock)
  cplx* d_logsum = nullptr;         // (nblock) sum_i log D(i,block)
  cplx* slater_q = nullptr;
  cplx* slater_d = nullptr;
  cplx* rmat = nullptr;             // (Ns,nelec)
  cplx* xmat = nullptr;             // (Ns,nelec) left factor, adjoint layout
  cplx* lmat = nullptr;             // (nelec,Ns)
  cplx* pbp = nullptr;              // (nelec,nelec)
  cplx* tau = nullptr;              // (nelec)
  cplx* dtmp = nullptr;             // (nelec)
  cplx* lcol = nullptr;             // (nelec)
  int* ipiv = nullptr;              // (nelec)
  pqmc::UpdCtl* ctl = nullptr;      // [2]
  pqmc::PlaqPre* pre = nullptr;     // (max_pla)
  pqmc::DevScalars* sc = nullptr;
  std::vector<pqmc::WrapItems> wrap;
  int upd_blocks = 0;
  bool have_g = false;
  bool have_meas = false;
  cudaStream_t stream = nullptr;
  // measurement
  int n_cell = 0;
  int* m_cell_sites = nullptr;
  int* m_cell_bf = nullptr;
  int* m_cell_xnb = nullptr;
  int* m_cell_ynb = nullptr;
  int* m_cell_cross = nullptr;
  int* m_c2_of = nullptr;           // (n_cell (c1), n_cell (ind)) -> c2
  cplx* m_kphase = nullptr;         // (n_cell,n_cell) Fortran (ik,ic)
  cplx* m_acc = nullptr;            // record accumulator
  cplx h_bc[2];
  double hop = 1.0, ep = 1.0;
  cplx* m_gtmp = nullptr;           // g = I - g_h
  // host copy of the model's scalars (table pointers cleared)
  pqmc_model hmodel;
  // global moves (pqmc_set_global)
  bool have_global = false;
  pqmc_global_params gp;
  std::vector<double> g_rpos;
  long long g_acc = 0, g_rej = 0;
  // finite temperature (pqmc_set_temperature): the Q/D/R strings of
  // init_g_FT and its work buffers, finite_t.cu
  bool finite_t = false;
  pqmc::FtState* ft = nullptr;
  bool in_batch = false;            // owned by a pqmc_batch (projector path only)
};

namespace pqmc {
// weight and error bookkeeping kernels of chain.cu, shared with finite_t.cu
__global__ void k_scalars_zero(DevScalars* sc);
__global__ void k_finish_weight(DevScalars* sc, int tr_weight, int ncopy, int compare);
__global__ void k_maxdiff(long n, const cplx* __restrict__ a, const cplx* __restrict__ b, double* out);
__global__ void k_set_errg(DevScalars* sc, const double* e);
int do_init_g_ft(pqmc_chain* c, int start_time);
int do_g_scratch_ft(pqmc_chain* c, int time, bool forward);
int do_new_weight_ft(pqmc_chain* c);
int ft_free(pqmc_chain* c);
int chain_alloc(pqmc_chain* c, const pqmc_model* m, cudaStream_t s);
int chain_free(pqmc_chain* c);
int launch_init_expkv(pqmc_chain* c, int t0, int nt);
int launch_update(pqmc_chain* c, int pf, int time);
int update_setup(pqmc_chain* c);
int launch_wrap(pqmc_chain* c, int pf, int time, bool left);
int launch_propagate(pqmc_chain* c, cplx* X, int n, int t_from, int t_to, bool forward);
int do_init_g(pqmc_chain* c, int start_time);
int do_g_scratch(pqmc_chain* c, int time, bool forward, int loop);
int do_new_weight(pqmc_chain* c);
int do_new_weight_ck(pqmc_chain* c, cplx* ck);
int block_log(pqmc_chain* c, int blk1);
int do_measure(pqmc_chain* c, int time);
int do_finish_record(pqmc_chain* c, int meas_number);
}  // namespace pqmc
