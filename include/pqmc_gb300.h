/*
 * pqmc_gb300.h -- C-ABI of the GB300 projector-DQMC hot path.
 *
 * Every entry point replaces one Fortran subroutine of the reference
 * (LEOMMM816/PQMC_allinone) on its local-update / B-string / measurement
 * path.  The Fortran side keeps its subroutine signatures and forwards to
 * these functions through a thin ISO_C_BINDING shim.  All state the
 * reference keeps as module globals
 * (src/input.f90:72-96) lives on the device inside an opaque handle; the
 * host passes plain pointers and sizes.
 *
 * Conventions
 *   - complex numbers are interleaved (re, im) doubles, i.e. complex(dp);
 *   - matrices are column-major like Fortran arrays;
 *   - site, plaquette and boson indices inside the tables are 0-based
 *     (the shim subtracts 1); `time`, `pf_id` arguments are 1-based, exactly
 *     as the Fortran callers pass them;
 *   - every function returns an int status: PQMC_OK or one of PQMC_ERR_*.
 *     The reference stops the program on LAPACK failures
 *     (src/mod_matrixlib.f90:405-503); the shim maps a non-zero status to
 *     `error stop`.
 *   - one host thread per handle (the reference is single-threaded per
 *     process, scripts/mpi_32c_copilot.sh:74-75).
 */
#ifndef PQMC_GB300_H
#define PQMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PQMC_OK 0
#define PQMC_ERR_ARG 1        /* bad argument or size out of range            */
#define PQMC_ERR_CUDA 2       /* a CUDA runtime call failed                   */
#define PQMC_ERR_SINGULAR 3   /* LU found an exact zero pivot (zgetrf info>0) */
#define PQMC_ERR_TIMEOUT 4    /* a bounded device-side wait gave up           */
#define PQMC_ERR_STATE 5      /* call order violated (e.g. no init_g yet)      */
#define PQMC_ERR_NOMEM 6      /* device allocation failed                     */

/* expKV generator, the procedure pointer get_expKV bound in
 * setup_expKV (src/mod_phonon_field.f90:472-496). */
#define PQMC_EXPKV_GENERAL 0      /* get_expKV_general, expm via eigen :497-532 */
#define PQMC_EXPKV_EPSOCZ 1       /* get_expKV_epsocz closed form      :534-569 */
#define PQMC_EXPKV_EPSOC 2        /* get_expKV_epsoc closed form       :572-604 */
#define PQMC_EXPKV_EPSOCZ_BLOCK 3 /* epsocz form with the norm taken from the
                                     actual 2x2 hopping block; valid for any
                                     block with h^H h proportional to 1 (static
                                     spin-orbit term added to Kmatrix).  No
                                     reference counterpart.                    */

/* proposal law for the local move */
#define PQMC_PROPOSAL_UNIFORM 0   /* jump_distance*ran_sysm(), mod_update.f90:84 */
#define PQMC_PROPOSAL_GAUSSIAN 1  /* jump_distance*N(0,1) by Box-Muller on two
                                     ran2 draws (extension, not in reference)   */

#define PQMC_MAX_DIM 4            /* largest plaquette dimension supported     */

/* Flattened model: the module globals of src/input.f90:48-96 after
 * set_pf_main / init / init_pf_para, in the flat layout of
 * set_pf_expKV_mat (src/mod_phonon_field.f90:605-636). */
typedef struct pqmc_model {
  int32_t ns;            /* Ns                                              */
  int32_t nelec;         /* nelec = nint(Ns*filling)                        */
  int32_t ntime;         /* Lt                                              */
  int32_t ngroup;        /* slices between QDR stabilisations               */
  int32_t n_pf;          /* n_phonon_field (checkerboard families)          */
  int32_t max_dim;       /* pdim = max plaquette dim, <= PQMC_MAX_DIM        */
  int32_t max_pla;       /* max n_plaquette over families                   */
  int32_t n_bf;          /* n_boson_field = bf_sets*N_cell                  */
  int32_t expkv_kind;    /* PQMC_EXPKV_*                                    */
  int32_t ncopy;         /* flavours: weight ratio raised to ncopy          */
  int32_t tr_weight;     /* TR_weight: ratio multiplied by its conjugate    */
  int32_t metropolis;    /* Metropolis (1) or heat bath (0)                 */
  int32_t greatest_decent; /* floor(prob) when set                          */
  int32_t local_update;  /* local_update flag of the sweep driver           */
  int32_t proposal_kind; /* PQMC_PROPOSAL_*                                 */
  int32_t reserved;
  double delt;           /* dtau                                            */
  double mass;           /* M                                               */
  double stiff;          /* D                                               */
  double biased_phonon;  /* linear term of the phonon action               */
  double jump_distance;  /* already scaled as in init (input.f90:183)       */
  /* per family (length n_pf) */
  const int32_t* pf_dim;
  const int32_t* pf_npla;
  const int32_t* pf_k_exist;
  const int32_t* pf_v_exist;
  const double* pf_k_coe;   /* complex, after init_pf_para (K_coe*(-hop)) */
  const double* pf_v_coe;   /* complex, after init_pf_para (V_coe*lambda) */
  const double* pf_kmat;    /* complex (max_dim,max_dim,n_pf)             */
  const double* pf_vmat;    /* complex (max_dim,max_dim,n_pf)             */
  /* plaquette tables */
  const int32_t* pla_site_list;     /* (max_dim,max_pla,n_pf), 0-based sites */
  const int32_t* bf_list;           /* (max_pla,n_pf), 0-based boson index   */
  const int32_t* boundary_crossing; /* (max_pla,n_pf)                        */
  const double* bc_phases;          /* complex (max_dim,max_dim,max_pla,n_pf)*/
} pqmc_model;

/* Lattice tables for the equal-time measurement (ms_take_measurement,
 * src/mod_meas.f90:210-544).  Two sub-sites per cell (spin up, spin down)
 * and two boson fields per cell (x bond, y bond), as the reference code
 * assumes there (mod_meas.f90:244-247). */
typedef struct pqmc_meas_layout {
  int32_t n_cell;
  int32_t reserved;
  const int32_t* cell_sites;   /* (2,n_cell) 0-based site of sub-site 1,2   */
  const int32_t* cell_bf;      /* (2,n_cell) 0-based boson x, y             */
  const int32_t* cell_xnb;     /* (n_cell) 0-based cell at dpos+(1,0)       */
  const int32_t* cell_ynb;     /* (n_cell) 0-based cell at dpos+(0,1)       */
  const int32_t* cell_cross;   /* (2,n_cell) dpos(i)==L_i-1                 */
  const int32_t* rel_index;    /* (n_cell,n_cell) 0-based relative index of
                                  c2 seen from c1: rel_index[c1+n*c2]       */
  const double* bc_phase;      /* complex (2) Lat%BC_phase                 */
  const double* k_phase;       /* complex (n_cell,n_cell) Lat%k_phase      */
  double hop;
  double ep_parameter;
} pqmc_meas_layout;

/* Observable slots of one measurement record (per-measurement vector,
 * like MeasurementSystem%data(:,m,b)).  Scalars first, then the r-space
 * block of the fields (width n_cell each, in the order below), then the
 * k-space block (the _k transform of each field, same order). */
#define PQMC_OBS_BF_KE 0
#define PQMC_OBS_BF_PE 1
#define PQMC_OBS_BF_X 2
#define PQMC_N_SCALAR 3
/* field order */
#define PQMC_F_BFX_BFX 0
#define PQMC_F_BFX_BFY 1
#define PQMC_F_BFY_BFY 2
#define PQMC_F_BFXY_BFXY 3
#define PQMC_F_JXX_JXX 4
#define PQMC_F_JXY_JXY 5
#define PQMC_F_JYX_JYX 6
#define PQMC_F_JYY_JYY 7
#define PQMC_F_JXX_JYX 8
#define PQMC_F_JXY_JYY 9
#define PQMC_F_JXXH_JXXH 10
#define PQMC_F_JXYH_JXYH 11
#define PQMC_F_JYXH_JYXH 12
#define PQMC_F_JYYH_JYYH 13
#define PQMC_F_JXXH_JYXH 14
#define PQMC_F_JXYH_JYYH 15
#define PQMC_F_JXXH_JYYH 16
#define PQMC_F_JXYH_JYXH 17
#define PQMC_F_DEN_DEN 18
#define PQMC_F_SC_SC 19
#define PQMC_F_SZ_SZ 20
#define PQMC_F_SX_SX 21
#define PQMC_F_SY_SY 22
#define PQMC_F_CJYX_CJYX 23
#define PQMC_F_CJXY_CJXY 24
#define PQMC_N_FIELD 25
/* record width (complex entries): PQMC_N_SCALAR + 2*PQMC_N_FIELD*n_cell
 * (r-space block of all fields, then k-space block of all fields). */

/* Per-chain scalar state (module globals of input.f90:7,53,72). */
typedef struct pqmc_state {
  double ln_cw[2];          /* complex ln_cw                               */
  double err_fast_max;      /* largest fast-vs-scratch error so far         */
  double err_fast;          /* last fast-vs-scratch error (G or ln_cw)      */
  int64_t positive_accept;  /* local moves accepted                          */
  int64_t negative_accept;  /* local moves rejected                          */
  int32_t rng[5];           /* iran0,jran0,kran0,mran0,nran0 of ran2_s       */
  int32_t reserved;
  double err_g;             /* max |G_fast - G_scratch| at the last recompute */
  double err_g_rel_max;     /* largest ||G_fast - G_scratch||_F/||G_scratch||_F
                               over all recomputes so far (no reference
                               counterpart: the drift of the fast path)     */
} pqmc_state;

typedef struct pqmc_chain pqmc_chain; /* opaque, one Markov chain on the GPU */

/* ---- lifetime ------------------------------------------------------- */
/* Allocates the device copies of every module global the hot path uses.
 * Replaces the allocations of init_g_T0 (mod_evolution.f90:57-62) and of
 * set_pf_expKV_mat (mod_phonon_field.f90:612-619). */
int pqmc_create(const pqmc_model* model, pqmc_chain** out);
int pqmc_destroy(pqmc_chain* chain);
/* Attach the measurement lattice tables (ms_init_meas, mod_meas.f90:577). */
int pqmc_set_meas_layout(pqmc_chain* chain, const pqmc_meas_layout* layout);

/* ---- state transfer ------------------------------------------------- */
/* boson_field(n_bf,ntime) in (input.f90:86); import_ph_field path of
 * init_boson_field (Main_PQMC.f90:355-369) with exact doubles. */
int pqmc_set_field(pqmc_chain* chain, const double* boson_field);
int pqmc_get_field(pqmc_chain* chain, double* boson_field);
/* boson_field(:, first_time .. first_time+n_times-1) from / to host memory
 * (columns of the column-major array are contiguous).  Setting a block
 * recomputes expKV/expKV_inv of those slices (set_pf_expKV_mat); it leaves
 * G alone, so the values must be those G was built with (a host copy kept
 * in step with the device) or a recompute must follow. */
int pqmc_set_field_slices(pqmc_chain* chain, int first_time, int n_times, const double* boson_field_block);
int pqmc_get_field_slices(pqmc_chain* chain, int first_time, int n_times, double* boson_field_block);
/* slater_Q(Ns,nelec), slater_D(nelec) complex, from set_nelec_occupied
 * (Main_PQMC.f90:279-305). */
int pqmc_set_slater(pqmc_chain* chain, const double* slater_q,
                    const double* slater_d);
/* g_h(Ns,Ns) complex (input.f90:88). */
int pqmc_get_g(pqmc_chain* chain, double* g_h);
int pqmc_set_g(pqmc_chain* chain, const double* g_h);
int pqmc_get_state(pqmc_chain* chain, pqmc_state* state);
/* ran2 state words; replaces init_rng_by_seed (mod_ranstate.f90:267-283)
 * when called with the five seeded words. */
int pqmc_set_rng(pqmc_chain* chain, const int32_t rng[5]);
/* Restore the ran2 state, accept counters and error maxima of a checkpoint
 * (pqmc_get_state of the saved chain; no reference counterpart: the
 * reference has no checkpoint writer, Main_PQMC.f90:166).  ln_cw is not
 * taken: the init_g_T0 that follows a restore recomputes it. */
int pqmc_set_state(pqmc_chain* chain, const pqmc_state* state);
/* Q_string(:,:,block) and D_string(:,block), block 1-based. */
int pqmc_get_qd(pqmc_chain* chain, int block, double* q, double* d);

/* ---- hot path: one call per reference subroutine --------------------- */
/* init_expKV for every family + set_pf_expKV_mat
 * (mod_phonon_field.f90:423-450, 605-636). */
int pqmc_init_expkv(pqmc_chain* chain);
/* init_g(start_time): init_g_T0 (mod_evolution.f90:46-111), or init_g_FT
 * on a chain set to finite temperature (the procedure pointer of
 * set_temperature, :30-45). */
int pqmc_init_g(pqmc_chain* chain, int start_time);
/* update_phonon_field(ppf_list(pf_id), time) (mod_update.f90:13-201). */
int pqmc_update_phonon_field(pqmc_chain* chain, int pf_id, int time);
/* left_evolve(time, g_h, Ns, pf_id, two_way) (mod_evolution.f90:236-285). */
int pqmc_left_evolve_g(pqmc_chain* chain, int time, int pf_id, int two_way);
/* right_evolve(time, g_h, Ns, pf_id, two_way) (mod_evolution.f90:287-328). */
int pqmc_right_evolve_g(pqmc_chain* chain, int time, int pf_id, int two_way);
/* left_evolve(time, mat(Ns,n), n, pf_id, .false.) on a caller matrix. */
int pqmc_left_evolve(pqmc_chain* chain, int time, int pf_id, double* mat,
                     int n);
/* right_evolve(time, mat(n,Ns), n, pf_id, .false.) on a caller matrix. */
int pqmc_right_evolve(pqmc_chain* chain, int time, int pf_id, double* mat,
                      int n);
/* get_g_scratch_T0(time, forward, loop) (mod_evolution.f90:113-195), or
 * get_g_scratch_FT at finite temperature; err_out (may be NULL) receives
 * max|gfast-g| and |Re(dln_cw)|. */
int pqmc_get_g_scratch(pqmc_chain* chain, int time, int forward, int loop,
                       double* err_out);
/* cal_new_weight_T0() (mod_evolution.f90:359-408), or cal_new_weight_FT
 * at finite temperature; ln_cw_out complex. */
int pqmc_cal_new_weight(pqmc_chain* chain, double* ln_cw_out);

/* ---- finite temperature (mod_evolution.f90:409-785) ------------------ */
/* set_temperature (mod_evolution.f90:30-45): proj = 1 selects the
 * projector path (the default), proj = 0 the finite-temperature one for
 * init_g, get_g_scratch, cal_new_weight and the sweep.  Finite temperature
 * needs ntime to be a multiple of ngroup and allocates the Ns x Ns Q and R
 * strings (2 x 16 Ns^2 (ntime/ngroup + 2) bytes); chains of a batch stay on
 * the projector path (PQMC_ERR_STATE).  Either switch drops G: call
 * pqmc_init_g next.  The weight is ln det(1 + B(beta,0)) (x2 Re under
 * TR_weight, x ncopy) and g_h = 1 - (1 + B(beta,0))^-1 at the slice in
 * progress.  Four departures from the reference's unfinished branch, each a
 * correction: the strings use a column-pre-pivoted Householder QR instead of
 * the SVD (which loses the small scales of the graded products); init_g_FT
 * closes with B(beta,beta) = 1 as the left factor; the left string's unitary
 * factor is its Q; cal_new_weight_FT scales column i by D(i) alone. */
int pqmc_set_temperature(pqmc_chain* chain, int proj);
int pqmc_get_temperature(pqmc_chain* chain, int* proj);
/* init_g_FT(start_time) (mod_evolution.f90:411-489). */
int pqmc_init_g_ft(pqmc_chain* chain, int start_time);
/* get_g_scratch_FT(time, forward, loop) (mod_evolution.f90:631-745). */
int pqmc_get_g_scratch_ft(pqmc_chain* chain, int time, int forward, int loop,
                          double* err_out);
/* cal_new_weight_FT() (mod_evolution.f90:748-785); strings and G intact. */
int pqmc_cal_new_weight_ft(pqmc_chain* chain, double* ln_cw_out);
/* One block of the finite-temperature strings: q, r (Ns x Ns) and d (Ns)
 * complex, any of them NULL.  Blocks below the current time hold
 * B(t_b,0) = Q D R; blocks above it hold B(beta,t_b)^H = Q D R. */
int pqmc_get_qdr_ft(pqmc_chain* chain, int block, double* q, double* d,
                    double* r);
/* Meas_sys%take_measurement(time) (mod_meas.f90:210-544): adds one
 * record into the device accumulator. */
int pqmc_take_measurement(pqmc_chain* chain, int time);
/* Meas_sys%begin_measure(forward,time) (mod_meas.f90:729-763): takes the
 * measurement and, at the last slice of the window, divides by
 * 2*meas_number+1, adds the k-space transform (ms_k_space_obs :546-566)
 * and copies the finished record to `record_out` (may be NULL); *done is
 * set to 1 when a record was finished. */
int pqmc_begin_measure(pqmc_chain* chain, int forward, int time,
                       int meas_number, double* record_out, int* done);
/* The sweep loop body of Main_PQMC.f90:81-156 for `n_sweeps` consecutive
 * values of `loop` starting at `first_loop` (global updates excluded).
 * Measurements are taken when loop>warmup and mod(loop-warmup,
 * meas_interval)==0; finished records are appended to `records`
 * (n_records_cap entries of record width), *n_records is their count. */
int pqmc_sweep(pqmc_chain* chain, int first_loop, int n_sweeps, int warmup,
               int meas_interval, int meas_number, double* records,
               int n_records_cap, int* n_records);
/* Slices tc = first_tc .. first_tc+n_slices-1 of sweep `loop` of that loop
 * body (no measurement); n_slices = ntime from first_tc = 1 is one whole
 * sweep.  Lets a driver advance a sweep in stabilisation blocks. */
int pqmc_sweep_slices(pqmc_chain* chain, int loop, int first_tc, int n_slices);

/* ---- global moves (update_global, src/mod_update.f90:250-467) ---------- */
/* update_type of update_global / generate_newfield_global */
#define PQMC_GLOBAL_SINGLE 0      /* default branch: flip or shift the whole
                                     time line of n_global_update bonds      */
#define PQMC_GLOBAL_EXCHANGE 1    /* "exchange": swap the time lines of two
                                     bonds, n_global_update times            */
#define PQMC_GLOBAL_KSPACE 2      /* "kspace": add a (pi,pi) staggered pattern
                                     to every slice                          */
#define PQMC_GLOBAL_KSPACE_TIME 3 /* "kspace_time": the same pattern on
                                     slices start_time..end_time             */
#define PQMC_GLOBAL_ROTATE 4      /* "rotate": rotate (or reflect) the two
                                     boson fields of every cell              */
typedef struct pqmc_global_params {
  int32_t n_global_update;    /* n_global_update (input.f90:74)             */
  int32_t global_update_loop; /* global_update_loop (input.f90:75)          */
  int32_t flip;               /* global_update_flip                          */
  int32_t shift;              /* global_update_shift                         */
  int32_t rotate;             /* the driver adds the "rotate" move (EPSOCZ
                                 models, Main_PQMC.f90:92)                   */
  int32_t lat_dim;            /* Lat%dim (2 for the k-space moves)          */
  int32_t n_cell;             /* Lat%N_cell                                  */
  int32_t bf_sets;            /* boson fields per cell (2 for "rotate")      */
  double distance;            /* global_update_distance*char_length
                                 (input.f90:184)                             */
  const double* cell_rpos;    /* (lat_dim, n_cell) p_cells(i)%rpos          */
} pqmc_global_params;
/* The field generation alone, on the host: the new boson_field (n_bf,
 * ntime, in place), the phonon-action part of the weight ph_ln_cw
 * (-delta_energy*delt) and the slices whose expKV change (1-based
 * t_first..t_last), advancing the ran2 state rng[5] by the draws the move
 * takes (generate_newfield_global, mod_update.f90:298-438).  Needs no GPU. */
int pqmc_global_generate(const pqmc_model* model, const pqmc_global_params* params,
                         int kind, int32_t rng[5], double* boson_field,
                         double* ph_ln_cw, int* t_first, int* t_last);
/* Copies the parameters into the chain (and enables the global step of
 * pqmc_sweep). */
int pqmc_set_global(pqmc_chain* chain, const pqmc_global_params* params);
/* update_global(update_type) (mod_update.f90:250-292): the new field, its
 * expKV and cal_new_weight_T0 on the device, the Metropolis test of
 * ln_cw_new + ph_ln_cw - ln_cw_old (cal_prob) with one more ran2 draw;
 * a rejected move restores field, expKV and ln_cw.  *accepted = 0 or 1.
 * G is not touched (the caller re-initialises it after accepted moves). */
int pqmc_update_global(pqmc_chain* chain, int kind, int* accepted);
/* The driver's global step before sweep `loop` (Main_PQMC.f90:87-96): when
 * the sweep runs backward and mod(loop+1, global_update_loop) == 0, the
 * "kspace", "rotate" (when enabled) and "kspace_time" moves, then
 * init_g_T0(1) if any was accepted.  *n_accepted (may be NULL) counts them.
 * pqmc_sweep runs this step itself once pqmc_set_global was called. */
int pqmc_global_step(pqmc_chain* chain, int loop, int* n_accepted);
/* global_accept / global_reject counters (input.f90:7) */
int pqmc_global_counters(pqmc_chain* chain, int64_t* accepted, int64_t* rejected);

/* ---- differentiable log-weight ---------------------------------------- */
/* boson_field from a DEVICE pointer (n_bf, ntime), e.g. a torch tensor. */
int pqmc_set_field_device(pqmc_chain* chain, const double* boson_field_dev);
/* Value and gradient of the projector log-weight
 *   W = Re log det(P^H B(Lt..1) P)  (cal_new_weight_T0, mod_evolution.f90:359)
 * with respect to every boson_field(b,tau).  The value goes to logw_out
 * (host, complex, as cal_new_weight_T0 returns it); the gradient of Re W
 * goes to grad_dev (DEVICE, (n_bf, ntime) doubles).  The gradient is the
 * Green's-function trace formula Re Tr[E^-1 dE/dx G] per plaquette, by a
 * right-to-left pass that checkpoints the orthonormal left factor every
 * ngroup slices and a left-to-right pass that recomputes G from the
 * checkpoints and wraps it through each block.  Needs the expKV of the
 * current field (pqmc_init_expkv) and the trial state; init_g_T0 is not
 * needed.  Leaves G and the Q/D strings as they were (the rank's
 * fast-update state is not disturbed); ln_cw is set to the value, as
 * cal_new_weight_T0 sets it.  Calls on different chains may run from
 * different host threads at the same time. */
int pqmc_logweight_grad(pqmc_chain* chain, double* logw_out, double* grad_dev);

/* ---- batched, mixed precision --------------------------------------- */
typedef struct pqmc_batch pqmc_batch; /* many chains in one device context */
#define PQMC_PREC_FP64 0   /* every product in FP64                        */
#define PQMC_PREC_MIXED 1  /* G held in double-float (two FP32 values,
                              48-bit significand); accept/reject from FP32
                              ratios; round update of G in double-float
                              with Ozaki-split BF16 tensor-core products
                              (exact level sums); double-float wraps, QR
                              (CholeskyQR2), recompute and log-det; ln_cw
                              accumulated in FP64                         */
int pqmc_batch_create(const pqmc_model* const* models, int n_chains,
                      int precision, pqmc_batch** out);
int pqmc_batch_destroy(pqmc_batch* batch);
int pqmc_batch_chain(pqmc_batch* batch, int i, pqmc_chain** chain);
/* delay depth of the mixed-precision update: accepted-move columns per
 * scan round, applied to G by one round update (default 64, at most 512;
 * the exact round update takes at most 64 and clamps deeper settings) */
int pqmc_batch_set_delay(pqmc_batch* batch, int depth);
/* round update of the mixed batch: 2 (default) = the exact update of G
 * from G itself (W^-1 by an FP32 inverse refined by a double-float Newton
 * step, Ozaki-split BF16 tcgen05 products with exact level sums, drift of
 * the fast-updated G ~1e-9 per block), with double-float wraps;
 * 1 = the scan's FP32 panels added by tcgen05 3xBF16 products (delay depth
 * <= 64; deeper delays use 0), FP32 wrap corrections (drift ~1e-5 per
 * block); 0 = the same with mma.sync split-BF16 tiles.  PQMC_WRAP_DF=0/1
 * forces the FP32 / double-float wrap in any mode. */
int pqmc_batch_set_flush(pqmc_batch* batch, int mode);
/* one sweep of every chain (Main_PQMC.f90:99-154); equal-time
 * measurements only after pqmc_batch_set_measure; chains with global moves
 * enabled (pqmc_set_global on pqmc_batch_chain) take the driver's global
 * step first (Main_PQMC.f90:87-96), the chains' steps run from worker
 * threads (PQMC_BATCH_THREADS, default 8) */
int pqmc_batch_sweep(pqmc_batch* batch, int loop);
/* Equal-time measurement inside batched sweeps with the reference's window
 * and cadence (loop > warmup, mod(loop-warmup, meas_interval) == 0, time in
 * ntime/2 +- meas_number; Main_PQMC.f90:142-152).  Every chain needs a
 * measurement layout.  Finished records accumulate per chain on the host. */
int pqmc_batch_set_measure(pqmc_batch* batch, int warmup, int meas_interval, int meas_number);
/* Takes up to `cap` finished records of chain i (oldest first; record width
 * as pqmc_take_measurement); *n is the number copied. */
int pqmc_batch_records(pqmc_batch* batch, int i, double* records, int cap, int* n);
/* Delay-depth autotuner (no reference counterpart): runs n_slices slices
 * of the sweep order per candidate depth, starting at (loop, first_tc) and
 * continuing block after block (these are genuine Monte Carlo steps of every
 * chain, so tune during warm-up), times each with CUDA events and keeps the
 * fastest depth (and the tcgen05 flush when it allows).  ms_out (optional,
 * n_candidates) receives the measured ms per slice. */
int pqmc_batch_autotune(pqmc_batch* batch, int loop, int first_tc, int n_slices,
                        const int* candidates, int n_candidates, int* best,
                        double* ms_out);
/* Tile shape of the mixed batch's two-way wrap: 1 or 2 column items per
 * k_bwrap_cols CTA (whole columns of G staged in shared memory; fewer items
 * let more CTAs share an SM, more items share the row items' tables), or 0
 * for the gathered form (32 x 4 blocks per CTA).  The same arithmetic for
 * every entry in every shape: the chains are bit-identical whichever runs.
 * Shapes whose columns do not fit in shared memory fall back to the largest
 * that fits.  Default 1 (0 with PQMC_WRAP_COLS=0). */
int pqmc_batch_set_wrap_tile(pqmc_batch* batch, int ci);
int pqmc_batch_get_wrap_tile(pqmc_batch* batch, int* ci);
/* Flush of the exact round update: 64 columns of G per CTA (k_xgemm<1>, one
 * CTA per SM: 3 x 128 tensor-memory columns, 160 KB of slice images in two
 * stages), 32 (k_xflush2, two CTAs per SM: 3 x 64 columns, 60 KB stages of a
 * quarter of the inner dimension), or the pipeline k_xflushp with 2 or 1
 * CTAs per 128-row tile of G (the row tile's X slices resident, Z's 32-column
 * tiles streamed in quarter stages, two tensor-memory accumulator buffers so
 * one tile's G read-modify-write overlaps the next tile's products).
 * Default 64.  k_xflush2 and k_xflushp sum the rounded level of the Ozaki
 * products stage by stage and agree bit for bit; k_xgemm<1> sums it in
 * another order, so its chains agree with theirs to that rounding (~2^-40
 * of the update). */
int pqmc_batch_set_flush_tile(pqmc_batch* batch, int ct);
int pqmc_batch_get_flush_tile(pqmc_batch* batch, int* ct);
/* Engine of the stabilised recompute's complex GEMMs (Gram matrices,
 * X R^-1, L R, R (L R)^-1, the new G; the zgemm calls of
 * src/mod_evolution.f90 cal_g_and_det_T0 / get_g_scratch_T0 and
 * src/mod_matrix.f90 qdr): 1 the Ozaki-split BF16 product on the tensor
 * cores (default; ozgemm.cu: six slices per operand, 21 slice products into
 * six FP32 level accumulators, levels 0-4 exact, summed in double-float;
 * ~1e-14 on an orthonormal Gram matrix), 0 the compensated double-float
 * product on the FP32 pipe (k_dfgemm2; Dot2, whose FP32 low-order sum grows
 * like K^1.5 u^2: ~1e-12 there).  The environment variable
 * PQMC_RECOMPUTE_GEMM=0 makes 0 the default.  Chains of the two engines
 * agree to the products' rounding, not bit for bit.  Mixed batches only. */
int pqmc_batch_set_gemm_engine(pqmc_batch* batch, int engine);
int pqmc_batch_get_gemm_engine(pqmc_batch* batch, int* engine);
/* Panel columns per streamed chunk of the scan (k_bscan's TMA stream of the
 * delayed panels through three shared-memory stages): 1 .. qc_max, the
 * largest chunk that fits (at most 8; the default).  The chunking does not
 * change the arithmetic, so the chains are bit-identical whichever runs.
 * qc_max may be NULL.  Uneven batches: set for every class, get the first
 * class's. */
int pqmc_batch_set_scan_chunk(pqmc_batch* batch, int qc);
int pqmc_batch_get_scan_chunk(pqmc_batch* batch, int* qc, int* qc_max);
/* Autotune the tile shapes at the batch's delay depth: every wrap tile
 * (0, 1, 2), then, with the exact round update, every flush (64, 32, 2, 1),
 * then the scan chunks qc_max, (3 qc_max + 3) / 4 and (qc_max + 1) / 2,
 * each timed over n_slices slices of sweep `loop` from first_tc with plain
 * launches (CUDA events on the batch stream; the chains advance
 * meanwhile); the fastest of each is kept.  Every wrap and scan-chunk slot
 * runs its n_slices (a wrap tile that does not fit runs them at the best so
 * far), and the four flush slots run with the exact round update only: 10
 * or 6 blocks of n_slices in all.  best (3 entries) receives the wrap tile,
 * the flush and the scan chunk; ms_out (10 entries: wrap 0, 1, 2, flush 64,
 * 32, 2, 1, the three scan chunks in that order; may be NULL) the ms per
 * slice of each, -1 where a shape does not fit or does not apply.  Uneven
 * batches tune each class; best is the first class's. */
int pqmc_batch_autotune_tiles(pqmc_batch* batch, int loop, int first_tc, int n_slices,
                              int* best, double* ms_out);
/* slices tc = first_tc .. first_tc+n_slices-1 of sweep `loop` of every chain */
int pqmc_batch_sweep_slices(pqmc_batch* batch, int loop, int first_tc, int n_slices);
/* init_expKV and init_g_T0(1) (mod_evolution.f90:46-111) of every chain
 * (the fields set per chain first).  Mixed batches build the Q/D strings of
 * all chains together (double-float propagation + CholeskyQR2). */
int pqmc_batch_init(pqmc_batch* batch);
/* the CUDA stream of the batch (cudaStream_t): a batched call starts after
 * the work queued on it and the call's last work is ordered before later
 * work on it (the chain groups run on their own streams in between) */
int pqmc_batch_stream(pqmc_batch* batch, void** stream);
/* info[5] = {chains, chain groups (streams), delay depth, flush engine,
 * precision}; the groups default to one per 8 chains (at most 8) and can
 * be set with the environment variable PQMC_BATCH_GROUPS (1..16) at creation.
 * A mixed batch wraps G with whole columns staged in shared memory where
 * they fit; PQMC_WRAP_COLS=0 at creation keeps the per-block gather form
 * (the same arithmetic, entry for entry). */
int pqmc_batch_info(pqmc_batch* batch, int* info);
/* Uneven batches (mixed precision): chains of different geometry (Ns, Lt,
 * families) are grouped into classes of equal geometry; each class runs
 * as a homogeneous batch with its own streams, chain groups, delay depth
 * and slice graphs, and the classes interleave their slices within one
 * call (pqmc_batch_sweep: every chain one sweep of its own ntime slices).
 * pqmc_batch_classes gives the number of classes (1 for an even batch);
 * pqmc_batch_class_info(k) fills info[6] = {chains, Ns, ntime, delay depth,
 * flush engine, chain groups} of class k.  Chain indices stay those of the
 * models array. */
int pqmc_batch_classes(pqmc_batch* batch, int* n);
/* Field blocks of every chain in one call: slices first_time ..
 * first_time+n_times-1 of each chain's boson_field (clipped to the chain's
 * ntime), host blocks chain after chain, each (n_bf, n) column-major.
 * to_device = 1 copies host -> device and refreshes expKV of those slices
 * (the batched pqmc_set_field_slices), 0 copies device -> host.  The copies
 * are queued on the chains' streams together and the call returns when they
 * are done; with pinned host memory they overlap each other. */
int pqmc_batch_field_slices(pqmc_batch* batch, int first_time, int n_times, double* host, int to_device);
/* pqmc_get_state of every chain (states[n_chains]) with one wait */
int pqmc_batch_states(pqmc_batch* batch, pqmc_state* states);
int pqmc_batch_class_info(pqmc_batch* batch, int k, int* info);
/* CUDA-event timers per phase of the mixed family step; set_timing clears
 * the totals, get_timing returns PQMC_N_PHASES totals (ms) and counts. */
#define PQMC_PHASE_PREP      0   /* ran2 draws + proposal data           */
#define PQMC_PHASE_SCAN      1   /* sequential ratios, delayed panels     */
#define PQMC_PHASE_FLUSH     2   /* tensor-core rank-K flush G += A B     */
#define PQMC_PHASE_WRAP      3   /* two-way wrap by a family             */
#define PQMC_PHASE_RECOMPUTE 4   /* stabilised recompute (get_g_scratch)  */
#define PQMC_PHASE_SPLIT     5   /* BF16 split of the panels for tcgen05  */
#define PQMC_N_PHASES        6
int pqmc_batch_set_timing(pqmc_batch* batch, int enable);
int pqmc_batch_get_timing(pqmc_batch* batch, double* ms, long long* launches);
/* Per chain (rounds[n_chains]): the rank-K flushes that had panel columns
 * to fold in since the last pqmc_batch_set_timing, i.e. the number of
 * read-modify-writes of the chain's G by the flush. */
int pqmc_batch_flush_rounds(pqmc_batch* batch, long long* rounds);
/* Per chain (no reference counterpart), since the last
 * pqmc_batch_set_timing(batch, 1): out[3i] the SM cycles the chain's
 * sequential scan CTA ran (device clock64 from its start to its last
 * bookkeeping, summed over the scan rounds), out[3i+1] the moves it
 * accepted and out[3i+2] the proposals it rejected.  Counted only while
 * phase timing is on. */
int pqmc_batch_scan_profile(pqmc_batch* batch, long long* out);
/* Slice graphs (mixed batches, on by default; no reference counterpart):
 * the family steps of a slice (draws, proposals, scan rounds, flushes,
 * wraps) are captured once per chain group, direction and G-buffer parity
 * into a
 * CUDA graph and replayed for every later slice; the slice's time index
 * lives in device memory, so one graph serves all slices.  The stabilised
 * recompute and the measurement window still run as plain launches, and
 * phase timing (pqmc_batch_set_timing) bypasses the graphs.  Results are
 * bit-identical with and without graphs. */
int pqmc_batch_set_graphs(pqmc_batch* batch, int enable);
/* number of captured slice graphs held by the batch */
int pqmc_batch_graph_count(pqmc_batch* batch, int* n);

/* ---- recompute without device allocation ---------------------------- */
/* No counterpart in the reference.  g_out = R (X^H R)^-1 X^H and
 * logdet_out = log det(X^H R) (complex), i.e. cal_g_and_det_T0 without the
 * D-string and TR/ncopy terms, for callers that cannot call cudaMalloc:
 * hosts that hand the whole device to a fixed memory arena at start-up (a
 * further allocation would fail or fragment it) and Fortran drivers whose
 * only CUDA binding is this library (they have no way to allocate device
 * memory of their own).  All pointers are DEVICE pointers: x_left and rmat
 * are Ns x nelec complex, column-major; g_out is Ns x Ns; logdet_out holds 2
 * doubles.  `stream` is a cudaStream_t (NULL: legacy default stream); the
 * call copies the pivot flag of its LU to the host and synchronises the
 * stream before it returns, so it cannot be recorded into a CUDA graph: on a
 * stream that is being captured it returns PQMC_ERR_ARG without touching
 * the GPU (the capture stays valid).  On PQMC_ERR_SINGULAR (an exact zero
 * pivot) g_out and logdet_out have been overwritten and hold no meaningful
 * values.  Work space: one file-scope device array of about 3.2 MB, reserved
 * when the library loads and held by every GPU that loads it until the
 * process exits; its device address is looked up on every call with the
 * caller's device current.  Sizes above PQMC_NOALLOC_MAX_NS /
 * PQMC_NOALLOC_MAX_NELEC return PQMC_ERR_ARG.  Every call shares that array,
 * which keeps the last call's contents: calls that overlap on the GPU race. */
#define PQMC_NOALLOC_MAX_NS 512
#define PQMC_NOALLOC_MAX_NELEC 256
int pqmc_cal_g_and_det_noalloc(const double* x_left, const double* rmat, int ns, int nelec, double* g_out,
                               double* logdet_out, void* stream);

/* ---- validation of the exact round update ---------------------------- */
/* No counterpart in the reference.  Applies to g (HOST, Ns x Ns complex,
 * column-major, in/out) the combined update of k/dim accepted moves of one
 * family, exactly as a mixed batch does after a scan round (the sequential
 * rank-dim updates of update_phonon_field, src/mod_update.f90:146-192):
 *   g <- g + g(:,S) Delta_S W^-1 (E_S - g(S,:)),  W = I + g(S,S) Delta_S,
 * with S = sites[0..k) (0-based, dim per move, in acceptance order) and
 * Delta_S block diagonal (delta: k/dim blocks of dim x dim complex,
 * column-major).  The arithmetic is the batch's: W^-1 from an FP32
 * Gauss-Jordan refined by one Newton step with a double-float residual, and
 * Ozaki-split BF16 tensor-core products.
 * Limits: 1 <= dim <= 4, k <= 64, k % dim == 0, k <= ns <= 4096. */
int pqmc_exact_update_check(int ns, int k, int dim, const int* sites, const double* delta, double* g);
/* The same with the flush chosen: 64 (k_xgemm<1>), 32 (k_xflush2), or 2 / 1
 * (the pipeline k_xflushp, CTAs per row tile). */
int pqmc_exact_update_check_tile(int ns, int k, int dim, const int* sites, const double* delta, double* g,
                                 int flush_tile);

/* ---- validation of the recompute's GEMMs ------------------------------- */
/* No counterpart in the reference (zgemm there).  C_i = op(A_i) op(B_i) for
 * i < count, complex FP64 on the HOST, column-major, the count matrices of
 * each operand consecutive (lda x cols, ldb x cols, ldc x n each); ta, tb
 * 'N' (as is) or 'C' (conjugate transpose); op(A) m x k, op(B) k x n.
 * engine as pqmc_batch_set_gemm_engine. */
int pqmc_recompute_gemm_check(char ta, char tb, int m, int n, int k, int count, const double* a, int lda,
                              const double* b, int ldb, double* c, int ldc, int engine);

/* ---- introspection --------------------------------------------------- */
const char* pqmc_version(void);
const char* pqmc_last_error(void);
/* number of kernel launches issued by this library since load */
int64_t pqmc_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* PQMC_GB300_H */
