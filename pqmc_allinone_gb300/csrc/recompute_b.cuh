// recompute_b.cuh -- batched stabilised recompute (recompute_b.cu)
#pragma once
#include <vector>
#include "chain.cuh"

struct dfc;

namespace pqmc {
struct GemmArgs;
struct ConvArgs;
struct CholArgs;
struct GJArgs;
struct PropArgs;
struct WeightArgs;
struct OgDesc;

struct BatchRecompute {
  int C = 0, ns = 0, ne = 0;
  cudaStream_t stream = nullptr;
  std::vector<pqmc_chain*> cs;
  GemmArgs* d_gemm = nullptr;
  ConvArgs* d_conv = nullptr;       // the operand splits of each GEMM slot
  float4* split_a = nullptr;        // A and B of a GEMM in double-float, per chain (ns x ne each)
  float4* split_b = nullptr;
  CholArgs* d_chol = nullptr;
  GJArgs* d_gj = nullptr;
  PropArgs* d_prop = nullptr;
  WeightArgs* d_weight = nullptr;
  ::dfc* work_df = nullptr;
  cplx* tmpX = nullptr;
  cplx* gram = nullptr;
  cplx* rinv = nullptr;
  cplx* pbp = nullptr;
  cplx* wmat = nullptr;
  cplx* logdet = nullptr;
  cplx* piv = nullptr;
  int* perm = nullptr;
  int* status = nullptr;
  ::dfc* ekv_df = nullptr;   // expKV of one block of slices in double-float, per chain
  size_t ekv_stride = 0;
  int ekv_slices = 0;
  bool gj_cluster = false;   // (L R)^-1 on a cluster of blocks with the matrix in shared memory
  // the GEMMs' engine: 0 the compensated double-float product on the FP32
  // pipe (k_dfgemm2), 1 the Ozaki-split product on the tensor cores
  // (ozgemm.cu; set by setup unless PQMC_RECOMPUTE_GEMM=0)
  int engine = 0;
  OgDesc* d_og = nullptr;
  unsigned char* og_img = nullptr;   // slice images, og_stride bytes per chain
  size_t og_stride = 0;
  int* err = nullptr;                // device error word for a wait that gives up (may be null)

  ~BatchRecompute();
  int setup(const std::vector<pqmc_chain*>& chains, cudaStream_t s);
  int set_engine(int e);
  int gemm(char ta, char tb, int m, int n, int k, const std::vector<GemmArgs>& a, int slot, int accumulate);
  int cholqr2(const std::vector<cplx*>& X, const std::vector<cplx*>& D);
  int g_and_det(const std::vector<cplx*>& XL, const std::vector<cplx*>& R, const std::vector<cplx*>& Gcur,
                const std::vector<cplx*>& Gnew, bool compare, int blk1, bool g_df);
  int propagate(const std::vector<cplx*>& X, int t_from, int t_to, bool forward);
  int scratch(int time, bool forward, int parity);   // G buffers of the mixed sweep: current = parity
  int init_g();   // init_g_T0(1) of every chain (needs ntime % ngroup == 0)
};
}  // namespace pqmc
