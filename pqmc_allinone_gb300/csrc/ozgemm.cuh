// ozgemm.cuh -- the recompute's complex GEMMs on the tensor cores (ozgemm.cu)
#pragma once
#include "common.cuh"

namespace pqmc {

struct OgDesc {   // one chain of a batched product C = op(A) op(B)
  const cplx* A;        // FP64 complex, column-major, lda
  const cplx* B;        // FP64 complex, column-major, ldb
  float4* C;            // column-major, ldc: double-float {re_hi, im_hi, re_lo, im_lo}, or FP64 complex
  unsigned char* img;   // slice images: ozgemm_img_bytes(m, n)
  int* err;             // PQMC_ERR_TIMEOUT when a wait gives up (may be null)
};

int ozgemm_setup();   // raises the product kernel's dynamic shared-memory limit
size_t ozgemm_img_bytes(int m, int n);
// C_c = op(A_c) op(B_c) for count chains, ta / tb in {'N', 'C'}; op(A) is
// m x k, op(B) k x n; C in FP64 when out_fp64, else double-float;
// stream-ordered, no synchronisation
int ozgemm_batched(cudaStream_t s, char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc,
                   const OgDesc* d_desc, int count, int out_fp64);

}  // namespace pqmc
