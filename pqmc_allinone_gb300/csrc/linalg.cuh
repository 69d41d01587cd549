// linalg.cuh -- host launchers of the FP64 complex dense kernels (linalg.cu)
#pragma once
#include "common.cuh"

namespace pqmc {
// C = alpha*op(A)*op(B) + beta*C, ta/tb in {'N','C'}
int zgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, cplx alpha, const cplx* A, int lda,
          const cplx* B, int ldb, cplx beta, cplx* C, int ldc);
// Householder QR, Q overwrites A (m x n), d = diag(R); tau: n scratch
int house_qr(cudaStream_t s, int m, int n, cplx* A, cplx* tau, cplx* d);
// the same, also returning R (n x n upper triangle, column-major) and
// ln det Q (a phase) when R / lndet are not null
int house_qr_r(cudaStream_t s, int m, int n, cplx* A, cplx* tau, cplx* d, cplx* R, cplx* lndet);
// LU with partial pivoting in place; info: device int
int lu_factor(cudaStream_t s, int n, cplx* A, int* ipiv, int* info, cplx* lcol);
int lu_solve(cudaStream_t s, int n, int nrhs, const cplx* LU, const int* ipiv, cplx* B, int ldb);
int lu_logdet(cudaStream_t s, int n, const cplx* LU, const int* ipiv, cplx* out);
int herm_t(cudaStream_t s, int m, int n, const cplx* a, cplx* out);
int coop_grid(const void* fn, int threads, int want);
}  // namespace pqmc
