// common.cuh -- complex FP64 helpers, error plumbing and launch accounting
// shared by every translation unit of libpqmc_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <atomic>
#include "../../include/pqmc_gb300.h"
#include "../../include/pqmc_boxmuller.h"

typedef double2 cplx;

__host__ __device__ __forceinline__ cplx mk(double r, double i = 0.0) { return make_double2(r, i); }
__host__ __device__ __forceinline__ cplx cadd(cplx a, cplx b) { return mk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cplx csub(cplx a, cplx b) { return mk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cplx cneg(cplx a) { return mk(-a.x, -a.y); }
__host__ __device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ cplx cscale(cplx a, double s) { return mk(a.x * s, a.y * s); }
// a + x*y with four fused multiply-adds (the FP64 pipe issues one warp
// instruction per 32 ns on GB300, so instruction count is what matters)
__host__ __device__ __forceinline__ cplx cfma(cplx x, cplx y, cplx a) {
  return mk(fma(x.x, y.x, fma(-x.y, y.y, a.x)), fma(x.x, y.y, fma(x.y, y.x, a.y)));
}
__host__ __device__ __forceinline__ cplx cconj(cplx a) { return mk(a.x, -a.y); }
// conj(a)*b
__host__ __device__ __forceinline__ cplx cmulc(cplx a, cplx b) {
  return mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double cabsd(cplx a) { return hypot(a.x, a.y); }
// Smith's complex division (the form gfortran and zladiv use)
__host__ __device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return mk((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return mk((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}
__host__ __device__ __forceinline__ cplx clog_(cplx a) { return mk(log(hypot(a.x, a.y)), atan2(a.y, a.x)); }
__host__ __device__ __forceinline__ cplx cexp_(cplx a) {
  double e = exp(a.x);
  return mk(e * cos(a.y), e * sin(a.y));
}

// ---- host-side error and launch accounting ------------------------------
namespace pqmc {
void set_error(const char* fmt, ...);
extern std::atomic<int64_t> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace pqmc

#define PQMC_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e__ = (call);                                                  \
    if (e__ != cudaSuccess) {                                                  \
      pqmc::set_error("%s:%d %s -> %s", __FILE__, __LINE__, #call,             \
                      cudaGetErrorString(e__));                                \
      return PQMC_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

#define PQMC_LAUNCHED()                                                        \
  do {                                                                         \
    pqmc::count_launch();                                                      \
    cudaError_t e__ = cudaGetLastError();                                      \
    if (e__ != cudaSuccess) {                                                  \
      pqmc::set_error("%s:%d launch -> %s", __FILE__, __LINE__,                \
                      cudaGetErrorString(e__));                                \
      return PQMC_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

// raise a kernel's dynamic shared-memory limit to at least `bytes`, never
// lower it: batches of different sizes live side by side in one context
template <typename F>
inline cudaError_t raise_dyn_smem(F* fn, int bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, (const void*)fn);
  if (e != cudaSuccess) return e;
  if (a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

#define PQMC_TRY(expr)                                                         \
  do {                                                                         \
    int s__ = (expr);                                                          \
    if (s__ != PQMC_OK) return s__;                                            \
  } while (0)
