// noalloc.cu -- pqmc_cal_g_and_det_noalloc: the Green's-function recompute
// from stabilised factors without any device allocation.
//
// Some callers cannot call cudaMalloc: hosts that hand the whole device to a
// fixed memory arena at start-up (any further allocation fails or fragments
// the arena), and Fortran drivers whose only CUDA binding is this C library
// (they have no allocator of their own to call).  For them this entry point
// keeps its work space in one file-scope device array of fixed size,
// reserved when the library is loaded and held by every GPU that loads it
// until the process exits.
//
// Limits: ns <= PQMC_NOALLOC_MAX_NS and nelec <= PQMC_NOALLOC_MAX_NELEC; larger
// problems are rejected with PQMC_ERR_ARG.  Every call uses the same array,
// so calls that overlap on the GPU (two host threads, or two streams without
// ordering between them) race on it.  The array keeps the last call's
// contents; this routine writes every word it reads before reading it.  The
// call ends by copying the LU pivot flag to the host and synchronising the
// stream; on PQMC_ERR_SINGULAR the outputs have been overwritten with
// meaningless values.  Because of that read-back the call cannot be
// recorded into a CUDA graph: on a capturing stream it returns PQMC_ERR_ARG
// before it touches the GPU, and the capture stays valid.
#include "chain.cuh"
#include "linalg.cuh"

namespace {

constexpr int kMaxNs = PQMC_NOALLOC_MAX_NS;
constexpr int kMaxNe = PQMC_NOALLOC_MAX_NELEC;
// complex words: P^H B P (ne*ne), L = X^H (ne*ns), LU scratch column (ne)
constexpr size_t kCplxWords = (size_t)kMaxNe * kMaxNe + (size_t)kMaxNe * kMaxNs + kMaxNe;
// int words: pivots (ne) and the LU info flag
constexpr size_t kIntWords = kMaxNe + 64;
constexpr size_t kScratchBytes = kCplxWords * sizeof(double2) + kIntWords * sizeof(int);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The host-side name g_noalloc_scratch is only a stand-in for the device
// array; its device address is looked up on every call, with the caller's
// device current (a cheap query, and never stale after a cudaDeviceReset).
int scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    pqmc::set_error("cal_g_and_det_noalloc: cudaGetSymbolAddress -> %s", cudaGetErrorString(e));
    return PQMC_ERR_CUDA;
  }
  *out = p;
  return PQMC_OK;
}

}  // namespace

extern "C" int pqmc_cal_g_and_det_noalloc(const double* x_left, const double* rmat, int ns, int nelec, double* g_out,
                                          double* logdet_out, void* stream) {
  if (!x_left || !rmat || !g_out || !logdet_out) {
    pqmc::set_error("cal_g_and_det_noalloc: null pointer argument");
    return PQMC_ERR_ARG;
  }
  if (ns < 1 || nelec < 1 || nelec > ns || ns > kMaxNs || nelec > kMaxNe) {
    pqmc::set_error("cal_g_and_det_noalloc: ns=%d nelec=%d outside 1 <= nelec <= ns, ns <= %d, nelec <= %d", ns,
                    nelec, kMaxNs, kMaxNe);
    return PQMC_ERR_ARG;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  PQMC_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) {
    pqmc::set_error("cal_g_and_det_noalloc: the stream is being captured; the call reads its LU pivot flag back "
                    "and synchronises the stream, which a capture does not allow");
    return PQMC_ERR_ARG;
  }
  void* base = nullptr;
  PQMC_TRY(scratch_address(&base));
  cplx* pbp = reinterpret_cast<cplx*>(base);
  cplx* lmat = pbp + (size_t)kMaxNe * kMaxNe;
  cplx* lcol = lmat + (size_t)kMaxNe * kMaxNs;
  int* ipiv = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(base) + kCplxWords * sizeof(double2));
  int* info = ipiv + kMaxNe;
  const cplx* X = reinterpret_cast<const cplx*>(x_left);
  const cplx* R = reinterpret_cast<const cplx*>(rmat);
  cplx* G = reinterpret_cast<cplx*>(g_out);
  // P^H B P = X^H R  (cal_g_and_det_T0, src/mod_evolution.f90:344)
  PQMC_TRY(pqmc::zgemm(s, 'C', 'N', nelec, nelec, ns, mk(1.0), X, ns, R, ns, mk(0.0), pbp, nelec));
  // log det (:345) and the LU factors for the inverse (:347)
  PQMC_TRY(pqmc::lu_factor(s, nelec, pbp, ipiv, info, lcol));
  PQMC_TRY(pqmc::lu_logdet(s, nelec, pbp, ipiv, reinterpret_cast<cplx*>(logdet_out)));
  // g_h = R (P^H B P)^-1 L with L = X^H  (:349-350)
  PQMC_TRY(pqmc::herm_t(s, ns, nelec, X, lmat));
  PQMC_TRY(pqmc::lu_solve(s, nelec, ns, pbp, ipiv, lmat, nelec));
  PQMC_TRY(pqmc::zgemm(s, 'N', 'N', ns, ns, nelec, mk(1.0), R, ns, lmat, nelec, mk(0.0), G, ns));
  int h_info = 0;
  PQMC_CUDA(cudaMemcpyAsync(&h_info, info, sizeof(int), cudaMemcpyDeviceToHost, s));
  PQMC_CUDA(cudaStreamSynchronize(s));
  if (h_info != 0) {
    pqmc::set_error("cal_g_and_det_noalloc: zero pivot %d in P^H B P", h_info);
    return PQMC_ERR_SINGULAR;
  }
  return PQMC_OK;
}
