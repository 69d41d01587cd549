// tc.cuh -- inline-PTX helpers shared by the batched kernels: mbarriers,
// 1-D and 2-D bulk copies (TMA) between global and shared memory, and the
// tcgen05 pieces (shared-memory operand and instruction descriptors, MMA
// issue and commit, tensor-memory loads) with the tile-image layout the
// tensor-core kernels read.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <utility>

namespace pqmc {

// ---- 1-D bulk copies (TMA) global -> shared with mbarrier completion ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok;
}
// wait for the phase of parity `parity` to complete; false after ~2 s
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > (4LL << 30)) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(b))
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
// 2-D tiled TMA load of the box at (x, y) of the tensor map into shared memory
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(b))
      : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_addr(ssrc)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit_wait_all() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- tile images (no-swizzle K-major core matrices) ----
constexpr int UM_KP = 64;                    // panel columns per flush on this path (delay depth <= 64)
constexpr int UM_IMG = 128 * 2 * UM_KP * 2;  // bytes per tile image slot (32 KB)

__host__ __device__ __forceinline__ int um_rtiles(int ns) { return (ns + 127) / 128; }
__host__ __device__ __forceinline__ int um_ctiles(int ns) { return (ns + 63) / 64; }
__host__ __device__ __forceinline__ size_t um_chain_bytes(int ns) {
  return (size_t)3 * (um_rtiles(ns) + um_ctiles(ns)) * UM_IMG;
}
// row groups of row tile t, column groups of column tile t
__host__ __device__ __forceinline__ int um_rg(int ns, int t) {
  const int g = (ns - 128 * t + 7) / 8;
  return g < 16 ? g : 16;
}
__host__ __device__ __forceinline__ int um_cg(int ns, int t) {   // 4 or 8, so im starts at TMEM column 32 or 64
  const int g = (ns - 64 * t + 7) / 8;
  return g <= 4 ? 4 : 8;
}
// byte offset of (row, k) in a tile image of nrg row groups
__device__ __forceinline__ int um_off(int row, int k, int nrg) {
  return (k >> 3) * nrg * 128 + (row >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// shared-memory operand descriptor (no swizzle, K-major), Blackwell format
__device__ __forceinline__ uint64_t um_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t dsc = (uint64_t)((saddr >> 4) & 0x3FFFu);
  dsc |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  dsc |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  dsc |= (uint64_t)1 << 46;   // descriptor version 1 (tcgen05)
  return dsc;                 // base offset 0, layout type 0 = no swizzle
}
// instruction descriptor: kind::f16, D = F32, A = B = BF16, both K-major,
// M = 128, N = n (a multiple of 16, at most 256)
__device__ __forceinline__ uint32_t um_idesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void um_mma(uint32_t dtm, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtm),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void um_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}
__device__ __forceinline__ void um_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void um_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
// 32 lanes x 32 consecutive FP32 columns of tensor memory into registers
__device__ __forceinline__ void um_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
// 32 lanes x 16 consecutive FP32 columns of tensor memory into registers
__device__ __forceinline__ void um_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// a launch of k on stream st, at priority prio when use is set (the
// attribute also marks the node when the stream is being captured)
template <typename... P, typename... A>
static cudaError_t launch_at(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool use, int prio,
                             A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  if (use) {
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = prio;
    cfg.attrs = at;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

}  // namespace pqmc
