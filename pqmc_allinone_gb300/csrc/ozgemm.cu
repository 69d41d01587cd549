// ozgemm.cu -- batched complex C = op(A) op(B) for the stabilised recompute
// (recompute_b.cu) on the tensor cores, accurate to the double-float level.
//
// The operands are FP64 complex, column-major with leading dimensions lda,
// ldb, read as double-float; op is the identity or the conjugate transpose.
// The inner dimension is taken in chunks of 64 complex entries (128 real:
// the real GEMM [Ar | Ai] x [[Br | -Bi]; [Bi | Br]]).  Per chunk every row
// of op(A) and every column of op(B) is cut into OG_S = 6 BF16 slices on a
// power-of-two grid set by its largest entry in the chunk (ozaki.cuh),
// written as tile images in the no-swizzle K-major core-matrix layout.  One
// CTA per 128 x 32 tile of C streams the 6 + 6 half-images of a half of the
// chunk through 144 KB of shared memory and issues the 21 slice pairs
// i + j < 6 as tcgen05 BF16 products, each level i + j into its own FP32
// accumulator in tensor memory (6 x 64 columns).  Levels 0 to 4 are exact:
// a level-l term is an integer of at most 2 x 256 x 129 + (l - 1) x 129^2
// units of the level's grid, and 128 of them stay below 2^24.  Level 5 is
// rounded at 2^-24 of itself, 2^-64 of level 0.  (One accumulator for levels
// 3 to 5 would be truncated at every product step of the tensor core, ~120
// times per chunk, and hold the result to ~2^-41.)  The epilogue sums the
// six levels in double-float, smallest first, and writes C (first chunk) or
// adds to it (later chunks), also in double-float; the last chunk writes the
// double-float form {re_hi, im_hi, re_lo, im_lo} or FP64 complex in the same
// 16 bytes.  The product is good to a few 2^-48 of the row-by-column
// magnitudes, as the compensated k_dfgemm2 on the FP32 pipe that it stands
// in for.  Rows and columns keep FP32's exponent range: the grids of the
// finest products, 2^(ea + eb - 56), stay normal while ea + eb >= -70.
#include <algorithm>
#include <cuda_bf16.h>
#include "ozaki.cuh"
#include "ozgemm.cuh"
#include "tc.cuh"

namespace pqmc {

constexpr int OG_S = 6;                         // slices per operand
constexpr int OG_LV = OG_S;                     // accumulators: levels i + j = 0 .. OG_S - 1
constexpr int OG_FLOOR = -78;                   // exponent floor: 2^(e - 48) stays normal
static_assert(OG_FLOOR >= 8 * OG_S - 126, "exponent floor");
constexpr int OG_BN = 32;                       // complex columns of C per tile
constexpr int OG_BIMG = 2 * OG_BN * 2 * UM_KP * 2;   // bytes per B image: 64 rows x 128 k (16 KB)
constexpr int OG_HA = UM_IMG / 2, OG_HB = OG_BIMG / 2;   // bytes of a half (the re or the im k range)
constexpr int OG_SMEM = OG_S * (OG_HA + OG_HB);  // 144 KB
constexpr int OG_THREADS = 256;
static_assert(OG_LV * 2 * OG_BN <= 512, "accumulators fit in tensor memory");

__host__ __device__ __forceinline__ int og_ctiles(int n) { return (n + OG_BN - 1) / OG_BN; }
// column groups of 8 in column tile t: 2 or 4, so the im rows of the B image
// start at row 16 or 32 and N = 16 x groups is 32 or 64
__host__ __device__ __forceinline__ int og_cg(int n, int t) { return (n - OG_BN * t + 7) / 8 <= 2 ? 2 : 4; }

// op(A)(r, k) and op(B)(k, c) of FP64 operands as double-float
// (conjugate-transposed when trans)
__device__ __forceinline__ dfc og_a(const cplx* A, int ld, int r, int k, int trans) {
  const cplx v = trans ? A[k + (size_t)ld * r] : A[r + (size_t)ld * k];
  return dfc{df_make(v.x), df_make(trans ? -v.y : v.y)};
}
__device__ __forceinline__ dfc og_b(const cplx* B, int ld, int k, int c, int trans) {
  const cplx v = trans ? B[c + (size_t)ld * k] : B[k + (size_t)ld * c];
  return dfc{df_make(v.x), df_make(trans ? -v.y : v.y)};
}

// Slices of one chunk (inner indices k0 .. k0 + kn - 1, kn <= 64).  A CTA
// takes 32 rows of op(A) (CTAs 0 .. n_a - 1) or 32 columns of op(B) (the
// rest): lane = row (column), warp w = inner indices 8w .. 8w + 7, so a
// warp's image stores are 512 contiguous bytes.  The row's (column's)
// exponent comes from the largest |hi| over its kn entries (a maximum over
// the eight warps in shared memory).
//   A' row r = [Ar | Ai] at image k and 64 + k;
//   B' re row c = [Br | -Bi], im row 8 ncg + c = [Bi | Br] of its
//   32-column tile.
// Entries past kn (to the chunk's multiple of 16) are written as zeros.
// Images: the A images of row tile t at (t OG_S + slice) UM_IMG, then the
// B images of column tile t at (t OG_S + slice) OG_BIMG.
constexpr int OG_SL_ROWS = 32;                    // rows (columns) per slicing CTA
static_assert(OG_THREADS / 32 * 8 == UM_KP, "a warp per k group of the chunk");
__global__ void __launch_bounds__(OG_THREADS) k_og_slice(const OgDesc* D, int m, int n, int k0, int kn, int lda,
                                                        int ldb, int ta, int tb, int n_a) {
  __shared__ float s_mx[OG_THREADS / 32][OG_SL_ROWS];
  __shared__ OgDesc sd;
  const int lane = threadIdx.x & 31, kg = threadIdx.x >> 5;
  if (threadIdx.x == 0) sd = D[blockIdx.y];
  __syncthreads();
  const OgDesc& d = sd;
  const bool is_a = (int)blockIdx.x < n_a;
  const int idx = (is_a ? (int)blockIdx.x : (int)blockIdx.x - n_a) * OG_SL_ROWS + lane;
  const int lim = is_a ? m : n;
  const int kn16 = (kn + 15) & ~15;
  dfc v[8];
  float mx = 0.f;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int k = kg * 8 + u;
    v[u] = dfc_zero();
    if (idx < lim && k < kn) v[u] = is_a ? og_a(d.A, lda, idx, k0 + k, ta) : og_b(d.B, ldb, k0 + k, idx, tb);
    mx = fmaxf(mx, fmaxf(fabsf(v[u].re.hi), fabsf(v[u].im.hi)));
  }
  s_mx[kg][lane] = mx;
  __syncthreads();
  if (idx >= lim || kg * 8 >= kn16) return;   // no barrier follows
  float rm = 0.f;
#pragma unroll
  for (int w = 0; w < OG_THREADS / 32; ++w) rm = fmaxf(rm, s_mx[w][lane]);
  const int e = oz_exp_f<OG_FLOOR>(rm);
  uint32_t wr[OG_S][4], wi[OG_S][4];
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    float r0[OG_S], r1[OG_S], i0[OG_S], i1[OG_S];
    oz_split_n<OG_S>(v[2 * h].re.hi, v[2 * h].re.lo, e, r0);
    oz_split_n<OG_S>(v[2 * h + 1].re.hi, v[2 * h + 1].re.lo, e, r1);
    oz_split_n<OG_S>(v[2 * h].im.hi, v[2 * h].im.lo, e, i0);
    oz_split_n<OG_S>(v[2 * h + 1].im.hi, v[2 * h + 1].im.lo, e, i1);
#pragma unroll
    for (int sl = 0; sl < OG_S; ++sl) {
      wr[sl][h] = oz_pack2(r0[sl], r1[sl]);
      wi[sl][h] = oz_pack2(i0[sl], i1[sl]);
    }
  }
  if (is_a) {
    const int t = idx / 128, row = idx % 128, nrg = um_rg(m, t);
#pragma unroll
    for (int sl = 0; sl < OG_S; ++sl) {
      unsigned char* im = d.img + (size_t)(t * OG_S + sl) * UM_IMG;
      *reinterpret_cast<uint4*>(im + um_off(row, kg * 8, nrg)) = make_uint4(wr[sl][0], wr[sl][1], wr[sl][2], wr[sl][3]);
      *reinterpret_cast<uint4*>(im + um_off(row, UM_KP + kg * 8, nrg)) =
          make_uint4(wi[sl][0], wi[sl][1], wi[sl][2], wi[sl][3]);
    }
    return;
  }
  const int RT = um_rtiles(m);
  const int tj = idx / OG_BN, cc = idx % OG_BN, ncg = og_cg(n, tj), nrg = 2 * ncg;
  unsigned char* bimg = d.img + (size_t)RT * OG_S * UM_IMG;
  constexpr uint32_t NEG2 = 0x80008000u;   // the sign bits of two BF16: -x exactly
#pragma unroll
  for (int sl = 0; sl < OG_S; ++sl) {
    unsigned char* im = bimg + (size_t)(tj * OG_S + sl) * OG_BIMG;
    const uint4 r4 = make_uint4(wr[sl][0], wr[sl][1], wr[sl][2], wr[sl][3]);
    const uint4 i4 = make_uint4(wi[sl][0], wi[sl][1], wi[sl][2], wi[sl][3]);
    *reinterpret_cast<uint4*>(im + um_off(cc, kg * 8, nrg)) = r4;
    *reinterpret_cast<uint4*>(im + um_off(cc, UM_KP + kg * 8, nrg)) =
        make_uint4(i4.x ^ NEG2, i4.y ^ NEG2, i4.z ^ NEG2, i4.w ^ NEG2);
    *reinterpret_cast<uint4*>(im + um_off(8 * ncg + cc, kg * 8, nrg)) = i4;
    *reinterpret_cast<uint4*>(im + um_off(8 * ncg + cc, UM_KP + kg * 8, nrg)) = r4;
  }
}

__device__ __forceinline__ void og_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// C tile (128 x 32 complex) = (first ? 0 : C) + op(A) op(B) of one chunk;
// C column-major, ldc, in double-float {re_hi, im_hi, re_lo, im_lo} between
// chunks; the last chunk writes FP64 complex when fp64 is set
__global__ void __launch_bounds__(OG_THREADS, 1) k_og_gemm(const OgDesc* D, int m, int n, int kn, int ldc, int first,
                                                          int fp64) {
  __shared__ OgDesc sd;
  __shared__ __align__(8) uint64_t s_load[2], s_mma[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail, s_last;
  extern __shared__ __align__(1024) unsigned char og_dyn[];   // OG_S A half-images, then OG_S B half-images
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
  __syncthreads();
  const OgDesc& d = sd;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&s_taddr))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const uint32_t taddr = s_taddr;
  const int RT = um_rtiles(m);
  const int ti = (int)blockIdx.x % RT, tj = (int)blockIdx.x / RT;
  const int nrg_a = um_rg(m, ti), ncg = og_cg(n, tj), nrg_b = 2 * ncg;
  const int kn16 = (kn + 15) & ~15;
  if (tid == 0) {
    const uint32_t ka = (uint32_t)nrg_a * 128, kb = (uint32_t)nrg_b * 128;   // bytes per k group of 8
    const uint32_t part_a = (uint32_t)(kn16 / 8) * ka, part_b = (uint32_t)(kn16 / 8) * kb;
    const uint32_t h2a = (uint32_t)(UM_KP / 8) * ka, h2b = (uint32_t)(UM_KP / 8) * kb;
    const uint32_t base = smem_addr(og_dyn), bbase = base + OG_S * OG_HA, idesc = um_idesc(16u * (uint32_t)ncg);
    const unsigned char* aimg = d.img + (size_t)ti * OG_S * UM_IMG;
    const unsigned char* bimg = d.img + (size_t)RT * OG_S * UM_IMG + (size_t)tj * OG_S * OG_BIMG;
    uint32_t started = 0;
    for (int half = 0; half < 2; ++half) {
      if (half == 1) {   // the products of half 0 have read the buffer
        if (!mbar_wait_bounded(&s_mma[0], 0)) {
          s_fail = 1;
          break;
        }
        um_fence_after();
      }
      mbar_arrive_tx(&s_load[half], (uint32_t)OG_S * (part_a + part_b));
      for (int sl = 0; sl < OG_S; ++sl) {
        bulk_g2s(og_dyn + (size_t)sl * OG_HA, aimg + (size_t)sl * UM_IMG + half * h2a, part_a, &s_load[half]);
        bulk_g2s(og_dyn + (size_t)OG_S * OG_HA + (size_t)sl * OG_HB, bimg + (size_t)sl * OG_BIMG + half * h2b, part_b,
                 &s_load[half]);
      }
      if (!mbar_wait_bounded(&s_load[half], 0)) {
        s_fail = 1;
        mbar_wait_bounded(&s_load[half], 0);   // a second bounded wait for the copies in flight
        break;
      }
      um_fence_after();
      for (int i = 0; i < OG_S; ++i)
        for (int j = 0; i + j < OG_S; ++j) {
          const int l = i + j;
          for (int kk = 0; kk < kn16 / 16; ++kk) {
            const uint64_t ad = um_desc(base + i * OG_HA + kk * 2 * ka, ka, 128);
            const uint64_t bd = um_desc(bbase + j * OG_HB + kk * 2 * kb, kb, 128);
            um_mma(taddr + (uint32_t)(l * 2 * OG_BN), ad, bd, idesc, (started >> l) & 1u);
            started |= 1u << l;
          }
        }
      um_commit(&s_mma[half]);   // also tracks every earlier product
      s_last = half;
    }
  }
  const int q = warp & 3, hf = warp >> 2;
  const int r = ti * 128 + q * 32 + lane;
  const int col0 = tj * OG_BN + hf * 16, ncol = min(16, n - col0);
  __syncthreads();
  const int last = s_last;
  if (last >= 0) {   // every exit path waits for the last commit (it tracks all earlier products)
    if (!mbar_wait_bounded(&s_mma[last], 0)) s_fail = 1;
    um_fence_after();
  }
  __syncthreads();
  const uint32_t tbase = taddr + ((uint32_t)(q * 32) << 16);
  if (!s_fail) {
#pragma unroll 1
    for (int ch = 0; ch < 2; ++ch) {
      const int c0 = ch * 8;
      if (ncol <= c0) break;   // warp-uniform
      float re[OG_LV][8], im[OG_LV][8];
#pragma unroll
      for (int l = 0; l < OG_LV; ++l) {
        og_ld8(tbase + l * 2 * OG_BN + hf * 16 + c0, re[l]);
        og_ld8(tbase + l * 2 * OG_BN + 8 * ncg + hf * 16 + c0, im[l]);
      }
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (r < m) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c0 + c >= ncol) continue;
          // levels smallest first, in double-float
          df vr = df{re[OG_LV - 1][c], 0.f}, vi = df{im[OG_LV - 1][c], 0.f};
#pragma unroll
          for (int l = OG_LV - 2; l >= 0; --l) {
            vr = df_add(vr, df{re[l][c], 0.f});
            vi = df_add(vi, df{im[l][c], 0.f});
          }
          float4* p = d.C + r + (size_t)ldc * (col0 + c0 + c);
          if (!first) {
            const float4 g = *p;
            vr = df_add(df{g.x, g.z}, vr);
            vi = df_add(df{g.y, g.w}, vi);
          }
          if (fp64)
            *reinterpret_cast<cplx*>(p) = mk((double)vr.hi + (double)vr.lo, (double)vi.hi + (double)vi.lo);
          else
            *p = make_float4(vr.hi, vi.hi, vr.lo, vi.lo);
        }
      }
    }
  } else if (tid == 0 && d.err) {
    atomicExch(d.err, PQMC_ERR_TIMEOUT);
  }
  um_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(taddr) : "memory");
}

int ozgemm_setup() {
  PQMC_CUDA(raise_dyn_smem(k_og_gemm, OG_SMEM));
  return PQMC_OK;
}

size_t ozgemm_img_bytes(int m, int n) {
  return (size_t)OG_S * ((size_t)um_rtiles(m) * UM_IMG + (size_t)og_ctiles(n) * OG_BIMG);
}

int ozgemm_batched(cudaStream_t s, char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc,
                   const OgDesc* d_desc, int count, int out_fp64) {
  if (m <= 0 || n <= 0 || k <= 0 || count <= 0) {
    set_error("ozgemm: empty product (m %d, n %d, k %d, count %d)", m, n, k, count);
    return PQMC_ERR_ARG;
  }
  const int n_a = (m + OG_SL_ROWS - 1) / OG_SL_ROWS, n_b = (n + OG_SL_ROWS - 1) / OG_SL_ROWS;
  const int tiles = um_rtiles(m) * og_ctiles(n);
  for (int k0 = 0; k0 < k; k0 += UM_KP) {
    const int kn = std::min(UM_KP, k - k0);
    k_og_slice<<<dim3(n_a + n_b, count), OG_THREADS, 0, s>>>(d_desc, m, n, k0, kn, lda, ldb, ta == 'C', tb == 'C',
                                                              n_a);
    PQMC_LAUNCHED();
    k_og_gemm<<<dim3(tiles, count), OG_THREADS, OG_SMEM, s>>>(d_desc, m, n, kn, ldc, k0 == 0 ? 1 : 0,
                                                              (out_fp64 && k0 + kn == k) ? 1 : 0);
    PQMC_LAUNCHED();
  }
  return PQMC_OK;
}

}  // namespace pqmc
