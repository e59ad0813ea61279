// mh_bf16x3.cu -- the FP32 complex LU trailing update (the factors of MH_PREC_MIXED) on the
// BF16 tensor cores by three-way splitting.
//
// Every FP32 entry x of L21 and U12 is cut into three BF16 terms, x0 = bf16(x),
// x1 = bf16(x - x0), x2 = bf16(x - x0 - x1) (8 + 8 + 8 significant bits for FP32's 24), and
// A22 -= L21 U12 is accumulated in FP32 tensor memory from the six products x_p y_q with
// p + q <= 2; the three dropped products are 2^-24 of the leading one, the size of FP32
// rounding.  Each product of two BF16 terms is exact in FP32.  These factors only seed the
// FP64 iterative refinement (the FP64 residual decides convergence), so FP32 accuracy is all
// they need; the CUDA-core FP32 update they replace reached ~18 % of the FP32 FMA peak.
//
// Kernels per panel step (batched over the matrices):
//   bx3_split_rows: L21 -> A tiles [row tile][re/im][term] of 128 x 32 BF16 (8 KB each, in
//     the canonical no-swizzle K-major layout);
//   bx3_split_cols: U12 -> B tiles [column tile][re/im][term] of 128 x 32 BF16;
//   bx3_gemm: one CTA per (128-row tile, group of 128-column tiles, matrix).  The six A tiles
//     stay in shared memory, the B tiles are double-buffered through TMA bulk copies; per
//     column tile one thread issues 48 tcgen05.mma (M = N = 128, K = 16: 6 term pairs x 2
//     K-steps x 4 real products, the -Im Im product through the negate-A bit) into a Re and
//     an Im FP32 accumulator (256 TMEM columns).  The accumulators are double-buffered, so the
//     next tile's products run while this tile's epilogue subtracts its result from A22.
// Every wait is bounded: on timeout the kernel raises the caller's flag, drains its copies
// and products (bounded) and frees its tensor memory.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "mh_internal.cuh"
#include "mh_tc.cuh"

namespace mh {

namespace {

constexpr int kBxTerms = 3;
constexpr int kBxK = 32;                                 // panel width (the LU's kNB)
constexpr int kBxNB = kBxK;
constexpr int kBxTile = 128;                             // rows of an A tile = columns of a B tile
constexpr int kBxPlane = kBxTile * kBxK * 2;             // bytes of one 128 x 32 BF16 plane
constexpr int kBxTileBytes = 2 * kBxTerms * kBxPlane;    // 48 KB: re/im x 3 terms
constexpr int kBxGroupMax = 8;                           // column tiles per CTA: 1..8 from the
                                                         // launch-shape table (default 4)
constexpr int kBxThreads = 256;                          // two threads per output row
constexpr uint32_t kBxTmemCols = 512;                    // 2 buffers x (Re 128 + Im 128)
constexpr uint32_t kBxWaitPolls = 1u << 26;

__device__ __forceinline__ void split3(float x, __nv_bfloat16 (&t)[kBxTerms]) {
  t[0] = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(t[0]);
  t[1] = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(t[1]);
  t[2] = __float2bfloat16_rn(r2);
}

// eight consecutive K values of one row of a tile -> six 16-byte chunks (re/im x 3 terms)
__device__ __forceinline__ void store_terms8(unsigned char* tile, int r, int k8, const float2 (&v)[8]) {
  uint32_t pk[2][kBxTerms][4];
#pragma unroll
  for (int c = 0; c < 8; c += 2) {
    __nv_bfloat16 a0[kBxTerms], a1[kBxTerms], b0[kBxTerms], b1[kBxTerms];
    split3(v[c].x, a0);
    split3(v[c + 1].x, a1);
    split3(v[c].y, b0);
    split3(v[c + 1].y, b1);
#pragma unroll
    for (int p = 0; p < kBxTerms; ++p) {
      pk[0][p][c >> 1] = (uint32_t)__bfloat16_as_ushort(a0[p]) | ((uint32_t)__bfloat16_as_ushort(a1[p]) << 16);
      pk[1][p][c >> 1] = (uint32_t)__bfloat16_as_ushort(b0[p]) | ((uint32_t)__bfloat16_as_ushort(b1[p]) << 16);
    }
  }
  const uint32_t off = tc::kmajor_offset(r, k8, kBxK);
#pragma unroll
  for (int part = 0; part < 2; ++part)
#pragma unroll
    for (int p = 0; p < kBxTerms; ++p)
      *reinterpret_cast<uint4*>(tile + (part * kBxTerms + p) * kBxPlane + off) =
          make_uint4(pk[part][p][0], pk[part][p][1], pk[part][p][2], pk[part][p][3]);
}

// L21 of matrix b at panel step k: rows k+kb .. n-1, columns k .. k+kb-1 (kb <= 32); four
// threads per row, eight columns each
__device__ __forceinline__ void bx3_split_rows(int64_t bx, const BatchDesc& d, const float2* __restrict__ A, int64_t k, int kb, int64_t rest,
                                      int64_t ntile, unsigned char* __restrict__ tiles) {
  const int64_t t = bx * (int64_t)blockDim.x + threadIdx.x;
  const int64_t r = t >> 2;  // padded row of the trailing block
  const int kq = (int)(t & 3);
  const int64_t b = blockIdx.y;
  if (r >= ntile * kBxTile) return;
  // a grouped batch: this matrix's order, panel width and trailing size (the launch's tile
  // count stays the stride of the term tiles)
  const int64_t n = d.order(b);
  if (k + kBxNB >= n) return;
  kb = (int)((k + kBxNB < n) ? kBxNB : n - k);
  const float2* Ab = A + d.offset(b);
  const bool live = r < n - k - kb;
  float2 v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int kk = 8 * kq + c;
    v[c] = (live && kk < kb) ? Ab[(k + kb + r) + (k + kk) * n] : make_float2(0.f, 0.f);
  }
  store_terms8(tiles + (b * ntile + r / kBxTile) * (int64_t)kBxTileBytes, (int)(r % kBxTile), 8 * kq, v);
}

// U12 of matrix b at panel step k: rows k .. k+kb-1, columns k+kb .. n-1; four threads per
// column, eight rows each
__device__ __forceinline__ void bx3_split_cols(int64_t bx, const BatchDesc& d, const float2* __restrict__ A, int64_t k, int kb, int64_t rest,
                                      int64_t ntile, unsigned char* __restrict__ tiles) {
  const int64_t t = bx * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = t >> 2;  // padded column of the trailing block
  const int kq = (int)(t & 3);
  const int64_t b = blockIdx.y;
  if (c >= ntile * kBxTile) return;
  const int64_t n = d.order(b);
  if (k + kBxNB >= n) return;
  kb = (int)((k + kBxNB < n) ? kBxNB : n - k);
  const float2* Ab = A + d.offset(b);
  const bool live = c < n - k - kb;
  float2 v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int kk = 8 * kq + q;
    v[q] = (live && kk < kb) ? Ab[(k + kk) + (k + kb + c) * n] : make_float2(0.f, 0.f);
  }
  store_terms8(tiles + (b * ntile + c / kBxTile) * (int64_t)kBxTileBytes, (int)(c % kBxTile), 8 * kq, v);
}

// Both splits of a panel step in one launch: CTAs [0, half) cut L21, the rest U12.
__global__ void __launch_bounds__(256) bx3_split_kernel(BatchDesc d, const float2* __restrict__ A, int64_t k, int kb,
                                                        int64_t rest, int64_t ntile, int64_t half,
                                                        unsigned char* __restrict__ tA, unsigned char* __restrict__ tB) {
  if ((int64_t)blockIdx.x < half) bx3_split_rows(blockIdx.x, d, A, k, kb, rest, ntile, tA);
  else bx3_split_cols(blockIdx.x - half, d, A, k, kb, rest, ntile, tB);
}

__global__ void __launch_bounds__(kBxThreads) bx3_gemm_kernel(BatchDesc d, float2* __restrict__ A, int64_t k, int kb,
                                                            int64_t rest, int64_t ntile,
                                                            const unsigned char* __restrict__ tA,
                                                            const unsigned char* __restrict__ tB,
                                                            int* __restrict__ timeout_flag, int group) {
  extern __shared__ __align__(1024) unsigned char bsm[];
  __shared__ __align__(8) uint64_t mbar_load[2];
  __shared__ __align__(8) uint64_t mbar_mma[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t rt = blockIdx.x, b = blockIdx.z;
  const int64_t ct0 = blockIdx.y * (int64_t)group;
  // a grouped batch: CTAs past this matrix's trailing block leave before any barrier or
  // tensor-memory allocation
  const int64_t n = d.order(b);
  if (k + kBxNB >= n) return;
  kb = (int)((k + kBxNB < n) ? kBxNB : n - k);
  rest = n - k - kb;
  if (rt * kBxTile >= rest || ct0 * kBxTile >= rest) return;
  const int64_t ntile_b = (rest + kBxTile - 1) / kBxTile;
  const int ntiles = (int)((ntile_b - ct0) < group ? (ntile_b - ct0) : group);
  unsigned char* As = bsm;
  unsigned char* Bs[2] = {bsm + kBxTileBytes, bsm + 2 * kBxTileBytes};
  const unsigned char* srcA = tA + (b * ntile + rt) * (int64_t)kBxTileBytes;
  auto srcB = [&](int64_t ct) { return tB + (b * ntile + ct) * (int64_t)kBxTileBytes; };
  if (tid == 0) {
    tc::mbar_init(&mbar_load[0], 1);
    tc::mbar_init(&mbar_load[1], 1);
    tc::mbar_init(&mbar_mma[0], 1);
    tc::mbar_init(&mbar_mma[1], 1);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kBxTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  // a 48 KB tile as three 16 KB bulk copies
  auto load_tile = [&](unsigned char* dst, const unsigned char* src, uint64_t* bar) {
    for (int q = 0; q < kBxTileBytes; q += 16384) tc::bulk_g2s(dst + q, src + q, 16384, bar);
  };
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&mbar_load[0], 2 * kBxTileBytes);
    load_tile(As, srcA, &mbar_load[0]);
    load_tile(Bs[0], srcB(ct0), &mbar_load[0]);
    if (ntiles > 1) {
      tc::mbar_arrive_expect_tx(&mbar_load[1], kBxTileBytes);
      load_tile(Bs[1], srcB(ct0 + 1), &mbar_load[1]);
    }
  }
  const uint32_t id = tc::idesc_bf16_f32(kBxTile, kBxTile), id_neg = tc::idesc_bf16_f32_nega(kBxTile, kBxTile);
  constexpr uint32_t sbo = (kBxK / 8) * 128;  // 8-row core groups are K * 16 bytes apart
  const int lrow = tid & (kBxTile - 1), half = tid >> 7;  // TMEM lane (output row) and column half
  const int64_t r = rt * kBxTile + lrow;
  const bool row_live = r < rest;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  float2* crow = A + d.offset(b) + (k + kb + r) + (k + kb) * n;  // this thread's row of A22
  bool failed = false;
  int loads_pending = ntiles > 1 ? 2 : 1, mma_pending = 0;

  // the 48 products of column tile t into accumulator buffer t & 1
  auto issue = [&](int t) {
    tc::fence_after_sync();
    const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs[t & 1]);
    const uint32_t t_re = tmem + (uint32_t)(t & 1) * 256u, t_im = t_re + 128u;
    bool first = true;
#pragma unroll
    for (int p = 0; p < kBxTerms; ++p)
#pragma unroll
      for (int q = 0; q + p < kBxTerms; ++q)
#pragma unroll
        for (int kk = 0; kk < kBxK / 16; ++kk) {
          const uint32_t ko = (uint32_t)kk * 256;
          const uint64_t ar = tc::smem_desc(a0 + (uint32_t)p * kBxPlane + ko, 128, sbo);
          const uint64_t ai = tc::smem_desc(a0 + (uint32_t)(kBxTerms + p) * kBxPlane + ko, 128, sbo);
          const uint64_t br = tc::smem_desc(b0 + (uint32_t)q * kBxPlane + ko, 128, sbo);
          const uint64_t bi = tc::smem_desc(b0 + (uint32_t)(kBxTerms + q) * kBxPlane + ko, 128, sbo);
          const uint32_t acc = first ? 0u : 1u;
          tc::mma_bf16(t_re, ar, br, id, acc);
          tc::mma_bf16(t_re, ai, bi, id_neg, 1u);
          tc::mma_bf16(t_im, ar, bi, id, acc);
          tc::mma_bf16(t_im, ai, br, id, 1u);
          first = false;
        }
    tc::mma_commit(&mbar_mma[t & 1]);
  };
  // A22 -= the accumulators of column tile t (this thread: its row, 64 of the 128 columns)
  auto epilogue = [&](int t) {
    const int64_t cbase = (ct0 + t) * kBxTile + half * 64;
    const uint32_t t_re = tmem + lane_off + (uint32_t)(t & 1) * 256u + (uint32_t)(half * 64), t_im = t_re + 128u;
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 32) {
      // all 32 loads of A22 first (loads and stores through one pointer would otherwise be
      // issued one after another; 32 in flight per thread keep HBM busier than 16), then the
      // accumulators, then the stores
      float2 cv[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int64_t c = cbase + c0 + q;
        cv[q] = (row_live && c < rest) ? crow[c * n] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int h = 0; h < 32; h += 16) {
        float re[16], im[16];
        tc::tmem_ld16(t_re + (uint32_t)(c0 + h), re);
        tc::tmem_ld16(t_im + (uint32_t)(c0 + h), im);
        if (row_live) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int64_t c = cbase + c0 + h + q;
            if (c < rest) crow[c * n] = make_float2(cv[h + q].x - re[q], cv[h + q].y - im[q]);
          }
        }
      }
    }
  };

  for (int t = 0; t < ntiles && !failed; ++t) {
    bool ok = tc::mbar_wait(&mbar_load[t & 1], (uint32_t)((t >> 1) & 1), kBxWaitPolls);
    if (__syncthreads_or(!ok)) { failed = true; break; }
    --loads_pending;
    if (tid == 0) issue(t);
    ++mma_pending;
    if (t > 0) {
      // tile t-1: its products are done, so its B buffer takes tile t+1 and its result is read
      ok = tc::mbar_wait(&mbar_mma[(t - 1) & 1], (uint32_t)(((t - 1) >> 1) & 1), kBxWaitPolls);
      if (__syncthreads_or(!ok)) { failed = true; break; }
      --mma_pending;
      tc::fence_after_sync();
      if (t + 1 < ntiles) {
        if (tid == 0) {
          tc::mbar_arrive_expect_tx(&mbar_load[(t + 1) & 1], kBxTileBytes);
          load_tile(Bs[(t + 1) & 1], srcB(ct0 + t + 1), &mbar_load[(t + 1) & 1]);
        }
        ++loads_pending;
      }
      epilogue(t - 1);
      // every read of buffer (t-1) & 1 is done before tile t+1's products overwrite it
      tc::fence_before_sync();
      __syncthreads();
    }
  }
  if (!failed) {
    const int t = ntiles - 1;
    const bool ok = tc::mbar_wait(&mbar_mma[t & 1], (uint32_t)((t >> 1) & 1), kBxWaitPolls);
    if (__syncthreads_or(!ok)) failed = true;
    else {
      --mma_pending;
      tc::fence_after_sync();
      epilogue(t);
    }
  }
  if (failed) {
    // reported by the host as a timeout; drain what is in flight (bounded) before the tensor
    // memory and the shared memory are released
    if (tid == 0) atomicExch(timeout_flag, 1);
    if (mma_pending > 0) {
      tc::mbar_wait(&mbar_mma[0], 0, kBxWaitPolls);
      tc::mbar_wait(&mbar_mma[1], 0, kBxWaitPolls);
    }
    if (loads_pending > 0) {
      tc::mbar_wait(&mbar_load[0], 0, kBxWaitPolls);
      tc::mbar_wait(&mbar_load[1], 0, kBxWaitPolls);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kBxTmemCols);
}

}  // namespace

size_t bx3_workspace_bytes(int64_t n, int64_t batch) {
  const int64_t t = (n + kBxTile - 1) / kBxTile;
  return (size_t)batch * 2 * (size_t)t * kBxTileBytes + 1024;
}

void bx3_trailing_update(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, float2* A, int64_t k, int kb,
                         void* ws, int* timeout_flag) {
  const int64_t rest = d.n - k - kb;
  if (rest <= 0) return;
  const int64_t nt = (rest + kBxTile - 1) / kBxTile, nt_max = (d.n + kBxTile - 1) / kBxTile;
  unsigned char* tA = static_cast<unsigned char*>(ws);
  unsigned char* tB = tA + d.batch * nt_max * (int64_t)kBxTileBytes;
  dim3 gs((unsigned)(nt * 4), (unsigned)d.batch);  // 4 threads per row / column, 256 per CTA; rows then columns
  MH_LAUNCH(lc, st, "lu_bx3_split", bx3_split_kernel<<<gs, 256, 0, st>>>(d, A, k, kb, rest, nt, nt * 2, tA, tB));
  const size_t smem = 3 * (size_t)kBxTileBytes;
  cudaFuncSetAttribute(bx3_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int group = lc.tile(d.n).bx_group;
  group = group < 1 ? 1 : (group > kBxGroupMax ? kBxGroupMax : group);
  dim3 gg((unsigned)nt, (unsigned)((nt + group - 1) / group), (unsigned)d.batch);
  MH_LAUNCH(lc, st, "lu_gemm_bx3",
            bx3_gemm_kernel<<<gg, kBxThreads, smem, st>>>(d, A, k, kb, rest, nt, tA, tB, timeout_flag, group));
}

}  // namespace mh
