// mh_zgemv_tc.cu -- Y = A X (or R = B - A X) for a batch of dense complex FP64 matrices and up
// to 8 right-hand sides, FP64-accurate, on the BF16 tensor cores (Ozaki splitting).
//
// With 7 right-hand sides a complex matrix-vector product does 28 FP64 FMAs per 16 bytes of
// A, so on GB300 it is bound by the FP64 pipe, not by HBM (S B of the frequency sweep: 0.9
// TFLOP/s, 7.4 ms for 30 matrices of 2000 panels).  Here A is cut, 32 columns at a time,
// into eight balanced base-128 digits per entry (a 55-bit fixed point per row and block,
// exact in BF16), X likewise per column and block, and the digit products accumulate
// exactly in FP32 tensor memory, as in the LU's tensor-core update (mh_ozaki.cu).  Each
// block's exact partial sums are converted to FP64 once and added up over the blocks in
// FP64, so the result carries FP64 rounding (it feeds the FP64 residuals of the
// iterative refinement, which must be FP64-accurate).
//
//   zgemv_xsplit_kernel: X (n x g, g <= 8) -> per 32-row block one 128 x 32 BF16 operand
//     tile: row 16 q + 8 part + j is digit q of part (re/im) of column j, so digits q .. 7
//     stack along N; and one exponent per column and block.
//   zgemv_tc_kernel: one CTA (512 threads) per 128-row tile of one matrix, looping over the
//     32-column blocks: the FP64 block arrives by TMA bulk copies (one per column), four
//     threads per row cut it into 16 digit planes in shared memory (integer arithmetic on
//     the FP64 bit fields, no FP64 instructions), one thread issues 32 tcgen05.mma
//     (A digit p of Re A and Im A against the stacked X digits 0 .. 7-p, N = 16 (8-p)) into
//     one of two 256-column TMEM buffers, and while they run the previous block's
//     accumulators are combined (integers, then one FP64 add and two FMAs per real output).
// Every wait is bounded; on timeout the kernel raises the caller's flag, drains (bounded)
// and frees its tensor memory.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "mh_digits.cuh"
#include "mh_internal.cuh"
#include "mh_tc.cuh"

namespace mh {

namespace {

constexpr int kZvRows = 128;                 // rows per CTA (MMA M)
constexpr int kZvK = 32;                     // columns of A per block
constexpr int kZvDigits = 8;
constexpr int kZvRhs = 8;                    // right-hand sides per launch
constexpr int kZvPlane = kZvRows * kZvK * 2; // one 128 x 32 BF16 digit plane (8 KB)
constexpr int kZvA64 = kZvRows * kZvK * 16;  // the FP64 block (64 KB)
constexpr int kZvADig = 2 * kZvDigits * kZvPlane;  // 16 planes (128 KB)
constexpr int kZvXTile = kZvPlane;           // X operand tile: 128 N-rows x 32 K (8 KB)
constexpr int kZvThreads = 512;
constexpr uint32_t kZvTmemCols = 512;        // 2 buffers x (Re A: 128, Im A: 128)
constexpr uint32_t kZvWaitPolls = 1u << 26;
constexpr size_t kZvSmem = (size_t)kZvA64 + kZvADig + 2 * kZvXTile;

// BF16 bits of a small integer (|d| <= 64): through the FP32 magic number, exact
__device__ __forceinline__ uint32_t bf16_of_small(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return __float_as_uint(f) >> 16;
}

__device__ __forceinline__ void digits_of(long long X, int (&d8)[kZvDigits]) {
#pragma unroll
  for (int p = kZvDigits - 1; p > 0; --p) {
    const long long t = ((X + 64) & 127) - 64;
    d8[p] = (int)t;
    X = (X - t) >> 7;
  }
  d8[0] = (int)X;
}

__device__ __forceinline__ int scale_exp(double maxabs) {
  if (!(maxabs > 0.0)) return 0;
  int e;
  frexp(maxabs, &e);
  return e;
}

__device__ __forceinline__ double pow2i(int s) { return __longlong_as_double((long long)(s + 1023) << 52); }

// X columns r0 .. r0+g-1 of matrix b -> per block the operand tile and the column exponents
__global__ void __launch_bounds__(256) zgemv_xsplit_kernel(BatchDesc d, const double2* __restrict__ Xall,
                                                           int64_t xstride, int r0, int g, int64_t nkb,
                                                           unsigned char* __restrict__ xt, int* __restrict__ xexp) {
  const int64_t kb = blockIdx.x, b = blockIdx.y, n = d.n;
  const int j = threadIdx.x >> 5, kk = threadIdx.x & 31;  // warp j: column j, lane: row of the block
  const int64_t row = kb * kZvK + kk;
  double2 v = make_double2(0.0, 0.0);
  if (j < g && row < n) v = Xall[b * xstride + row + (int64_t)(r0 + j) * n];
  double mx = fmax(fabs(v.x), fabs(v.y));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  const int f = scale_exp(mx);
  if (kk == 0) xexp[(b * nkb + kb) * kZvRhs + j] = f;
  unsigned char* tile = xt + (b * nkb + kb) * (int64_t)kZvXTile;
  int dre[kZvDigits], dim[kZvDigits];
  digits_of(llrint(ldexp(v.x, 55 - f)), dre);
  digits_of(llrint(ldexp(v.y, 55 - f)), dim);
#pragma unroll
  for (int q = 0; q < kZvDigits; ++q) {
    const uint32_t o_re = tc::kmajor_offset(16 * q + j, kk, kZvK), o_im = tc::kmajor_offset(16 * q + 8 + j, kk, kZvK);
    *reinterpret_cast<uint16_t*>(tile + o_re) = (uint16_t)bf16_of_small(dre[q]);
    *reinterpret_cast<uint16_t*>(tile + o_im) = (uint16_t)bf16_of_small(dim[q]);
  }
}

// two consecutive FP32 TMEM columns of this thread's lane, no wait
__device__ __forceinline__ void tmem_ld2_nowait(uint32_t taddr, uint32_t& a, uint32_t& b) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(a), "=r"(b) : "r"(taddr) : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ int int_of_exact(uint32_t fbits) {
  return __float_as_int(__uint_as_float(fbits) + 12582912.0f) - 0x4B400000;
}

__global__ void __launch_bounds__(kZvThreads) zgemv_tc_kernel(BatchDesc d, const double2* __restrict__ Aall,
                                                            const double2* __restrict__ Ball,
                                                            double2* __restrict__ Yall, int64_t xstride, int r0,
                                                            int g, int64_t nkb,
                                                            const unsigned char* __restrict__ xt,
                                                            const int* __restrict__ xexp, int subtract,
                                                            int* __restrict__ timeout_flag) {
  extern __shared__ __align__(1024) unsigned char zsm[];
  __shared__ __align__(8) uint64_t mbar_load, mbar_mma;
  __shared__ uint32_t tmem_base;
  unsigned char* sA64 = zsm;                      // 32 columns x 128 rows x 16 B
  unsigned char* sAd = zsm + kZvA64;              // [part][digit] planes
  unsigned char* sX[2] = {sAd + kZvADig, sAd + kZvADig + kZvXTile};
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t n = d.n, b = blockIdx.y;
  const int64_t row0 = blockIdx.x * (int64_t)kZvRows;
  const int rows_valid = (int)((n - row0) < kZvRows ? (n - row0) : kZvRows);
  const double2* A = Aall + b * d.stride;
  if (tid == 0) {
    tc::mbar_init(&mbar_load, 1);
    tc::mbar_init(&mbar_mma, 1);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kZvTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  // block kb: its FP64 columns (one bulk copy each) and its X operand tile
  auto load_block = [&](int64_t kb) {
    const int kbw = (int)((n - kb * kZvK) < kZvK ? (n - kb * kZvK) : kZvK);
    const uint32_t colbytes = (uint32_t)rows_valid * 16u;
    tc::mbar_arrive_expect_tx(&mbar_load, colbytes * (uint32_t)kbw + kZvXTile);
    for (int c = 0; c < kbw; ++c)
      tc::bulk_g2s(sA64 + c * (kZvRows * 16), A + row0 + (kb * kZvK + c) * n, colbytes, &mbar_load);
    tc::bulk_g2s(sX[kb & 1], xt + (b * nkb + kb) * (int64_t)kZvXTile, kZvXTile, &mbar_load);
  };
  if (tid == 0) load_block(0);

  // split mapping: four threads per row, eight columns each
  const int srow = tid >> 2, sq = tid & 3;
  // epilogue mapping: TMEM lane = row (warp % 4 picks the lane quadrant), warp / 4 picks
  // the two right-hand sides j0, j0 + 1 of this thread
  const int erow = (warp & 3) * 32 + lane, j0 = 2 * (warp >> 2);
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  double2 acc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  __shared__ int s_rowexp[2][kZvRows];
  bool failed = false;
  int loads_pending = 1, mma_pending = 0;

  auto epilogue = [&](int64_t kb) {
    const uint32_t base = tmem + lane_off + (uint32_t)(kb & 1) * 256u;
    // (Re A | Im A) x (Xr | Xi) for digit sums d = 0..7 and this thread's two columns
    uint32_t v[kZvDigits][8];
#pragma unroll
    for (int dd = 0; dd < kZvDigits; ++dd) {
      const uint32_t c = base + (uint32_t)(16 * dd + j0);
      tmem_ld2_nowait(c, v[dd][0], v[dd][1]);               // Re A Xr (j0, j0+1)
      tmem_ld2_nowait(c + 8u, v[dd][2], v[dd][3]);          // Re A Xi
      tmem_ld2_nowait(c + 128u, v[dd][4], v[dd][5]);        // Im A Xr
      tmem_ld2_nowait(c + 136u, v[dd][6], v[dd][7]);        // Im A Xi
    }
    tmem_wait_ld();
    const int er = s_rowexp[kb & 1][erow];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int pr[4], pi[4];
#pragma unroll
      for (int dd = 0; dd < kZvDigits; ++dd) {
        // T_d of the complex product: Re = ReA Xr - ImA Xi, Im = ReA Xi + ImA Xr (|.| < 2^22)
        const int tr = int_of_exact(v[dd][0 + h]) - int_of_exact(v[dd][6 + h]);
        const int ti = int_of_exact(v[dd][2 + h]) + int_of_exact(v[dd][4 + h]);
        if (dd & 1) { pr[dd >> 1] = pr[dd >> 1] * 128 + tr; pi[dd >> 1] = pi[dd >> 1] * 128 + ti; }
        else { pr[dd >> 1] = tr; pi[dd >> 1] = ti; }
      }
      const long long kMagic = 0x4338000000000000LL;
      constexpr double kBias = 6755399441055744.0 + 25165824.0;  // 1.5 2^52 + 1.5 2^24
      const long long hr = (long long)pr[0] * 16384 + pr[1], lr = (long long)pr[2] * 16384 + pr[3];
      const long long hi = (long long)pi[0] * 16384 + pi[1], li = (long long)pi[2] * 16384 + pi[3];
      const double xr = fma(__longlong_as_double(lr + kMagic), 0x1p-28, __longlong_as_double(hr + kMagic) - kBias);
      const double xi = fma(__longlong_as_double(li + kMagic), 0x1p-28, __longlong_as_double(hi + kMagic) - kBias);
      const double sc = pow2i(er + __ldg(xexp + (b * nkb + kb) * kZvRhs + j0 + h) - 33);
      acc[h].x = fma(xr, sc, acc[h].x);
      acc[h].y = fma(xi, sc, acc[h].y);
    }
  };

  for (int64_t kb = 0; kb < nkb; ++kb) {
    bool ok = tc::mbar_wait(&mbar_load, (uint32_t)(kb & 1), kZvWaitPolls);
    if (__syncthreads_or(!ok)) { failed = true; break; }
    --loads_pending;
    if (kb > 0) {
      ok = tc::mbar_wait(&mbar_mma, (uint32_t)((kb - 1) & 1), kZvWaitPolls);
      if (__syncthreads_or(!ok)) { failed = true; break; }
      --mma_pending;
      tc::fence_after_sync();
    }
    // cut the FP64 block into digit planes (rows past n and columns past n are zero)
    {
      const int kbw = (int)((n - kb * kZvK) < kZvK ? (n - kb * kZvK) : kZvK);
      const bool live = srow < rows_valid;
      double2 vals[8];
      int emax = 0;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int col = 8 * sq + c;
        vals[c] = (live && col < kbw) ? *reinterpret_cast<const double2*>(sA64 + col * (kZvRows * 16) + srow * 16)
                                      : make_double2(0.0, 0.0);
        emax = max(emax, max(dg::biased_exp(vals[c].x), dg::biased_exp(vals[c].y)));
      }
      emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
      emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
      uint32_t pk[2][kZvDigits][4];  // [part][digit][pairs of columns]
      dg::split8(vals, emax, pk);
      const uint32_t off = tc::kmajor_offset(srow, 8 * sq, kZvK);
#pragma unroll
      for (int part = 0; part < 2; ++part)
#pragma unroll
        for (int p = 0; p < kZvDigits; ++p)
          *reinterpret_cast<uint4*>(sAd + (part * kZvDigits + p) * kZvPlane + off) =
              make_uint4(pk[part][p][0], pk[part][p][1], pk[part][p][2], pk[part][p][3]);
      // |v| < 2^E with E = emax - 1022 (the exponent scale of this row and block)
      if (sq == 0) s_rowexp[kb & 1][srow] = dg::scale_of(emax);
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sAd), x0 = tc::smem_u32(sX[kb & 1]);
      constexpr uint32_t sbo = (kZvK / 8) * 128;
      const uint32_t tb = tmem + (uint32_t)(kb & 1) * 256u;
#pragma unroll 1
      for (int p = 0; p < kZvDigits; ++p) {
        const uint32_t id = tc::idesc_bf16_f32(kZvRows, 16 * (kZvDigits - p));
#pragma unroll
        for (int part = 0; part < 2; ++part) {
          const uint32_t dst = tb + (uint32_t)(128 * part + 16 * p);
          const uint32_t ap = a0 + (uint32_t)(part * kZvDigits + p) * kZvPlane;
#pragma unroll
          for (int kk = 0; kk < kZvK / 16; ++kk) {
            const uint32_t ko = (uint32_t)kk * 256;
            tc::mma_bf16(dst, tc::smem_desc(ap + ko, 128, sbo), tc::smem_desc(x0 + ko, 128, sbo), id,
                         (p == 0 && kk == 0) ? 0u : 1u);
          }
        }
      }
      tc::mma_commit(&mbar_mma);
      // the FP64 block buffer and the other X buffer are free: fetch block kb + 1
      if (kb + 1 < nkb) load_block(kb + 1);
    }
    ++mma_pending;
    if (kb + 1 < nkb) ++loads_pending;
    if (kb > 0) epilogue(kb - 1);
    tc::fence_before_sync();
  }
  if (!failed) {
    const int64_t kb = nkb - 1;
    const bool ok = tc::mbar_wait(&mbar_mma, (uint32_t)(kb & 1), kZvWaitPolls);
    if (__syncthreads_or(!ok)) failed = true;
    else {
      --mma_pending;
      tc::fence_after_sync();
      epilogue(kb);
    }
  }
  if (failed) {
    if (tid == 0) atomicExch(timeout_flag, 1);
    if (mma_pending > 0) {
      tc::mbar_wait(&mbar_mma, 0, kZvWaitPolls);
      tc::mbar_wait(&mbar_mma, 1, kZvWaitPolls);
    }
    if (loads_pending > 0) {
      tc::mbar_wait(&mbar_load, 0, kZvWaitPolls);
      tc::mbar_wait(&mbar_load, 1, kZvWaitPolls);
    }
  } else {
    const int64_t i = row0 + erow;
    if (erow < rows_valid) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = j0 + h;
        if (j >= g) continue;
        const int64_t o = b * xstride + i + (int64_t)(r0 + j) * n;
        double2 y = acc[h];
        if (subtract) { const double2 bb = Ball[o]; y = make_double2(bb.x - y.x, bb.y - y.y); }
        Yall[o] = y;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kZvTmemCols);
}

}  // namespace

size_t tc_zgemv_workspace_bytes(int64_t n, int64_t batch) {
  const int64_t nkb = (n + kZvK - 1) / kZvK;
  return (size_t)batch * (size_t)nkb * ((size_t)kZvXTile + kZvRhs * sizeof(int)) + 256;
}

void tc_zgemv(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
              int64_t nrhs, int64_t xstride, double2* Y, const double2* B, void* ws, int* timeout_flag) {
  const int64_t n = d.n;
  if (n <= 0 || nrhs <= 0 || d.batch <= 0) return;
  const int64_t nkb = (n + kZvK - 1) / kZvK;
  unsigned char* xt = static_cast<unsigned char*>(ws);
  int* xexp = reinterpret_cast<int*>(xt + d.batch * nkb * (int64_t)kZvXTile);
  cudaFuncSetAttribute(zgemv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZvSmem);
  for (int64_t r0 = 0; r0 < nrhs; r0 += kZvRhs) {
    const int g = (int)((nrhs - r0) < kZvRhs ? (nrhs - r0) : kZvRhs);
    MH_LAUNCH(lc, st, "zgemv_tc_split",
              zgemv_xsplit_kernel<<<dim3((unsigned)nkb, (unsigned)d.batch), 256, 0, st>>>(d, X, xstride, (int)r0, g,
                                                                                           nkb, xt, xexp));
    MH_LAUNCH(lc, st, "zgemv_tc",
              zgemv_tc_kernel<<<dim3((unsigned)((n + kZvRows - 1) / kZvRows), (unsigned)d.batch), kZvThreads, kZvSmem,
                                st>>>(d, A, B, Y, xstride, (int)r0, g, nkb, xt, xexp, B != nullptr ? 1 : 0,
                                      timeout_flag));
  }
}

}  // namespace mh
