// mh_ozaki.cu -- the FP64 complex LU trailing update on the BF16 tensor cores (Ozaki splitting).
//
// The blocked LU's update A22 -= L21 U12 (K = 32 complex columns per panel step) is the
// dominant FP64 work of the plain path, and GB300's FP64 rate is ~1/1500 of its BF16 tensor
// rate.  Each row i of L21 is scaled by 2^-e_i (e_i: the exponent of the row's largest
// |re|, |im|) and each column j of U12 by 2^-f_j; a scaled value is rounded to a 55-bit
// fixed-point integer (54 significant bits for the row's largest entry, more than FP64's 53)
// and cut into seven balanced base-256 digits, each in [-128, 128] and exact in BF16:
//     x = 2^(e - 7) sum_p x_p 2^(-8 p),   p = 0 (most significant) .. 6.
// Then L21 U12 = 2^(e_i + f_j - 14) sum_d 2^(-8 d) T_d with T_d = sum_{p+q=d} X_p Y_q (complex),
// and every T_d is an integer of magnitude at most (d + 1) 2^20 < 2^23, so the tensor cores
// accumulate it exactly in FP32 (K = 32, d + 1 <= 7 digit pairs, 2 real products per
// complex term).  Terms with p + q > 6 are dropped: they are below 2^-55 of the row/column
// scale product, the size of FP64 rounding.  The T_d are combined exactly in 64-bit integers
// (d = 0..3 and 4..6 separately), rounded once to a 53-bit integer, scaled by the power of
// two and subtracted from A22 -- one FP64 operation per real element instead of the 128 FMAs
// of the FP64 update.  (Eight base-128 digits need 36 digit products for the same 55 bits;
// seven base-256 digits need 28.)
//
// Kernels per panel step (all batched over the matrices of the sweep):
//   ozaki_split (one launch, both halves) -- rows: L21 -> digit tiles A[row tile][digit][re/im]
//     (128 x 32 BF16 each, in the canonical no-swizzle K-major layout) and the row
//     exponents; columns: U12 -> digit tiles B[col tile][re/im][digit] (32 x 32 BF16) and the
//     column exponents; the seven digit tiles of one part are consecutive, so digits
//     q .. 6 form one (32 (7 - q)) x 32 operand;
//   ozaki_gemm: one CTA per 128-row tile and group of four 32-column tiles: the 14 A digit
//     tiles (112 KB) and double-buffered B tiles (2 x 28 KB) arrive in shared memory by TMA
//     bulk copies.  Per column tile and digit p of L21, one tcgen05.mma with N = 32 (7 - p)
//     multiplies X_p by the stacked Y_0 .. Y_{6-p} and accumulates X_p Y_q into the TMEM
//     columns of T_{p+q} (Re: 32 d, Im: 224 + 32 d), so 56 MMAs (7 digits x 2 K-steps x 4
//     real products) cover the 28 digit pairs.  (16-column tiles, whose two accumulator sets
//     fit TMEM twice so that the products overlap the epilogue, measured 12 % slower: they
//     read every A tile twice as often.)  The epilogue converts the exact integers with
//     magic-number additions (no integer-to-FP64 conversion instructions), combines them in
//     32/64-bit integers, rounds hi + lo 2^-24 to one 53-bit integer, builds its scaled double
//     with integer operations and applies it with one FP64 subtraction per real entry; C is
//     prefetched into registers while the MMAs run.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "mh_digits.cuh"
#include "mh_internal.cuh"
#include "mh_tc.cuh"

namespace mh {

namespace {

constexpr int kOzDigits = 7;       // balanced base-256 digits (mh_digits.cuh, digits7)
constexpr int kNB_oz = 32;          // the LU's panel width
constexpr int kOzK = 32;            // panel width (the LU's kNB)
constexpr int kOzRows = 128;        // output rows per CTA (MMA M)
constexpr int kOzCols = 32;         // output columns per CTA (MMA N)
constexpr int kOzATile = kOzRows * kOzK * 2;    // bytes of one A digit tile (128 x 32 BF16)
constexpr int kOzBTile = kOzCols * kOzK * 2;    // bytes of one B digit tile (32 x 32 BF16)
constexpr int kOzABytes = kOzDigits * 2 * kOzATile;   // 112 KB per row tile
constexpr int kOzBBytes = kOzDigits * 2 * kOzBTile;   // 28 KB per column tile
constexpr uint32_t kOzTmemCols = 512;
constexpr uint32_t kOzWaitPolls = 1u << 26;

// L21 of matrix b at panel step k: rows k+kb .. n-1, columns k .. k+kb-1 (kb <= 32).  Four
// threads per row, eight columns each: the row's largest exponent by shuffles, then its
// digits with integer arithmetic (mh_digits.cuh), one 16-byte store per digit plane.
__device__ __forceinline__ void ozaki_split_rows(int64_t bx, const BatchDesc& d, const double2* __restrict__ A, int64_t k,
                                                               int kb, int64_t rest, int64_t nrt,
                                                               unsigned char* __restrict__ digA,
                                                               int* __restrict__ rowexp) {
  const int64_t t = bx * (int64_t)blockDim.x + threadIdx.x;
  const int64_t r = t >> 2;  // padded row of the trailing block
  const int kq = (int)(t & 3);
  const int64_t b = blockIdx.y;
  if (r >= nrt * kOzRows) return;  // whole groups of four leave together
  // a grouped batch: this matrix's order, panel width and trailing size (the launch's `rest`
  // stays the stride of the exponent arrays); kb: the launch's panel width (32, or 16 inside a
  // two-level panel)
  const int64_t n = d.order(b);
  kb = (int)((k + kb < n) ? kb : n - k);
  if (k + kb >= n) return;
  const int64_t rest_b = n - k - kb;
  const double2* Ab = A + d.offset(b);
  const bool live = r < rest_b;
  double2 v[8];
  int emax = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int kk = 8 * kq + c;
    v[c] = (live && kk < kb) ? Ab[(k + kb + r) + (k + kk) * n] : make_double2(0.0, 0.0);
    emax = max(emax, max(dg::biased_exp(v[c].x), dg::biased_exp(v[c].y)));
  }
  emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
  emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
  if (live && kq == 0) rowexp[b * (d.n + d.extra) + r] = dg::scale_of(emax);
  uint32_t pk[2][dg::kDigits7][4];
  dg::split7(v, emax, pk);
  unsigned char* tiles = digA + ((b * nrt + r / kOzRows) * kOzDigits * 2) * (int64_t)kOzATile;
  const uint32_t off = tc::kmajor_offset((int)(r % kOzRows), 8 * kq, kOzK);
#pragma unroll
  for (int p = 0; p < kOzDigits; ++p) {
    *reinterpret_cast<uint4*>(tiles + (2 * p) * kOzATile + off) = make_uint4(pk[0][p][0], pk[0][p][1], pk[0][p][2], pk[0][p][3]);
    *reinterpret_cast<uint4*>(tiles + (2 * p + 1) * kOzATile + off) = make_uint4(pk[1][p][0], pk[1][p][1], pk[1][p][2], pk[1][p][3]);
  }
}

// U12 of matrix b at panel step k: rows k .. k+kb-1, columns k+kb .. n-1; four threads per
// column, eight rows each
__device__ __forceinline__ void ozaki_split_cols(int64_t bx, const BatchDesc& d, const double2* __restrict__ A, int64_t k,
                                                               int kb, int64_t rest, int64_t nct,
                                                               unsigned char* __restrict__ digB,
                                                               int* __restrict__ colexp) {
  const int64_t t = bx * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = t >> 2;  // padded column of the trailing block
  const int kq = (int)(t & 3);
  const int64_t b = blockIdx.y;
  if (c >= nct * kOzCols) return;
  const int64_t n = d.order(b);
  kb = (int)((k + kb < n) ? kb : n - k);
  if (k + kb >= n) return;
  // columns of U12 (appended right-hand sides included), at most the launch's `rest` (which is
  // the column limit of the update inside a two-level panel)
  const int64_t rest_b = min(rest, n + d.extra - k - kb);
  const double2* Ab = A + d.offset(b);
  const bool live = c < rest_b;
  double2 v[8];
  int emax = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int kk = 8 * kq + q;
    v[q] = (live && kk < kb) ? Ab[(k + kk) + (k + kb + c) * n] : make_double2(0.0, 0.0);
    emax = max(emax, max(dg::biased_exp(v[q].x), dg::biased_exp(v[q].y)));
  }
  emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
  emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
  if (live && kq == 0) colexp[b * (d.n + d.extra) + c] = dg::scale_of(emax);
  uint32_t pk[2][dg::kDigits7][4];
  dg::split7(v, emax, pk);
  unsigned char* tiles = digB + ((b * nct + c / kOzCols) * kOzDigits * 2) * (int64_t)kOzBTile;
  const uint32_t off = tc::kmajor_offset((int)(c % kOzCols), 8 * kq, kOzK);
#pragma unroll
  for (int p = 0; p < kOzDigits; ++p) {
    *reinterpret_cast<uint4*>(tiles + p * kOzBTile + off) = make_uint4(pk[0][p][0], pk[0][p][1], pk[0][p][2], pk[0][p][3]);
    *reinterpret_cast<uint4*>(tiles + (kOzDigits + p) * kOzBTile + off) = make_uint4(pk[1][p][0], pk[1][p][1], pk[1][p][2], pk[1][p][3]);
  }
}

// Both splits of a panel step in one launch: CTAs [0, row_ctas) cut L21, the rest U12.
__global__ void __launch_bounds__(256) ozaki_split_kernel(BatchDesc d, const double2* __restrict__ A, int64_t k, int kb,
                                                          int64_t rest, int64_t nrt, int64_t nct, int64_t row_ctas,
                                                          unsigned char* __restrict__ digA,
                                                          unsigned char* __restrict__ digB, int* __restrict__ rowexp,
                                                          int* __restrict__ colexp) {
  if ((int64_t)blockIdx.x < row_ctas) ozaki_split_rows(blockIdx.x, d, A, k, kb, rest, nrt, digA, rowexp);
  else ozaki_split_cols(blockIdx.x - row_ctas, d, A, k, kb, rest, nct, digB, colexp);
}

// ---- U12 = L11^-1 A12 on the tensor cores -------------------------------------------------
// The triangular solve of a panel step is the product U12^T = A12^T (L11^-1)^T: rows = the
// columns of A12 (the A operand, 128-row tiles, K = the panel's 32 rows), columns = the 32
// rows of U12 (one B tile).  ozaki_trsm_prep_kernel: CTAs [0, row_ctas) cut the columns of
// A12 into A digit tiles (their 32 entries are contiguous); the last CTA of each matrix
// inverts the unit lower triangular L11 in FP64 (column-oriented forward substitution of
// L X = I over all its threads) and cuts the columns of (L11^-1)^T into the B tile.
// ozaki_gemm_kernel<true> then writes the products into U12.  The inverse of a unit lower
// triangular matrix whose multipliers are bounded by partial pivoting is well conditioned
// in practice; the error of U12 is of the order of the substitution's (Higham, Accuracy and
// Stability of Numerical Algorithms, 2nd ed., sec. 14.2).
__global__ void __launch_bounds__(256) ozaki_trsm_prep_kernel(BatchDesc d, const double2* __restrict__ A, int64_t k,
                                                              int64_t rest, int64_t nrt, int64_t row_ctas,
                                                              unsigned char* __restrict__ digA,
                                                              unsigned char* __restrict__ digB, int* __restrict__ rowexp,
                                                              int* __restrict__ colexp) {
  const int64_t b = blockIdx.y;
  const int64_t n = d.order(b);
  if (k + kNB_oz > n) return;  // no full panel at this step
  const int kb = kNB_oz;
  const int64_t rest_b = n + d.extra - k - kb;  // columns of A12 (appended right-hand sides included)
  if (rest_b <= 0) return;
  const double2* Ab = A + d.offset(b);
  if ((int64_t)blockIdx.x < row_ctas) {
    // column c of A12 (rows k .. k+31) as row c of the A operand; four threads per column
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t c = t >> 2;
    const int kq = (int)(t & 3);
    if (c >= nrt * kOzRows) return;  // whole groups of four leave together
    const bool live = c < rest_b;
    double2 v[8];
    int emax = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = live ? Ab[(k + 8 * kq + q) + (k + kb + c) * n] : make_double2(0.0, 0.0);
      emax = max(emax, max(dg::biased_exp(v[q].x), dg::biased_exp(v[q].y)));
    }
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
    if (live && kq == 0) rowexp[b * (d.n + d.extra) + c] = dg::scale_of(emax);
    uint32_t pk[2][dg::kDigits7][4];
    dg::split7(v, emax, pk);
    unsigned char* tiles = digA + ((b * nrt + c / kOzRows) * kOzDigits * 2) * (int64_t)kOzATile;
    const uint32_t off = tc::kmajor_offset((int)(c % kOzRows), 8 * kq, kOzK);
#pragma unroll
    for (int p = 0; p < kOzDigits; ++p) {
      *reinterpret_cast<uint4*>(tiles + (2 * p) * kOzATile + off) = make_uint4(pk[0][p][0], pk[0][p][1], pk[0][p][2], pk[0][p][3]);
      *reinterpret_cast<uint4*>(tiles + (2 * p + 1) * kOzATile + off) = make_uint4(pk[1][p][0], pk[1][p][1], pk[1][p][2], pk[1][p][3]);
    }
    return;
  }
  // L11 and its inverse X in shared memory.  L X = I column-oriented (right-looking): once row
  // r of X is final, rows s > r take -L[s][r] X[r][c] for c <= r -- (31 - r)(r + 1) entries per
  // step spread over all threads (GB300's FP64 rate per SM sub-partition is a quarter of
  // the SM's, so the work has to reach every warp scheduler)
  __shared__ double2 sL[kNB_oz][kNB_oz + 1];
  __shared__ double2 sX[kNB_oz][kNB_oz + 1];
  for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
    const int r = idx % kb, q = idx / kb;
    sL[r][q] = Ab[(k + r) + (k + q) * n];
    sX[r][q] = make_double2(r == q ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int r = 0; r < kb - 1; ++r) {
    const int w = r + 1, ne = (kb - 1 - r) * w;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const int srow = r + 1 + e / w, c = e % w;
      const double2 l = sL[srow][r], x = sX[r][c];
      double2 t = sX[srow][c];
      t.x = fma(-l.x, x.x, fma(l.y, x.y, t.x));
      t.y = fma(-l.x, x.y, fma(-l.y, x.x, t.y));
      sX[srow][c] = t;
    }
    __syncthreads();
  }
  // B tile: column j of (L11^-1)^T is row j of X, K index q; four threads per column
  if (threadIdx.x < 4 * kNB_oz) {
    const int j = threadIdx.x >> 2, kq = threadIdx.x & 3;
    double2 v[8];
    int emax = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = sX[j][8 * kq + q];
      emax = max(emax, max(dg::biased_exp(v[q].x), dg::biased_exp(v[q].y)));
    }
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
    if (kq == 0) colexp[b * (d.n + d.extra) + j] = dg::scale_of(emax);
    uint32_t pk[2][dg::kDigits7][4];
    dg::split7(v, emax, pk);
    unsigned char* tiles = digB + (b * kOzDigits * 2) * (int64_t)kOzBTile;  // one column tile per matrix
    const uint32_t off = tc::kmajor_offset(j, 8 * kq, kOzK);
#pragma unroll
    for (int p = 0; p < kOzDigits; ++p) {
      *reinterpret_cast<uint4*>(tiles + p * kOzBTile + off) = make_uint4(pk[0][p][0], pk[0][p][1], pk[0][p][2], pk[0][p][3]);
      *reinterpret_cast<uint4*>(tiles + (kOzDigits + p) * kOzBTile + off) = make_uint4(pk[1][p][0], pk[1][p][1], pk[1][p][2], pk[1][p][3]);
    }
  }
}

// v 2^s as a double, exactly, for |v| < 2^53, built from the integer's bits (leading-zero
// count, shift, exponent field) without the FP64 pipe.  Results below the normal range are
// flushed to zero (they lie below 2^-1022).
__device__ __forceinline__ double scaled_i64(long long v, int s) {
  const unsigned long long sign = (unsigned long long)v & 0x8000000000000000ULL;
  unsigned long long m = (unsigned long long)(v < 0 ? -v : v);
  const int msb = 63 - __clzll(m);  // <= 52
  m <<= (52 - msb);
  const long long e = (long long)msb + s + 1023;
  const unsigned long long bits = sign | ((unsigned long long)e << 52) | (m & 0x000FFFFFFFFFFFFFULL);
  return (v == 0 || e <= 0) ? 0.0 : __longlong_as_double((long long)bits);
}

constexpr int kOzGroupMax = 8; // column tiles per CTA (the A tiles are loaded once for all of them):
                               // 1..8, from the launch-shape table (default 4)
constexpr int kOzThreads = 256; // two threads per output row: warps w and w + 4 share TMEM lanes
                                // 32 (w % 4) .. and take one half of the 32 columns each

// One CTA per (row tile, group of `group` column tiles, matrix).  The A digit tiles and the
// first B tile arrive by TMA bulk copies on one mbarrier; the B tiles are double-buffered,
// the next one prefetched while the current tile's products and epilogue run.
template <bool TRSM>
__global__ void __launch_bounds__(kOzThreads) ozaki_gemm_kernel(BatchDesc d, double2* __restrict__ A, int64_t k, int kb,
                                                              int64_t rest, int64_t nrt, int64_t nct,
                                                              const unsigned char* __restrict__ digA,
                                                              const unsigned char* __restrict__ digB,
                                                              const int* __restrict__ rowexp,
                                                              const int* __restrict__ colexp,
                                                              int* __restrict__ timeout_flag, int group) {
  extern __shared__ __align__(1024) unsigned char osm[];
  __shared__ __align__(8) uint64_t mbar_load[2];
  __shared__ __align__(8) uint64_t mbar_mma;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t rt = blockIdx.x, b = blockIdx.z;
  const int64_t ct0 = blockIdx.y * (int64_t)group;
  // a grouped batch: this matrix's panel width and trailing size; CTAs past its trailing
  // block leave before any barrier or tensor-memory allocation
  const int64_t n = d.order(b);
  if (TRSM ? k + kNB_oz > n : k + kb >= n) return;
  kb = (int)((k + kb < n) ? kb : n - k);  // the launch's panel width (32, or 16 inside a two-level panel)
  // output rows: trailing rows of A22, or (TRSM) the columns of A12; output columns: the
  // columns of A22 right of the panel (appended right-hand sides included, at most the launch's
  // `rest`), or the 32 rows of U12
  const int64_t rest_b = TRSM ? n + d.extra - k - kb : n - k - kb;
  const int64_t rest_cb = TRSM ? kb : min(rest, n + d.extra - k - kb);
  if (rt * kOzRows >= rest_b || ct0 * kOzCols >= rest_cb) return;
  // TRSM: one 32-column tile, the rows of U12 (the output is U12 transposed)
  const int64_t nct_b = TRSM ? 1 : (rest_cb + kOzCols - 1) / kOzCols;
  const int ntile = (int)((nct_b - ct0) < group ? (nct_b - ct0) : group);
  unsigned char* As = osm;
  unsigned char* Bs[2] = {osm + kOzABytes, osm + kOzABytes + kOzBBytes};
  const unsigned char* srcA = digA + (b * nrt + rt) * (int64_t)kOzABytes;
  auto srcB = [&](int64_t ct) { return digB + (b * nct + ct) * (int64_t)kOzBBytes; };
  if (tid == 0) {
    tc::mbar_init(&mbar_load[0], 1);
    tc::mbar_init(&mbar_load[1], 1);
    tc::mbar_init(&mbar_mma, 1);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kOzTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&mbar_load[0], kOzABytes + kOzBBytes);
    for (int q = 0; q < kOzABytes; q += 16384) tc::bulk_g2s(As + q, srcA + q, 16384, &mbar_load[0]);
    tc::bulk_g2s(Bs[0], srcB(ct0), kOzBBytes, &mbar_load[0]);
    if (ntile > 1) {
      tc::mbar_arrive_expect_tx(&mbar_load[1], kOzBBytes);
      tc::bulk_g2s(Bs[1], srcB(ct0 + 1), kOzBBytes, &mbar_load[1]);
    }
  }
  constexpr uint32_t sbo = (kOzK / 8) * 128;  // 8-row core groups are K * 16 bytes apart
  const int lrow = tid & (kOzRows - 1), half = tid >> 7;  // TMEM lane (output row) and column half
  const int64_t r = rt * kOzRows + lrow;       // row of the trailing block
  const bool row_live = r < rest_b;
  const int er = row_live ? rowexp[b * (d.n + d.extra) + r] : 0;
  const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  double2* Ab = A + d.offset(b);
  double2* crow = Ab + (k + kb + r) + (k + kb) * n;  // this thread's row of A22
  double2* ucol = Ab + k + (k + kb + r) * n;         // TRSM: column k + kb + r of U12
  bool failed = false;
  int outstanding_load = ntile > 1 ? 2 : 1;  // loads in flight (for the drain after a timeout)
  for (int t = 0; t < ntile; ++t) {
    const int buf = t & 1;
    const int64_t ct = ct0 + t;
    bool ok = tc::mbar_wait(&mbar_load[buf], (uint32_t)((t >> 1) & 1), kOzWaitPolls);
    if (__syncthreads_or(!ok)) { failed = true; break; }
    --outstanding_load;
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs[buf]);
      const uint32_t bre = b0, bim = b0 + (uint32_t)kOzDigits * kOzBTile;  // Y_0 of each part
#pragma unroll 1
      for (int p = 0; p < kOzDigits; ++p) {
        const int nn = kOzCols * (kOzDigits - p);  // Y_0 .. Y_{6-p} stacked along N
        const uint32_t id = tc::idesc_bf16_f32(kOzRows, nn), id_neg = tc::idesc_bf16_f32_nega(kOzRows, nn);
        const uint32_t t_re = tmem + (uint32_t)(kOzCols * p), t_im = t_re + (uint32_t)(kOzCols * kOzDigits);
        const uint32_t ar = a0 + (uint32_t)(2 * p) * kOzATile, ai = ar + kOzATile;
        const int nks = (kb + 15) / 16;  // K = 16 steps with data (the digits beyond kb are zero)
#pragma unroll
        for (int kk = 0; kk < kOzK / 16; ++kk) {
          if (kk >= nks) break;
          const uint32_t ko = (uint32_t)kk * 256;  // two K-adjacent core matrices per K = 16 step
          const uint32_t acc = (p == 0 && kk == 0) ? 0u : 1u;
          const uint64_t dar = tc::smem_desc(ar + ko, 128, sbo), dai = tc::smem_desc(ai + ko, 128, sbo);
          const uint64_t dbr = tc::smem_desc(bre + ko, 128, sbo), dbi = tc::smem_desc(bim + ko, 128, sbo);
          tc::mma_bf16(t_re, dar, dbr, id, acc);      // Re T += Xre Yre
          tc::mma_bf16(t_re, dai, dbi, id_neg, 1u);   // Re T -= Xim Yim
          tc::mma_bf16(t_im, dar, dbi, id, acc);      // Im T += Xre Yim
          tc::mma_bf16(t_im, dai, dbr, id, 1u);       // Im T += Xim Yre
        }
      }
      tc::mma_commit(&mbar_mma);
    }
    // while the products run: this thread's 16 entries of A22 and their column exponents
    double2 cv[kOzCols / 2];
    int ce[kOzCols / 2];
    const int64_t cbase = ct * kOzCols + half * (kOzCols / 2);
#pragma unroll
    for (int q = 0; q < kOzCols / 2; ++q) {
      const int64_t c = cbase + q;
      const bool live = row_live && c < rest_cb;
      cv[q] = (live && !TRSM) ? crow[c * n] : make_double2(0.0, 0.0);
      ce[q] = live ? colexp[b * (d.n + d.extra) + c] : 0;
    }
    ok = tc::mbar_wait(&mbar_mma, (uint32_t)(t & 1), kOzWaitPolls);
    if (__syncthreads_or(!ok)) { failed = true; break; }
    tc::fence_after_sync();
    // this B buffer is free again: prefetch tile t + 2 into it
    if (tid == 0 && t + 2 < ntile) {
      tc::mbar_arrive_expect_tx(&mbar_load[buf], kOzBBytes);
      tc::bulk_g2s(Bs[buf], srcB(ct + 2), kOzBBytes, &mbar_load[buf]);
    }
    if (t + 2 < ntile) ++outstanding_load;
#pragma unroll
    for (int h8 = 0; h8 < 2; ++h8) {
      const int c0 = half * (kOzCols / 2) + 8 * h8;
      // T_d as exact integers, paired: (T0 2^8 + T1, T2 2^8 + T3, T4 2^8 + T5, T6), re and im.
      // |T_d| <= (d + 1) 2^20 (d + 1 digit pairs, K = 32, two real products, |digit| <= 2^7)
      int pr[4][8], pi[4][8];
#pragma unroll
      for (int dd = 0; dd < kOzDigits; ++dd) {
        float vr[8], vi[8];
        tc::tmem_ld8(trow + (uint32_t)(dd * kOzCols + c0), vr);
        tc::tmem_ld8(trow + (uint32_t)(kOzDigits * kOzCols + dd * kOzCols + c0), vi);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          int ir, ii;
          if (dd <= 3) {
            // |T| <= 2^22: adding 1.5 2^23 puts the integer in the low mantissa bits exactly
            ir = __float_as_int(vr[q] + 12582912.0f) - 0x4B400000;
            ii = __float_as_int(vi[q] + 12582912.0f) - 0x4B400000;
          } else {
            // |T| < 2^23: 1.5 2^24 rounds T to an even integer 2 h exactly; the remainder
            // T - 2 h in {-1, 0, 1} is exact too
            const float yr = vr[q] + 25165824.0f, yi = vi[q] + 25165824.0f;
            const float rr = vr[q] - (yr - 25165824.0f), ri = vi[q] - (yi - 25165824.0f);
            ir = 2 * (__float_as_int(yr) - 0x4BC00000) + (__float_as_int(rr + 12582912.0f) - 0x4B400000);
            ii = 2 * (__float_as_int(yi) - 0x4BC00000) + (__float_as_int(ri + 12582912.0f) - 0x4B400000);
          }
          if (dd == 6) { pr[3][q] = ir; pi[3][q] = ii; }
          else if (dd & 1) { pr[dd >> 1][q] = pr[dd >> 1][q] * 256 + ir; pi[dd >> 1][q] = pi[dd >> 1][q] * 256 + ii; }
          else { pr[dd >> 1][q] = ir; pi[dd >> 1][q] = ii; }
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int qq = 8 * h8 + q;
        // hi = T0 2^24 + T1 2^16 + T2 2^8 + T3 (< 2^44.01), lo = T4 2^16 + T5 2^8 + T6 (< 2^38.4);
        // L21 U12 = 2^(e_i + f_j - 38) (hi + lo 2^-24); v = hi 2^8 + lo 2^-16, rounded to an
        // integer (|v| < 2^52.1), is scaled into a double by integer operations, so the FP64
        // pipe does one subtraction per real entry
        const long long hr = (long long)pr[0][q] * 65536 + pr[1][q], lr = (long long)pr[2][q] * 256 + pr[3][q];
        const long long hi = (long long)pi[0][q] * 65536 + pi[1][q], li = (long long)pi[2][q] * 256 + pi[3][q];
        const long long vr = hr * 256 + ((lr + (1LL << 15)) >> 16);
        const long long vi = hi * 256 + ((li + (1LL << 15)) >> 16);
        const int sc = er + ce[qq] - 46;
        if (TRSM) {
          cv[qq] = make_double2(scaled_i64(vr, sc), scaled_i64(vi, sc));
        } else {
          cv[qq].x -= scaled_i64(vr, sc);
          cv[qq].y -= scaled_i64(vi, sc);
        }
      }
    }
    if (row_live) {
#pragma unroll
      for (int q = 0; q < kOzCols / 2; ++q) {
        if (TRSM) {
          if (cbase + q < rest_cb) ucol[cbase + q] = cv[q];
        } else {
          if (cbase + q < rest_cb) crow[(cbase + q) * n] = cv[q];
        }
      }
    }
    // every TMEM read of this tile is done before the next tile's products overwrite it
    tc::fence_before_sync();
    __syncthreads();
  }
  if (failed) {
    // reported by the host as a timeout; drain the products and copies in flight (bounded)
    // before the tensor memory and shared memory are released
    if (tid == 0) atomicExch(timeout_flag, 1);
    tc::mbar_wait(&mbar_mma, 0, kOzWaitPolls);
    tc::mbar_wait(&mbar_mma, 1, kOzWaitPolls);
    if (outstanding_load > 0) {
      tc::mbar_wait(&mbar_load[0], 0, kOzWaitPolls);
      tc::mbar_wait(&mbar_load[1], 0, kOzWaitPolls);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kOzTmemCols);
}

}  // namespace

// workspace layout per batch: A digit tiles (row tiles of the widest operand), B digit tiles,
// row and column exponents (n + extra per matrix, indexed b (n + extra) + row or column)
static int64_t oz_row_tiles(const BatchDesc& d) { return (d.n + d.extra + kOzRows - 1) / kOzRows; }
static int64_t oz_col_tiles(const BatchDesc& d) { return (d.n + d.extra + kOzCols - 1) / kOzCols; }

size_t ozaki_workspace_bytes(int64_t n, int64_t batch, int64_t extra) {
  const int64_t w = n + extra;
  const int64_t t = (w + kOzRows - 1) / kOzRows, c = (w + kOzCols - 1) / kOzCols;
  return (size_t)batch * ((size_t)t * kOzABytes + (size_t)c * kOzBBytes + 2 * sizeof(int) * (size_t)w) + 1024;
}

void ozaki_trailing_update(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, double2* A, int64_t k, int kb,
                           void* ws, int* timeout_flag, int64_t cols) {
  const int64_t rows = d.n - k - kb;                           // trailing rows
  const int64_t rest = std::min(cols, d.n + d.extra - k - kb);  // trailing columns: the exponent arrays' stride
  if (rows <= 0) return;
  const int64_t nrt = (rows + kOzRows - 1) / kOzRows, nct = (rest + kOzCols - 1) / kOzCols;
  unsigned char* digA = static_cast<unsigned char*>(ws);
  unsigned char* digB = digA + d.batch * oz_row_tiles(d) * (int64_t)kOzABytes;
  int* rowexp = reinterpret_cast<int*>(digB + d.batch * oz_col_tiles(d) * (int64_t)kOzBBytes);
  int* colexp = rowexp + d.batch * (d.n + d.extra);
  const int64_t row_ctas = (nrt * kOzRows * 4 + 255) / 256, col_ctas = (nct * kOzCols * 4 + 255) / 256;
  dim3 gs((unsigned)(row_ctas + col_ctas), (unsigned)d.batch);
  MH_LAUNCH(lc, st, "lu_ozaki_split",
            ozaki_split_kernel<<<gs, 256, 0, st>>>(d, A, k, kb, rest, nrt, nct, row_ctas, digA, digB, rowexp, colexp));
  const size_t smem = kOzABytes + 2 * kOzBBytes;
  cudaFuncSetAttribute(ozaki_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int group = lc.tile(d.n).oz_group;
  group = group < 1 ? 1 : (group > kOzGroupMax ? kOzGroupMax : group);
  dim3 gg((unsigned)nrt, (unsigned)((nct + group - 1) / group), (unsigned)d.batch);
  MH_LAUNCH(lc, st, "lu_gemm_ozaki",
            ozaki_gemm_kernel<false><<<gg, kOzThreads, smem, st>>>(d, A, k, kb, rest, nrt, nct, digA, digB, rowexp,
                                                                 colexp, timeout_flag, group));
}

void ozaki_trsm(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, double2* A, int64_t k, void* ws,
                int* timeout_flag) {
  const int kb = kNB_oz;
  const int64_t rest = d.n + d.extra - k - kb;  // columns of A12 (appended right-hand sides included)
  if (rest <= 0) return;
  const int64_t nrt = (rest + kOzRows - 1) / kOzRows, nct = 1;
  unsigned char* digA = static_cast<unsigned char*>(ws);
  unsigned char* digB = digA + d.batch * oz_row_tiles(d) * (int64_t)kOzABytes;
  int* rowexp = reinterpret_cast<int*>(digB + d.batch * oz_col_tiles(d) * (int64_t)kOzBBytes);
  int* colexp = rowexp + d.batch * (d.n + d.extra);
  const int64_t row_ctas = (nrt * kOzRows * 4 + 255) / 256;
  dim3 gs((unsigned)(row_ctas + 1), (unsigned)d.batch);
  MH_LAUNCH(lc, st, "lu_trsm_ozaki_prep",
            ozaki_trsm_prep_kernel<<<gs, 256, 0, st>>>(d, A, k, rest, nrt, row_ctas, digA, digB, rowexp, colexp));
  const size_t smem = kOzABytes + 2 * kOzBBytes;
  cudaFuncSetAttribute(ozaki_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 gg((unsigned)nrt, 1u, (unsigned)d.batch);
  MH_LAUNCH(lc, st, "lu_trsm_ozaki",
            ozaki_gemm_kernel<true><<<gg, kOzThreads, smem, st>>>(d, A, k, kb, rest, nrt, nct, digA, digB, rowexp,
                                                                colexp, timeout_flag, 1));
}

}  // namespace mh
