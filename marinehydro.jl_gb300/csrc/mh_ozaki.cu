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
// scale product, the size of FP64 rounding.  T_0..T_3 are combined exactly in 64-bit integers,
// T_4..T_6 (which only need to be right to a fraction of the last unit) in FP32, and the sum
// is rounded to a 53-bit integer within 0.76 of the exact value, scaled by the power of two
// and subtracted from A22 -- one FP64 operation per real element instead of the 128 FMAs of
// the FP64 update.  (Eight base-128 digits need 36 digit products for the same 55 bits;
// seven base-256 digits need 28.)
//
// Kernels per panel step (all batched over the matrices of the sweep):
//   ozaki_split (one launch, both halves) -- rows: L21 -> digit tiles A[row tile][digit][re/im]
//     (128 x 32 BF16 each, in the canonical no-swizzle K-major layout) and the row
//     exponents; columns: U12 -> digit tiles B[col tile][re/im][digit] (32 x 32 BF16) and the
//     column exponents; the seven digit tiles of one part are consecutive, so digits
//     q .. 6 form one (32 (7 - q)) x 32 operand;
//   ozaki_gemm: a persistent kernel, one CTA of 512 threads per SM walking a slice of the
//     128 x 32 output tiles: the 14 A digit tiles of the current row tile (112 KB) and one B
//     tile (28 KB) arrive in shared memory by TMA bulk copies.  Per column tile and digit p
//     of L21, one tcgen05.mma with N = 32 (7 - p)
//     multiplies X_p by the stacked Y_0 .. Y_{6-p} and accumulates X_p Y_q into the TMEM
//     columns of T_{p+q} (Re: 32 d, Im: 224 + 32 d), so 56 MMAs (7 digits x 2 K-steps x 4
//     real products) cover the 28 digit pairs.  (16-column tiles, whose two accumulator sets
//     fit TMEM twice, measured 12 % slower: they read every A tile twice as often.)  The
//     epilogue converts the exact integers T0..T3 with magic-number additions (no
//     integer-to-FP64 conversion instructions) and combines them in 32/64-bit integers, adds
//     T4 + T5 2^-8 + T6 2^-16 formed in FP32, builds the scaled double of the 53-bit integer
//     with integer operations and applies it with one FP64 subtraction per real entry.  The
//     subtractions of one column tile run while the tensor cores compute the next one (the
//     accumulators of a tile fill 448 of the 512 TMEM columns, so the TMEM reads of a tile
//     come first); four warps per SM sub-partition keep its FP64 pipe busy, and each tile of
//     A22 is prefetched into L2 one tile ahead.
//   The triangular solve of a panel step (U12 = L11^-1 A12) runs as the same product with
//   ozaki_trsm_prep cutting the operands and ozaki_gemm<true> assigning the products.
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

constexpr int kOzThreads = 512; // four threads per output row: warps w, w + 4, w + 8, w + 12 share
                                // the TMEM lanes 32 (w % 4) .. and take a quarter of the columns each

// The eight MMAs of digit p of L21 for one column tile (one thread): X_p (A tiles at a0)
// times the stacked Y_0 .. Y_{6-p} (B tiles at b0) into the TMEM columns of T_p .. T_6, Re and
// Im; K = 16 steps past the panel width kb are skipped (their digits are zero)
__device__ __forceinline__ void ozaki_issue_digit(uint32_t tmem, uint32_t a0, uint32_t b0, int p, int kb) {
  constexpr uint32_t sbo = (kOzK / 8) * 128;  // 8-row core groups are K * 16 bytes apart
  const uint32_t bre = b0, bim = b0 + (uint32_t)kOzDigits * kOzBTile;  // Y_0 of each part
  const int nn = kOzCols * (kOzDigits - p);
  const uint32_t id = tc::idesc_bf16_f32(kOzRows, nn), id_neg = tc::idesc_bf16_f32_nega(kOzRows, nn);
  const uint32_t t_re = tmem + (uint32_t)(kOzCols * p), t_im = t_re + (uint32_t)(kOzCols * kOzDigits);
  const uint32_t ar = a0 + (uint32_t)(2 * p) * kOzATile, ai = ar + kOzATile;
  const int nks = (kb + 15) / 16;
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

constexpr int kOzSmem = kOzABytes + kOzBBytes;  // 140 KB: the A digit tiles and one B tile

// x + 1.5 2^23 holds an integer-valued x with |x| <= 2^22 in its low mantissa bits exactly
__device__ __forceinline__ int exact_int22(float x) { return __float_as_int(x + 12582912.0f) - 0x4B400000; }
// the integer nearest x, |x| < 2^23: 1.5 2^24 rounds x to an even integer 2 h exactly, and the
// remainder x - 2 h (exact, |.| <= 1) is rounded by 1.5 2^23
__device__ __forceinline__ int rint23(float x) {
  const float y = x + 25165824.0f;
  const float rr = x - (y - 25165824.0f);
  return 2 * (__float_as_int(y) - 0x4BC00000) + exact_int22(rr);
}

// The products of 8 columns of this thread's lane (TMEM columns c0 ..) as integers:
// v = (T0 2^24 + T1 2^16 + T2 2^8 + T3) 2^8 + rint(T4 + T5 2^-8 + T6 2^-16).  T0..T3 (|T_d| <=
// (d + 1) 2^20 <= 2^22) convert exactly and combine in 32/64-bit integers; the low sum is formed
// in FP32 (two FMAs, rounding error below 0.26), so v is within 0.76 of the exact
// sum_d T_d 2^(32 - 8 d) (|v| < 2^52.1).  Four TMEM waits per 8 columns.
__device__ __forceinline__ void ozaki_levels_to_int(uint32_t trow, int c0, long long* vr, long long* vi) {
  constexpr uint32_t im = kOzDigits * kOzCols;  // the Im accumulators follow the Re ones
  auto col = [&](int d, bool imag) { return trow + (imag ? im : 0u) + (uint32_t)(d * kOzCols + c0); };
  int hr[8], hi[8], gr[8], gi[8];
  float f[4][8];
  {
    const uint32_t a[4] = {col(0, false), col(0, true), col(1, false), col(1, true)};
    tc::tmem_ld8x4(a, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      hr[q] = exact_int22(f[0][q]) * 256 + exact_int22(f[2][q]);
      hi[q] = exact_int22(f[1][q]) * 256 + exact_int22(f[3][q]);
    }
  }
  {
    const uint32_t a[4] = {col(2, false), col(2, true), col(3, false), col(3, true)};
    tc::tmem_ld8x4(a, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      gr[q] = exact_int22(f[0][q]) * 256 + exact_int22(f[2][q]);
      gi[q] = exact_int22(f[1][q]) * 256 + exact_int22(f[3][q]);
    }
  }
  float lr[8], li[8];
  {
    const uint32_t a[4] = {col(5, false), col(5, true), col(6, false), col(6, true)};
    tc::tmem_ld8x4(a, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      lr[q] = fmaf(f[2][q], 0.00390625f, f[0][q]);  // T5 + T6 2^-8
      li[q] = fmaf(f[3][q], 0.00390625f, f[1][q]);
    }
  }
  {
    float g[2][8];
    const uint32_t a[2] = {col(4, false), col(4, true)};
    tc::tmem_ld8x2(a, g);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int lor = rint23(fmaf(lr[q], 0.00390625f, g[0][q]));  // T4 + (T5 + T6 2^-8) 2^-8
      const int loi = rint23(fmaf(li[q], 0.00390625f, g[1][q]));
      vr[q] = ((long long)hr[q] * 65536 + gr[q]) * 256 + lor;
      vi[q] = ((long long)hi[q] * 65536 + gi[q]) * 256 + loi;
    }
  }
}

// A persistent kernel: one CTA of 512 threads per SM walks a contiguous slice of the launch's
// live tiles (matrix, 128-row tile, 32-column tile; column tiles innermost).  Four threads per
// output row (warps w, w + 4, w + 8, w + 12 share the TMEM lanes 32 (w % 4) .. and take 8 of
// the 32 columns each), so that four warps per SM sub-partition keep its FP64 pipe busy.
// Shared memory: the 14 A digit tiles of the current row tile (112 KB) and one B tile
// (28 KB).  Per tile t, with t' the CTA's next tile:
//   1. wait for tile t's products; thread 0 starts the bulk copies of t''s B tile and, when
//      t' starts another row tile, of its A tiles (both buffers are free once t's MMAs are
//      done); every thread prefetches its entries of t''s A22 tile into L2;
//   2. every thread reads its lane's accumulators for its 8 columns and forms the integers v;
//   3. once every thread has read the TMEM (and t''s tiles have arrived), thread 0 issues t''s
//      56 MMAs, while the other threads subtract t's products from their A22 entries (doubles
//      built from v by integer operations, one FP64 subtraction per real entry) and store
//      them; warps 4, 8 and 12 also take warp 0's entries (handed over in shared memory).
//      The FP64 work of one tile runs under the tensor work of the next, and a new row
//      tile's A digits load under the epilogue.
// TRSM: the tiles are (matrix, 128-row tile) with one column tile, whose products are
// assigned into U12.
template <bool TRSM>
__global__ void __launch_bounds__(kOzThreads, 1) ozaki_gemm_kernel(BatchDesc d, double2* __restrict__ A, int64_t k, int kb0,
                                                              int64_t rest, int64_t nrt, int64_t nct,
                                                              const unsigned char* __restrict__ digA,
                                                              const unsigned char* __restrict__ digB,
                                                              const int* __restrict__ rowexp,
                                                              const int* __restrict__ colexp,
                                                              int* __restrict__ timeout_flag) {
  extern __shared__ __align__(1024) unsigned char osm[];
  __shared__ __align__(8) uint64_t mbar_a, mbar_b, mbar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int sce[kOzCols];  // column exponents of the current tile
  __shared__ longlong2 shand[8 * 32];  // warp 0's integers, handed to warps 4, 8 and 12
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // The launch's tiles are enumerated matrix by matrix (only those inside each matrix's
  // trailing block: a grouped batch's matrices have orders of their own), row tiles by
  // column tiles within a matrix, and cut into gridDim.x equal contiguous slices.
  struct Tile {  // (32-bit fields: matrix orders and tile counts stay far below 2^31)
    int b, rt, ct, n, rest_b, rest_cb, kb, nr, nc;
  };
  // the geometry of matrix T.b at this panel step; false when its trailing block is empty
  auto fill = [&](Tile& T) -> bool {
    const int64_t nb = d.order(T.b);
    T.n = (int)nb;
    T.nr = T.nc = 0;
    if (TRSM ? k + kNB_oz > nb : k + kb0 >= nb) return false;
    T.kb = (int)((k + kb0 < nb) ? kb0 : nb - k);  // 32, or 16 inside a two-level panel
    // output rows: trailing rows of A22, or (TRSM) the columns of A12; output columns: the
    // columns of A22 right of the panel (appended right-hand sides included, at most the
    // launch's `rest`), or the 32 rows of U12
    T.rest_b = (int)(TRSM ? nb + d.extra - k - T.kb : nb - k - T.kb);
    T.rest_cb = (int)(TRSM ? T.kb : min(rest, nb + d.extra - k - T.kb));
    if (T.rest_b <= 0 || T.rest_cb <= 0) return false;
    T.nr = (T.rest_b + kOzRows - 1) / kOzRows;
    T.nc = (T.rest_cb + kOzCols - 1) / kOzCols;
    return true;
  };
  // the tile after T in the enumeration (no divisions)
  auto advance = [&](Tile& T) {
    if (++T.ct < T.nc) return;
    T.ct = 0;
    if (++T.rt < T.nr) return;
    T.rt = 0;
    do {
      ++T.b;
    } while (T.b < d.batch && !fill(T));
  };
  // warp 0 counts every matrix's tiles and locates the first tile of this CTA's slice
  __shared__ int s_slice[3];
  if (warp == 0) {
    long long tot = 0;
    for (int64_t b0 = 0; b0 < d.batch; b0 += 32) {
      Tile T;
      T.b = (int)(b0 + lane);
      int cnt = (b0 + lane < d.batch && fill(T)) ? T.nr * T.nc : 0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
      tot += cnt;
    }
    const long long l0 = blockIdx.x * tot / gridDim.x, l1 = (blockIdx.x + 1) * tot / gridDim.x;
    long long base = 0;
    int fb = -1, fj = 0;
    for (int64_t b0 = 0; b0 < d.batch && fb < 0 && l1 > l0; b0 += 32) {
      Tile T;
      T.b = (int)(b0 + lane);
      const int cnt = (b0 + lane < d.batch && fill(T)) ? T.nr * T.nc : 0;
      int incl = cnt;  // inclusive prefix sum over the lanes
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
      }
      const int chunk = __shfl_sync(0xffffffffu, incl, 31);
      if (base + chunk > l0) {  // matrix b0 + first holds tile l0: its tiles are [base + incl - cnt, base + incl)
        const unsigned hit = __ballot_sync(0xffffffffu, cnt > 0 && base + incl > l0);
        const int first = __ffs(hit) - 1;
        fb = (int)b0 + first;
        fj = (int)(l0 - base - __shfl_sync(0xffffffffu, incl - cnt, first));
      }
      base += chunk;
    }
    if (lane == 0) {
      s_slice[0] = fb;
      s_slice[1] = fj;
      s_slice[2] = (int)(l1 - l0);
    }
  }
  __syncthreads();
  int left = s_slice[2];  // tiles of the slice not yet finished
  if (left <= 0 || s_slice[0] < 0) return;  // nothing here: leave before any tensor-memory allocation
  Tile cur;
  cur.b = s_slice[0];
  fill(cur);
  cur.rt = s_slice[1] / cur.nc;
  cur.ct = s_slice[1] - cur.rt * cur.nc;
  unsigned char* As = osm;
  unsigned char* Bs = osm + kOzABytes;
  auto srcA = [&](const Tile& T) { return digA + ((int64_t)T.b * nrt + T.rt) * (int64_t)kOzABytes; };
  auto srcB = [&](const Tile& T) { return digB + ((int64_t)T.b * nct + T.ct) * (int64_t)kOzBBytes; };
  if (tid == 0) {
    tc::mbar_init(&mbar_a, 1);
    tc::mbar_init(&mbar_b, 1);
    tc::mbar_init(&mbar_mma, 1);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kOzTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const int lrow = tid & (kOzRows - 1), quarter = tid >> 7;  // TMEM lane (output row) and column quarter
  const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  // this thread's 8 entries of a tile of A22 into L2 (plain per-thread prefetches: a warp's 32
  // rows of one column are 512 contiguous bytes)
  auto prefetch_c = [&](const Tile& T) {
    const int rr = T.rt * kOzRows + lrow;
    if (rr >= T.rest_b) return;
    const double2* cr = A + d.offset(T.b) + (k + T.kb + rr) + (k + T.kb) * (int64_t)T.n;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int c = T.ct * kOzCols + quarter * 8 + q;
      if (c < T.rest_cb) asm volatile("prefetch.global.L2 [%0];" ::"l"(cr + (int64_t)c * T.n));
    }
  };
  // copies and products waited for, and those issued but not yet waited for (bits 1: A,
  // 2: B, 4: products); identical in every thread
  int a_wt = 0, b_wt = 0, m_wt = 0, pend = 0;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&mbar_a, kOzABytes);
    const unsigned char* sa = srcA(cur);
    for (int q = 0; q < kOzABytes; q += 16384) tc::bulk_g2s(As + q, sa + q, 16384, &mbar_a);
    tc::mbar_arrive_expect_tx(&mbar_b, kOzBBytes);
    tc::bulk_g2s(Bs, srcB(cur), kOzBBytes, &mbar_b);
  }
  if (!TRSM) prefetch_c(cur);
  pend = 3;
  bool failed = false;
  {
    bool ok = tc::mbar_wait(&mbar_a, 0u, kOzWaitPolls);
    ok = ok && tc::mbar_wait(&mbar_b, 0u, kOzWaitPolls);
    if (__syncthreads_or(!ok)) {
      failed = true;
    } else {
      a_wt = b_wt = 1;
      pend = 0;
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
#pragma unroll 1
        for (int p = 0; p < kOzDigits; ++p) ozaki_issue_digit(tmem, a0, b0, p, cur.kb);
        tc::mma_commit(&mbar_mma);
      }
      pend = 4;
    }
  }
  while (!failed) {
    bool more, new_a;
    Tile nxt = cur;
    {
      more = left > 1;
      if (more) advance(nxt);
      new_a = more && (nxt.b != cur.b || nxt.rt != cur.rt);
      bool ok = tc::mbar_wait(&mbar_mma, (uint32_t)(m_wt & 1), kOzWaitPolls);
      if (__syncthreads_or(!ok)) { failed = true; break; }
      ++m_wt;
      pend &= ~4;
      tc::fence_after_sync();
      // the B tile and the A tiles are free (this tile's products are done): bring in the next
      if (tid == 0 && more) {
        tc::mbar_arrive_expect_tx(&mbar_b, kOzBBytes);
        tc::bulk_g2s(Bs, srcB(nxt), kOzBBytes, &mbar_b);
        if (new_a) {
          tc::mbar_arrive_expect_tx(&mbar_a, kOzABytes);
          const unsigned char* sa = srcA(nxt);
          for (int q = 0; q < kOzABytes; q += 16384) tc::bulk_g2s(As + q, sa + q, 16384, &mbar_a);
        }
      }
    }
    if (more) pend |= 2;
    if (new_a) pend |= 1;
    if (!TRSM && more) prefetch_c(nxt);
    if (warp == 1) {
      const int c = cur.ct * kOzCols + lane;
      sce[lane] = c < cur.rest_cb ? colexp[(int64_t)cur.b * (d.n + d.extra) + c] : 0;
    }
    long long vr[8], vi[8];
    ozaki_levels_to_int(trow, quarter * 8, vr, vi);
    // while thread 0 issues the next products, warps 4, 8 and 12 (on warp 0's SM sub-partition)
    // subtract warp 0's entries
    const bool handoff = more && !TRSM;
    if (handoff && warp == 0) {
#pragma unroll
      for (int q = 0; q < 8; ++q) shand[q * 32 + lane] = make_longlong2(vr[q], vi[q]);
    }
    bool okw = true;
    if (more) okw = tc::mbar_wait(&mbar_b, (uint32_t)(b_wt & 1), kOzWaitPolls);
    if (new_a && okw) okw = tc::mbar_wait(&mbar_a, (uint32_t)(a_wt & 1), kOzWaitPolls);
    // every TMEM read of this tile is done before thread 0 issues the next products
    tc::fence_before_sync();
    if (__syncthreads_or(!okw)) { failed = true; break; }
    if (more) ++b_wt;
    if (new_a) ++a_wt;
    pend &= ~3;
    tc::fence_after_sync();
    if (more && tid == 0) {
      const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
#pragma unroll 1
      for (int p = 0; p < kOzDigits; ++p) ozaki_issue_digit(tmem, a0, b0, p, nxt.kb);
      tc::mma_commit(&mbar_mma);
    }
    if (more) pend |= 4;
    // this tile's geometry
    const int64_t n = cur.n;
    const int64_t kb = cur.kb;
    const int r = cur.rt * kOzRows + lrow;  // row of the trailing block
    const bool row_live = r < cur.rest_b;
    const int er = row_live ? rowexp[(int64_t)cur.b * (d.n + d.extra) + r] : 0;
    double2* Ab = A + d.offset(cur.b);
    double2* crow = Ab + (k + kb + r) + (k + kb) * n;  // this thread's row of A22
    double2* ucol = Ab + k + (k + kb + r) * n;         // TRSM: column k + kb + r of U12
    // v 2^(e_i + f_j - 46) as a double by integer operations, one FP64 subtraction per real entry
    if (!(handoff && warp == 0)) {
      const int cbase = cur.ct * kOzCols + quarter * 8;
      // warp 0's entries q0 .. q0 + nx - 1 (column quarter 0): three each for warps 4 and 8, two
      // for warp 12
      const bool recv = handoff && (warp & 3) == 0;
      const int q0 = 3 * (quarter - 1), nx = recv ? min(3, 8 - q0) : 0;
      double2 cv[8], xv[3];
      long long xr[3], xi[3];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const bool live = row_live && cbase + q < cur.rest_cb;
        cv[q] = (live && !TRSM) ? crow[(int64_t)(cbase + q) * n] : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (j < nx) {
          const int c = cur.ct * kOzCols + q0 + j;
          xv[j] = (row_live && c < cur.rest_cb) ? crow[(int64_t)c * n] : make_double2(0.0, 0.0);
          const longlong2 w = shand[(q0 + j) * 32 + lane];
          xr[j] = w.x;
          xi[j] = w.y;
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int c = cbase + q;
        const bool live = row_live && c < cur.rest_cb;
        const int sc = er + sce[quarter * 8 + q] - 46;
        const double sr = scaled_i64(vr[q], sc), si = scaled_i64(vi[q], sc);
        if (TRSM) {
          if (live) ucol[c] = make_double2(sr, si);
        } else {
          cv[q].x -= sr;
          cv[q].y -= si;
          if (live) crow[(int64_t)c * n] = cv[q];
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (j < nx) {
          const int c = cur.ct * kOzCols + q0 + j;
          const int sc = er + sce[q0 + j] - 46;
          xv[j].x -= scaled_i64(xr[j], sc);
          xv[j].y -= scaled_i64(xi[j], sc);
          if (row_live && c < cur.rest_cb) crow[(int64_t)c * n] = xv[j];
        }
      }
    }
    if (!more) break;
    --left;
    cur = nxt;
  }
  if (failed) {
    // reported by the host as a timeout; drain the products and copies in flight (bounded)
    // before the tensor memory and shared memory are released
    if (tid == 0) atomicExch(timeout_flag, 1);
    if (pend & 4) tc::mbar_wait(&mbar_mma, (uint32_t)(m_wt & 1), kOzWaitPolls);
    if (pend & 1) tc::mbar_wait(&mbar_a, (uint32_t)(a_wt & 1), kOzWaitPolls);
    if (pend & 2) tc::mbar_wait(&mbar_b, (uint32_t)(b_wt & 1), kOzWaitPolls);
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

// the persistent GEMM kernel's grid: one CTA per SM (at most one per tile)
template <bool TRSM>
static unsigned oz_grid(int64_t ntiles) {
  static const int sms = [] {
    int dev = 0, v = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v;
  }();
  cudaFuncSetAttribute(ozaki_gemm_kernel<TRSM>, cudaFuncAttributeMaxDynamicSharedMemorySize, kOzSmem);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ntiles, sms));
}

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
  MH_LAUNCH(lc, st, "lu_gemm_ozaki",
            ozaki_gemm_kernel<false><<<oz_grid<false>(d.batch * nrt * nct), kOzThreads, kOzSmem, st>>>(
                d, A, k, kb, rest, nrt, nct, digA, digB, rowexp, colexp, timeout_flag));
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
  MH_LAUNCH(lc, st, "lu_trsm_ozaki",
            ozaki_gemm_kernel<true><<<oz_grid<true>(d.batch * nrt), kOzThreads, kOzSmem, st>>>(
                d, A, k, kb, rest, nrt, nct, digA, digB, rowexp, colexp, timeout_flag));
}

}  // namespace mh
