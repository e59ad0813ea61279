// mh_lu.cu -- batched dense complex LU with partial pivoting and multi-RHS solves.
//
// Replaces linsolve / _linearsolve / gpu_linsolve (matrix_assembly.jl:396-434),
// whose CPU path is LinearSolve LUFactorization -> LAPACK zgetrf/zgetrs and whose
// CUDA path is cuSOLVER through `\` on a CuArray.  Same semantics as zgetrf:
// right-looking blocked LU, pivot = first row of maximal |re|+|im| (izamax), rows
// swapped across the whole matrix, info = index of the first exactly-zero pivot.
//
// Work split per panel step k (nb = 32 columns):
//   panel_cluster_kernel  a thread-block cluster of P CTAs per matrix: the panel's
//                  rows are split over the P CTAs and held in shared memory; pivot
//                  candidates and the pivot row travel through distributed shared
//                  memory with two cluster barriers per column, so the panel's FP64
//                  rank-1 updates run on P SMs instead of one
//   panel_kernel   the same on one CTA straight from global memory, for panels too
//                  tall for the cluster's shared memory
//   laswp_kernel   the panel's row interchanges applied to every column outside it,
//                  as one permutation of at most 64 rows (a warp per column)
//   trsm_kernel    U12 = L11^-1 A12, one thread per column, L11 in shared memory
//   gemm_kernel    A22 -= L21 U12, 64x64 tiles, 4x4 complex outputs per thread
// Templated on the real type: double (the plain FP64 path) and float (the factor
// used by mixed-precision iterative refinement).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "mh_fixpoint.cuh"
#include "mh_internal.cuh"

namespace mh {

namespace {

constexpr int kNB = 32;

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C> __device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
// c - a*b with fused multiply-adds
template <typename C> __device__ __forceinline__ C cfms(C c, C a, C b) {
  C r;
  r.x = fma(-a.x, b.x, c.x); r.x = fma(a.y, b.y, r.x);
  r.y = fma(-a.x, b.y, c.y); r.y = fma(-a.y, b.x, r.y);
  return r;
}
// c + a*b
template <typename C> __device__ __forceinline__ C cfma(C c, C a, C b) {
  C r;
  r.x = fma(a.x, b.x, c.x); r.x = fma(-a.y, b.y, r.x);
  r.y = fma(a.x, b.y, c.y); r.y = fma(a.y, b.x, r.y);
  return r;
}
template <typename C> __device__ __forceinline__ C crecip(C a) {
  // 1 / a (Smith)
  C r;
  if (fabs(a.x) >= fabs(a.y)) {
    auto q = a.y / a.x; auto den = a.x + a.y * q;
    r.x = 1 / den; r.y = -q / den;
  } else {
    auto q = a.x / a.y; auto den = a.y + a.x * q;
    r.x = q / den; r.y = -1 / den;
  }
  return r;
}
// FP64: 1/a = conj(a) f / |a f|^2 with a scaled by a power of two f (so |a f| is near 1), the
// reciprocal of the squared magnitude on the integer pipe (fx::recip): seven FP64 operations
// instead of Smith's three divisions -- this is the pivot reciprocal on the panel's
// per-column critical path, computed by one lane while the CTA waits.  Within a few ulps.
template <> __device__ __forceinline__ double2 crecip<double2>(double2 a) {
  const int ex = (int)((__double_as_longlong(a.x) >> 52) & 0x7FF);
  const int ey = (int)((__double_as_longlong(a.y) >> 52) & 0x7FF);
  const int e = ex > ey ? ex : ey;  // biased exponent of the larger part (a != 0)
  const double f = __longlong_as_double((long long)(2046 - e) << 52);  // 2^(1023 - (e - 1023)), exact
  const double sx = a.x * f, sy = a.y * f;
  const double rf = fx::recip(fma(sx, sx, sy * sy)) * f;
  return make_double2(sx * rf, -sy * rf);
}
template <typename C> __device__ __forceinline__ C cdiv(C a, C b) { return cmul(a, crecip(b)); }
template <typename C> __device__ __forceinline__ C czero() { C r; r.x = 0; r.y = 0; return r; }

__device__ __forceinline__ double2 shfl_c(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ float2 shfl_c(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// ------------------------------- panel ---------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) panel_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                    int32_t* __restrict__ ipiv_all, int32_t* __restrict__ info_all,
                                                    int64_t k) {
  using C = typename cplx_t<T>::type;
  __shared__ T wv[16];
  __shared__ int wi[16];
  __shared__ int s_piv;
  __shared__ T s_best;
  const int64_t n = d.order(blockIdx.x);
  if (k >= n) return;  // a grouped batch: this matrix is factored
  C* A = Aall + d.offset(blockIdx.x);
  int32_t* ipiv = ipiv_all + blockIdx.x * d.n;
  const int64_t kend = (k + kNB < n) ? k + kNB : n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  for (int64_t j = k; j < kend; ++j) {
    T best = -1;
    int bi = (int)n;
    for (int64_t i = j + tid; i < n; i += blockDim.x) {
      C a = A[i + j * n];
      T v = fabs(a.x) + fabs(a.y);
      if (v > best) { best = v; bi = (int)i; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      T ob = __shfl_down_sync(0xffffffffu, best, off);
      int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) { wv[warp] = best; wi[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
      best = lane < nwarp ? wv[lane] : (T)-1;
      bi = lane < nwarp ? wi[lane] : (int)n;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        T ob = __shfl_down_sync(0xffffffffu, best, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) { s_piv = bi; s_best = best; }
    }
    __syncthreads();
    const int64_t p = s_piv;
    if (tid == 0) ipiv[j] = (int32_t)p;
    if (!(s_best > 0)) {
      // exactly zero column: zgetf2 records info and moves on
      if (tid == 0 && info_all[blockIdx.x] == 0) info_all[blockIdx.x] = (int32_t)(j + 1);
      if (tid == 0) ipiv[j] = (int32_t)j;
      __syncthreads();
      continue;
    }
    if (p != j) {  // inside the panel; laswp_kernel moves the rest of the rows
      for (int64_t c = k + tid; c < kend; c += blockDim.x) {
        C t = A[j + c * n];
        A[j + c * n] = A[p + c * n];
        A[p + c * n] = t;
      }
    }
    __syncthreads();
    const C inv = crecip(A[j + j * n]);
    for (int64_t i = j + 1 + tid; i < n; i += blockDim.x) A[i + j * n] = cmul(A[i + j * n], inv);
    __syncthreads();
    const int64_t m = n - j - 1, w = kend - j - 1;
    if (w > 0) {
      for (int64_t idx = tid; idx < m * w; idx += blockDim.x) {
        int64_t r = idx % m, c = idx / m;
        int64_t i = j + 1 + r, cc = j + 1 + c;
        A[i + cc * n] = cfms(A[i + cc * n], A[i + j * n], A[j + cc * n]);
      }
    }
    __syncthreads();
  }
}

// ---------------------------- panel on a cluster -------------------------------
constexpr int kPanelThreads = 512;
// panel rows one CTA holds in shared memory (32 complex columns each, < 227 KB)
template <typename T> struct PanelRows;
template <> struct PanelRows<double> { static constexpr int value = 432; };
template <> struct PanelRows<float> { static constexpr int value = 864; };

// Pivot candidates compare |re| + |im| through the bit pattern of the (non-negative) value as
// a signed integer, which orders like the value: FP64 comparisons run on GB300's narrow FP64
// pipe, integer ones do not.  -1 stands below every candidate.
template <typename T> struct PivotKey;
template <> struct PivotKey<double> {
  using type = long long;
  __device__ static __forceinline__ long long of(double v) { return __double_as_longlong(v); }
};
template <> struct PivotKey<float> {
  using type = int;
  __device__ static __forceinline__ int of(float v) { return __float_as_int(v); }
};

// (value, row) of the larger |re| + |im|; ties go to the smaller row (izamax's first maximum)
template <typename T> __device__ __forceinline__ void argmax_merge(T& v, int& i, T ov, int oi) {
  if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
}
template <typename T> __device__ __forceinline__ void warp_argmax(T& v, int& i) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) argmax_merge(v, i, __shfl_xor_sync(0xffffffffu, v, off),
                                                       __shfl_xor_sync(0xffffffffu, i, off));
}

// split cluster barrier: arrive (releasing this thread's writes), later wait (acquiring
// every thread's writes before their arrive)
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }

// Rows k .. n-1 of the panel (m = n - k panel rows, panel row r = matrix row k + r) are
// split into chunks of `chunk` rows, chunk >= kb, so CTA 0 holds the kb diagonal rows.
// Thread t of a CTA owns its chunk's rows t, t + 512, ...: it alone writes them in shared
// memory.  Rows cross CTAs only through double-buffered publication slots, so one cluster
// barrier per column suffices.  Per column j:
//   every CTA posts its best candidate (value, row) and a copy of that row; CTA 0 also
//   posts a copy of row j;  cluster barrier
//   warp 0 of every CTA reduces the P candidates and fetches the pivot row (and, in the
//   CTA that owns the pivot row, row j) from the winners' slots through distributed
//   shared memory;  CTA barrier
//   the owners write the interchanged rows, then every thread scales its rows' entry j and
//   applies the rank-1 update to columns j+1 .. kb-1, searching column j+1 as it goes.
// Slots of parity j are rewritten at column j + 2, after every CTA has passed the barrier
// of column j + 1 and so finished its reads of column j.  (Posting column j+1 before the
// rest of the update and overlapping that update with a split barrier was measured slower:
// the extra CTA barriers cost more than the overlap saves.)  Same arithmetic, in the same
// order, as panel_kernel.
template <typename T>
__global__ void __launch_bounds__(kPanelThreads) panel_cluster_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                                     int32_t* __restrict__ ipiv_all,
                                                                     int32_t* __restrict__ info_all, int64_t k,
                                                                     int chunk_cap, int width) {
  using C = typename cplx_t<T>::type;
  using K = typename PivotKey<T>::type;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char panel_smem[];
  C* sp = reinterpret_cast<C*>(panel_smem);  // chunk x kb, column-major (leading dimension chunk)
  __shared__ C pub_row[2][kNB];               // this CTA's candidate row, by column parity
  __shared__ C pub_j[2][kNB];                 // CTA 0: row j
  __shared__ K cand_v[2];
  __shared__ int cand_i[2];
  __shared__ C urow[kNB], jrow[kNB];
  __shared__ K red_v[kPanelThreads / 32];
  __shared__ int red_i[kPanelThreads / 32];
  __shared__ int s_piv;
  __shared__ C s_inv;
  const int P = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t bmat = blockIdx.y, n = d.order(bmat);
  if (k >= n) return;  // a grouped batch: this matrix is factored (the whole cluster leaves)
  C* A = Aall + d.offset(bmat);
  const int64_t m = n - k;
  const int kb = (int)(m < width ? m : width);  // panel width: 32, or 16 for a half of a two-level panel
  // rows per CTA for this matrix: at most the launch's capacity, at least the diagonal block
  const int chunk = (int)max((int64_t)kb, min((int64_t)chunk_cap, (m + P - 1) / P));
  const int r0 = rank * chunk;  // first panel row of this CTA
  const int rows = (int)((m - r0) < chunk ? ((m - r0) > 0 ? (m - r0) : 0) : chunk);

  for (int c = 0; c < kb; ++c)
    for (int i = tid; i < rows; i += kPanelThreads) sp[c * chunk + i] = A[(k + r0 + i) + (k + c) * n];
  // candidate for column 0 (each thread reads only its own rows)
  K best = -1;
  int bi = INT_MAX;
  for (int i = tid; i < rows; i += kPanelThreads) {
    const C a = sp[i];
    argmax_merge(best, bi, PivotKey<T>::of(fabs(a.x) + fabs(a.y)), r0 + i);
  }
  for (int j = 0; j < kb; ++j) {
    const int par = j & 1;
    // post this CTA's candidate for column j with a copy of its row, and (CTA 0) row j
    warp_argmax(best, bi);
    if (lane == 0) { red_v[warp] = best; red_i[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
      best = lane < kPanelThreads / 32 ? red_v[lane] : (K)-1;
      bi = lane < kPanelThreads / 32 ? red_i[lane] : INT_MAX;
      warp_argmax(best, bi);
      if (lane == 0) { cand_v[par] = best; cand_i[par] = bi; }
      if (bi != INT_MAX && lane < kb) pub_row[par][lane] = sp[lane * chunk + (bi - r0)];
      if (rank == 0 && lane < kb) pub_j[par][lane] = sp[lane * chunk + j];
    }
    cl.sync();  // candidates and rows posted
    if (warp == 0) {
      K v = -1;
      int vi = INT_MAX;
      if (lane < P) {
        v = *cl.map_shared_rank(&cand_v[par], (unsigned)lane);
        vi = *cl.map_shared_rank(&cand_i[par], (unsigned)lane);
      }
      warp_argmax(v, vi);
      const bool zero = !(v > 0);
      const int p = zero ? j : vi;  // panel row of the pivot
      const int owner = p / chunk;
      C u = czero<C>(), rj = czero<C>();
      if (lane < kb) {
        rj = cl.map_shared_rank(&pub_j[par][0], 0u)[lane];
        u = (p == j) ? rj : cl.map_shared_rank(&pub_row[par][0], (unsigned)owner)[lane];
        urow[lane] = u;
        jrow[lane] = rj;
      }
      if (lane == j) s_inv = zero ? czero<C>() : crecip(u);
      if (lane == 0) {
        s_piv = p;
        if (rank == 0) {
          ipiv_all[bmat * d.n + k + j] = (int32_t)(k + p);
          if (zero && info_all[bmat] == 0) info_all[bmat] = (int32_t)(k + j + 1);
        }
      }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != j) {
      if (rank == 0 && tid == j)
        for (int c = 0; c < kb; ++c) sp[c * chunk + j] = urow[c];
      const int owner = p / chunk, lp = p - owner * chunk;
      if (rank == owner && tid == lp % kPanelThreads)
        for (int c = 0; c < kb; ++c) sp[c * chunk + lp] = jrow[c];
    }
    const C inv = s_inv;
    best = -1;
    bi = INT_MAX;
    for (int i = tid; i < rows; i += kPanelThreads) {
      const int pr = r0 + i;
      if (pr <= j) continue;
      const C l = cmul(sp[j * chunk + i], inv);
      sp[j * chunk + i] = l;
      for (int c = j + 1; c < kb; ++c) {
        const C v = cfms(sp[c * chunk + i], l, urow[c]);
        sp[c * chunk + i] = v;
        if (c == j + 1) argmax_merge(best, bi, PivotKey<T>::of(fabs(v.x) + fabs(v.y)), pr);
      }
    }
  }
  // other CTAs may still read this CTA's slots of the last column: wait for them
  cl.sync();
  for (int c = 0; c < kb; ++c)
    for (int i = tid; i < rows; i += kPanelThreads) A[(k + r0 + i) + (k + c) * n] = sp[c * chunk + i];
}

// The interchanges of panel step k as one permutation: final row dst = original row src for
// at most 64 (dst, src) pairs (-1: none).  Slot s < 32 is panel row s, slot 32 + q is the
// row below the diagonal block that step q chose first.  Runs on warp 0.
__device__ void panel_permutation(const int32_t* __restrict__ ipiv, int64_t k, int kb, int* s_slot,
                                  int* s_content, int* s_dst, int* s_src) {
  const int lane = threadIdx.x & 31;
  const int p = lane < kb ? (int)(ipiv[k + lane] - k) : lane;  // panel row chosen at step lane
  int first = lane;
  for (int q = 31; q >= 0; --q) {
    const int pq = __shfl_sync(0xffffffffu, p, q);
    if (q < lane && pq == p) first = q;
  }
  s_slot[lane] = p < kNB ? p : kNB + first;
  s_content[lane] = lane;
  s_content[lane + 32] = lane + 32;
  __syncwarp();
  if (lane == 0)
    for (int j = 0; j < kb; ++j) {
      const int a = j, b = s_slot[j];
      const int t = s_content[a];
      s_content[a] = s_content[b];
      s_content[b] = t;
    }
  __syncwarp();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int sl = lane + 32 * h;
    const int src = s_content[sl];
    const int q = src >= kNB ? src - kNB : 0;
    const int psrc = __shfl_sync(0xffffffffu, p, q);
    const bool live = src != sl;
    s_dst[sl] = live ? (int)(k + (sl < kNB ? sl : p)) : -1;  // slot 32 + lane is the row p of this lane
    s_src[sl] = live ? (int)(k + (src < kNB ? src : psrc)) : -1;
  }
}

// Applies panel step k's interchanges to the columns outside the panel: one warp per
// column, all loads of a column before its stores.
constexpr int kSwpCols = 64;  // columns per CTA (the permutation is built once per CTA)
template <typename T>
__global__ void __launch_bounds__(256) laswp_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                   const int32_t* __restrict__ ipiv_all, int64_t k, int kb) {
  using C = typename cplx_t<T>::type;
  __shared__ int s_slot[32], s_content[64], s_dst[64], s_src[64];
  const int64_t bmat = blockIdx.y, n = d.order(bmat);
  if (k >= n) return;  // a grouped batch: this matrix is factored
  kb = (int)((k + kNB < n) ? kNB : n - k);
  if (threadIdx.x < 32) panel_permutation(ipiv_all + bmat * d.n, k, kb, s_slot, s_content, s_dst, s_src);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int d0 = s_dst[lane], s0 = s_src[lane], d1 = s_dst[lane + 32], s1 = s_src[lane + 32];
  C* A = Aall + d.offset(bmat);
  const int64_t nout = n + d.extra - kb;  // columns outside the panel, appended right-hand sides included
  const int64_t q0 = blockIdx.x * (int64_t)kSwpCols;
  const int64_t q1 = (q0 + kSwpCols < nout) ? q0 + kSwpCols : nout;
  for (int64_t q = q0 + warp; q < q1; q += 8) {
    C* col = A + (q < k ? q : q + kb) * n;
    C v0 = czero<C>(), v1 = czero<C>();
    if (d0 >= 0) v0 = col[s0];
    if (d1 >= 0) v1 = col[s1];
    __syncwarp();
    if (d0 >= 0) col[d0] = v0;
    if (d1 >= 0) col[d1] = v1;
  }
}

// The interchanges of the kb panel rows at k applied to the columns [c0, c1) (the other half
// of a two-level panel); one warp per column as in laswp_kernel.
template <typename T>
__global__ void __launch_bounds__(256) laswp_cols_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                        const int32_t* __restrict__ ipiv_all, int64_t k, int kb,
                                                        int64_t c0, int64_t c1) {
  using C = typename cplx_t<T>::type;
  __shared__ int s_slot[32], s_content[64], s_dst[64], s_src[64];
  const int64_t bmat = blockIdx.y, n = d.order(bmat);
  if (k + kb > n) return;
  if (threadIdx.x < 32) panel_permutation(ipiv_all + bmat * d.n, k, kb, s_slot, s_content, s_dst, s_src);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int d0 = s_dst[lane], s0 = s_src[lane], d1 = s_dst[lane + 32], s1 = s_src[lane + 32];
  C* A = Aall + d.offset(bmat);
  const int64_t q0 = c0 + blockIdx.x * (int64_t)kSwpCols;
  const int64_t q1 = (q0 + kSwpCols < c1) ? q0 + kSwpCols : c1;
  for (int64_t q = q0 + warp; q < q1; q += 8) {
    C* col = A + q * n;
    C v0 = czero<C>(), v1 = czero<C>();
    if (d0 >= 0) v0 = col[s0];
    if (d1 >= 0) v1 = col[s1];
    __syncwarp();
    if (d0 >= 0) col[d0] = v0;
    if (d1 >= 0) col[d1] = v1;
  }
}

// U12' = L11'^-1 A[k:k+16, k+16:k+32] of a two-level panel (L11' the unit lower 16 x 16 block of
// the left half): the column-oriented forward substitution with the (15 - r) x 16 updates of
// step r spread over the CTA's threads (GB300's FP64 work has to reach all four schedulers).
template <typename T>
__global__ void __launch_bounds__(256) trsm16_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                    int64_t k) {
  using C = typename cplx_t<T>::type;
  constexpr int H = kNB / 2;
  __shared__ C sL[H][H + 1], sB[H][H + 1];
  const int64_t n = d.order(blockIdx.x);
  if (k + kNB > n) return;
  C* A = Aall + d.offset(blockIdx.x);
  for (int idx = threadIdx.x; idx < H * H; idx += blockDim.x) {
    const int r = idx % H, q = idx / H;
    sL[r][q] = A[(k + r) + (k + q) * n];
    sB[r][q] = A[(k + r) + (k + H + q) * n];
  }
  __syncthreads();
  for (int r = 0; r < H - 1; ++r) {
    const int ne = (H - 1 - r) * H;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const int srow = r + 1 + e / H, c = e % H;
      sB[srow][c] = cfms(sB[srow][c], sL[srow][r], sB[r][c]);
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < H * H; idx += blockDim.x) {
    const int r = idx % H, q = idx / H;
    A[(k + r) + (k + H + q) * n] = sB[r][q];
  }
}

// ------------------------------- U12 -----------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) trsm_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                   int64_t k) {
  using C = typename cplx_t<T>::type;
  __shared__ C sL[kNB][kNB + 1];
  const int64_t n = d.order(blockIdx.y), ncols = n + d.extra;
  if (k >= n) return;  // this matrix is factored (grouped batches)
  C* A = Aall + d.offset(blockIdx.y);
  const int kb = (int)((k + kNB < n) ? kNB : n - k);
  if (k + kb >= ncols) return;  // nothing right of the panel
  for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
    int r = idx % kb, q = idx / kb;
    sL[r][q] = A[(k + r) + (k + q) * n];
  }
  __syncthreads();
  const int64_t c = k + kb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  C x[kNB];
#pragma unroll
  for (int r = 0; r < kNB; ++r) x[r] = (r < kb) ? A[(k + r) + c * n] : czero<C>();
#pragma unroll
  for (int r = 1; r < kNB; ++r) {
#pragma unroll
    for (int q = 0; q < r; ++q) x[r] = cfms(x[r], sL[r][q], x[q]);
  }
#pragma unroll
  for (int r = 0; r < kNB; ++r)
    if (r < kb) A[(k + r) + c * n] = x[r];
}

// ------------------------------ trailing update -------------------------------
// Tile shapes per precision: FP64 is FP64-pipe bound already with 64x64 CTA tiles
// and 4x4 complex outputs per thread; FP32 needs 8x8 outputs per thread (128x128
// CTA tiles) so that the shared-memory loads keep up with the FP32 FMA rate.
template <typename T> struct GemmTile;
template <> struct GemmTile<double> { static constexpr int RM = 4, TM = 64, KC = 16; };
template <> struct GemmTile<float> { static constexpr int RM = 8, TM = 128, KC = 32; };  // whole panel depth

template <typename T>
__global__ void __launch_bounds__(256) gemm_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ Aall,
                                                   int64_t k) {
  using C = typename cplx_t<T>::type;
  constexpr int RM = GemmTile<T>::RM, TM = GemmTile<T>::TM, KC = GemmTile<T>::KC;
  extern __shared__ unsigned char gemm_smem[];
  C (*sA)[TM + 1] = reinterpret_cast<C (*)[TM + 1]>(gemm_smem);
  C (*sB)[TM + 1] = reinterpret_cast<C (*)[TM + 1]>(gemm_smem + sizeof(C) * KC * (TM + 1));
  const int64_t n = d.order(blockIdx.z);
  if (k + kNB >= n) return;  // no trailing block for this matrix (grouped batches)
  C* A = Aall + d.offset(blockIdx.z);
  const int kb = (int)((k + kNB < n) ? kNB : n - k);
  const int64_t base = k + kb;
  const int64_t row0 = base + blockIdx.x * (int64_t)TM;
  const int64_t col0 = base + blockIdx.y * (int64_t)TM;
  if (row0 >= n || col0 >= n) return;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  C acc[RM][RM];
#pragma unroll
  for (int r = 0; r < RM; ++r)
#pragma unroll
    for (int c = 0; c < RM; ++c) acc[r][c] = czero<C>();
  for (int k0 = 0; k0 < kb; k0 += KC) {
    for (int idx = threadIdx.x; idx < KC * TM; idx += 256) {
      int r = idx % TM, q = idx / TM;
      int64_t gi = row0 + r;
      int kk = k0 + q;
      sA[q][r] = (gi < n && kk < kb) ? A[gi + (k + kk) * n] : czero<C>();
    }
    for (int idx = threadIdx.x; idx < KC * TM; idx += 256) {
      int q = idx % KC, c = idx / KC;
      int64_t gc = col0 + c;
      int kk = k0 + q;
      sB[q][c] = (gc < n && kk < kb) ? A[(k + kk) + gc * n] : czero<C>();
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KC; ++q) {
      C a[RM], b[RM];
#pragma unroll
      for (int r = 0; r < RM; ++r) a[r] = sA[q][tx + 16 * r];
#pragma unroll
      for (int c = 0; c < RM; ++c) b[c] = sB[q][ty + 16 * c];
#pragma unroll
      for (int r = 0; r < RM; ++r)
#pragma unroll
        for (int c = 0; c < RM; ++c) acc[r][c] = cfma(acc[r][c], a[r], b[c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < RM; ++c) {
    int64_t gc = col0 + ty + 16 * c;
    if (gc >= n) continue;
#pragma unroll
    for (int r = 0; r < RM; ++r) {
      int64_t gi = row0 + tx + 16 * r;
      if (gi < n) {
        C v = A[gi + gc * n];
        v.x -= acc[r][c].x;
        v.y -= acc[r][c].y;
        A[gi + gc * n] = v;
      }
    }
  }
}

// A22 -= L21 U12 in FP64 with Gauss's three-multiplication complex product (the ZGEMM3M
// scheme): per complex multiply-add P1 += ar br, P2 += ai bi, P3 += (ar + ai)(br + bi), and
// at the end Re = P1 - P2, Im = P3 - P1 - P2 -- three FP64 FMAs instead of four.  The sums
// ar + ai, br + bi are formed once per element when the tiles are staged in shared memory
// (three planes: Re, Im, Re + Im).  The product is normwise stable (its error is bounded by
// a small multiple of the unit roundoff times |L21| |U12|), which is the property the LU's
// backward stability rests on; componentwise the imaginary parts can differ from the
// four-multiplication product in the last digits.
constexpr int kG3TM = 64, kG3RM = 4, kG3KC = 16;
constexpr size_t kG3Smem = 6 * sizeof(double) * kG3KC * (kG3TM + 1);

__global__ void __launch_bounds__(256) gemm3m_kernel(BatchDesc d, double2* __restrict__ Aall, int64_t k) {
  extern __shared__ unsigned char gemm_smem[];
  double (*sAr)[kG3TM + 1] = reinterpret_cast<double (*)[kG3TM + 1]>(gemm_smem);
  double (*sAi)[kG3TM + 1] = sAr + kG3KC;
  double (*sAs)[kG3TM + 1] = sAi + kG3KC;
  double (*sBr)[kG3TM + 1] = sAs + kG3KC;
  double (*sBi)[kG3TM + 1] = sBr + kG3KC;
  double (*sBs)[kG3TM + 1] = sBi + kG3KC;
  const int64_t n = d.order(blockIdx.z);
  if (k + kNB >= n) return;  // no trailing block for this matrix (grouped batches)
  double2* A = Aall + d.offset(blockIdx.z);
  const int kb = (int)((k + kNB < n) ? kNB : n - k);
  const int64_t base = k + kb;
  const int64_t row0 = base + blockIdx.x * (int64_t)kG3TM;
  const int64_t col0 = base + blockIdx.y * (int64_t)kG3TM;
  if (row0 >= n || col0 >= n) return;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double p1[kG3RM][kG3RM], p2[kG3RM][kG3RM], p3[kG3RM][kG3RM];
#pragma unroll
  for (int r = 0; r < kG3RM; ++r)
#pragma unroll
    for (int c = 0; c < kG3RM; ++c) p1[r][c] = p2[r][c] = p3[r][c] = 0.0;
  for (int k0 = 0; k0 < kb; k0 += kG3KC) {
    for (int idx = threadIdx.x; idx < kG3KC * kG3TM; idx += 256) {
      const int r = idx % kG3TM, q = idx / kG3TM;
      const int64_t gi = row0 + r;
      const int kk = k0 + q;
      const double2 v = (gi < n && kk < kb) ? A[gi + (k + kk) * n] : make_double2(0.0, 0.0);
      sAr[q][r] = v.x;
      sAi[q][r] = v.y;
      sAs[q][r] = v.x + v.y;
    }
    for (int idx = threadIdx.x; idx < kG3KC * kG3TM; idx += 256) {
      const int q = idx % kG3KC, c = idx / kG3KC;
      const int64_t gc = col0 + c;
      const int kk = k0 + q;
      const double2 v = (gc < n && kk < kb) ? A[(k + kk) + gc * n] : make_double2(0.0, 0.0);
      sBr[q][c] = v.x;
      sBi[q][c] = v.y;
      sBs[q][c] = v.x + v.y;
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < kG3KC; ++q) {
      double ar[kG3RM], ai[kG3RM], as[kG3RM];
#pragma unroll
      for (int r = 0; r < kG3RM; ++r) {
        ar[r] = sAr[q][tx + 16 * r];
        ai[r] = sAi[q][tx + 16 * r];
        as[r] = sAs[q][tx + 16 * r];
      }
#pragma unroll
      for (int c = 0; c < kG3RM; ++c) {
        const double br = sBr[q][ty + 16 * c], bi = sBi[q][ty + 16 * c], bs = sBs[q][ty + 16 * c];
#pragma unroll
        for (int r = 0; r < kG3RM; ++r) {
          p1[r][c] = fma(ar[r], br, p1[r][c]);
          p2[r][c] = fma(ai[r], bi, p2[r][c]);
          p3[r][c] = fma(as[r], bs, p3[r][c]);
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < kG3RM; ++c) {
    const int64_t gc = col0 + ty + 16 * c;
    if (gc >= n) continue;
#pragma unroll
    for (int r = 0; r < kG3RM; ++r) {
      const int64_t gi = row0 + tx + 16 * r;
      if (gi < n) {
        double2 v = A[gi + gc * n];
        v.x -= p1[r][c] - p2[r][c];
        v.y -= p3[r][c] - p1[r][c] - p2[r][c];
        A[gi + gc * n] = v;
      }
    }
  }
}

// ------------------------------ substitution ---------------------------------
// x_r[i] -= sum_{j in [jb, je)} M[i, j] x_r[j] for the g right-hand sides of the
// group (M = the stored factor, or its conjugate transpose when CT); every matrix
// element is loaded once and applied to up to kSG vectors held in registers.
constexpr int kSG = 8;


// Diagonal 32x32 block solves done by one warp: the block sits in shared memory
// (blk, 32 x 33 padded, blk[l*33+q] = M[jb+l, jb+q] as stored), lane l owns
// entry jb+l of the solution, and solved entries travel by shuffle.
// KIND 0: unit lower L; 1: upper U; 2: lower U^H; 3: unit upper L^H.
template <typename C>
__device__ __forceinline__ void load_diag_block(const C* __restrict__ LU, int64_t n, int64_t jb, int bw, C* blk) {
  for (int idx = threadIdx.x; idx < bw * bw; idx += blockDim.x) {
    int r = idx % bw, q = idx / bw;
    blk[r * 33 + q] = LU[(jb + r) + (jb + q) * n];
  }
}

template <typename C, int KIND>
__device__ __forceinline__ void diag_block_solve(const C* blk, int64_t n, int64_t jb, int bw, C* xs, int g,
                                                 int lane) {
  for (int r = 0; r < g; ++r) {
    C* x = xs + (int64_t)r * n;
    C xl = lane < bw ? x[jb + lane] : czero<C>();
    if (KIND == 0 || KIND == 2) {
#pragma unroll 4
      for (int q = 0; q < bw; ++q) {
        C m = (KIND == 0) ? blk[lane * 33 + q] : cconj(blk[q * 33 + lane]);
        if (KIND == 2 && lane == q) xl = cdiv(xl, m);
        C xq = shfl_c(xl, q);
        if (lane > q && lane < bw) xl = cfms(xl, m, xq);
      }
    } else {
#pragma unroll 4
      for (int q = bw - 1; q >= 0; --q) {
        C m = (KIND == 1) ? blk[lane * 33 + q] : cconj(blk[q * 33 + lane]);
        if (KIND == 1 && lane == q) xl = cdiv(xl, m);
        C xq = shfl_c(xl, q);
        if (lane < q) xl = cfms(xl, m, xq);
      }
    }
    if (lane < bw) x[jb + lane] = xl;
  }
}

template <typename C, bool CT>
__device__ __forceinline__ void update_row(const C* __restrict__ LU, int64_t n, int64_t i, int64_t jb, int64_t je,
                                           C* xs, int g) {
  for (int r0 = 0; r0 < g; r0 += kSG) {
    C acc[kSG];
#pragma unroll
    for (int r = 0; r < kSG; ++r) acc[r] = czero<C>();
    const int gr = (g - r0 < kSG) ? g - r0 : kSG;
    if (je - jb == 32) {
#pragma unroll 8
      for (int jj = 0; jj < 32; ++jj) {
        const int64_t j = jb + jj;
        C m = CT ? cconj(LU[j + i * n]) : LU[i + j * n];
#pragma unroll
        for (int r = 0; r < kSG; ++r)
          if (r < gr) acc[r] = cfma(acc[r], m, xs[(r0 + r) * n + j]);
      }
    } else {
      for (int64_t j = jb; j < je; ++j) {
        C m = CT ? cconj(LU[j + i * n]) : LU[i + j * n];
#pragma unroll
        for (int r = 0; r < kSG; ++r)
          if (r < gr) acc[r] = cfma(acc[r], m, xs[(r0 + r) * n + j]);
      }
    }
#pragma unroll
    for (int r = 0; r < kSG; ++r)
      if (r < gr) xs[(r0 + r) * n + i] = csub(xs[(r0 + r) * n + i], acc[r]);
  }
}

// One CTA per (group of right-hand sides, matrix); the group's vectors live in
// shared memory.  Forward: unit lower L; backward: upper U; both in 32-column
// blocks (warp 0 solves the diagonal block, all threads update the rest).
// ADJ: solves A^H x = b = U^H L^H P^T x.
template <typename T, bool ADJ>
__global__ void __launch_bounds__(512) solve_kernel(BatchDesc d, const typename cplx_t<T>::type* __restrict__ LUall,
                                                    const int32_t* __restrict__ ipiv_all,
                                                    typename cplx_t<T>::type* __restrict__ Xall, int64_t nrhs,
                                                    int64_t xstride, int group, int upper_only) {
  using C = typename cplx_t<T>::type;
  extern __shared__ unsigned char smem_raw[];
  C* blk = reinterpret_cast<C*>(smem_raw);
  C* xs = blk + 32 * 33;
  const int64_t n = d.order(blockIdx.y);
  const C* LU = LUall + d.offset(blockIdx.y);
  const int32_t* ipiv = ipiv_all + blockIdx.y * d.n;
  C* X = Xall + d.xoffset(blockIdx.y, xstride);
  const int64_t r0 = blockIdx.x * (int64_t)group;
  const int g = (int)((r0 + group <= nrhs) ? group : nrhs - r0);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int64_t idx = tid; idx < g * n; idx += blockDim.x) {
    int64_t r = idx / n, i = idx % n;
    xs[r * n + i] = X[i + (r0 + r) * n];
  }
  __syncthreads();
  if (!ADJ) {
    if (tid < g && !upper_only) {  // apply the row interchanges in order (zgetrs / zlaswp)
      C* x = xs + tid * n;
      for (int64_t j = 0; j < n; ++j) {
        int64_t p = ipiv[j];
        if (p != j) { C t = x[j]; x[j] = x[p]; x[p] = t; }
      }
    }
    __syncthreads();
    // L y = b
    for (int64_t jb = 0; jb < (upper_only ? 0 : n); jb += 32) {
      const int64_t je = (jb + 32 < n) ? jb + 32 : n;
      load_diag_block(LU, n, jb, (int)(je - jb), blk);
      __syncthreads();
      if (warp == 0) diag_block_solve<C, 0>(blk, n, jb, (int)(je - jb), xs, g, lane);
      __syncthreads();
      for (int64_t i = je + tid; i < n; i += blockDim.x) update_row<C, false>(LU, n, i, jb, je, xs, g);
      __syncthreads();
    }
    // U x = y
    const int64_t nblk = (n + 31) / 32;
    for (int64_t bI = nblk - 1; bI >= 0; --bI) {
      const int64_t jb = bI * 32, je = (jb + 32 < n) ? jb + 32 : n;
      load_diag_block(LU, n, jb, (int)(je - jb), blk);
      __syncthreads();
      if (warp == 0) diag_block_solve<C, 1>(blk, n, jb, (int)(je - jb), xs, g, lane);
      __syncthreads();
      for (int64_t i = tid; i < jb; i += blockDim.x) update_row<C, false>(LU, n, i, jb, je, xs, g);
      __syncthreads();
    }
  } else {
    // U^H w = b (lower triangular, conj(U) transposed)
    for (int64_t jb = 0; jb < n; jb += 32) {
      const int64_t je = (jb + 32 < n) ? jb + 32 : n;
      load_diag_block(LU, n, jb, (int)(je - jb), blk);
      __syncthreads();
      if (warp == 0) diag_block_solve<C, 2>(blk, n, jb, (int)(je - jb), xs, g, lane);
      __syncthreads();
      for (int64_t i = je + tid; i < n; i += blockDim.x) update_row<C, true>(LU, n, i, jb, je, xs, g);
      __syncthreads();
    }
    // L^H v = w (upper, unit diagonal)
    const int64_t nblk = (n + 31) / 32;
    for (int64_t bI = nblk - 1; bI >= 0; --bI) {
      const int64_t jb = bI * 32, je = (jb + 32 < n) ? jb + 32 : n;
      load_diag_block(LU, n, jb, (int)(je - jb), blk);
      __syncthreads();
      if (warp == 0) diag_block_solve<C, 3>(blk, n, jb, (int)(je - jb), xs, g, lane);
      __syncthreads();
      for (int64_t i = tid; i < jb; i += blockDim.x) update_row<C, true>(LU, n, i, jb, je, xs, g);
      __syncthreads();
    }
    if (tid < g) {  // x = P v: undo the interchanges in reverse order
      C* x = xs + tid * n;
      for (int64_t j = n - 1; j >= 0; --j) {
        int64_t p = ipiv[j];
        if (p != j) { C t = x[j]; x[j] = x[p]; x[p] = t; }
      }
    }
    __syncthreads();
  }
  for (int64_t idx = tid; idx < g * n; idx += blockDim.x) {
    int64_t r = idx / n, i = idx % n;
    X[i + (r0 + r) * n] = xs[r * n + i];
  }
}

// ---------------------------- solve on a cluster --------------------------------
// One cluster of P CTAs per (group of g <= kSG right-hand sides, matrix).  The 32-row
// blocks of the solution are dealt out cyclically (block b to CTA b % P), each CTA keeps
// its blocks' entries of the g vectors in shared memory.  The solve is a sequence of
// 2 nblk block steps (L then U, or U^H then L^H).  At step s the owner of block s has
// already solved it and posted its entries in a double-buffered slot; every CTA copies
// the slot through distributed shared memory and subtracts the block's contribution from
// its own rows.  The owner of block s + 1 first updates that block's rows, solves it (one
// warp per vector, reciprocals of the diagonal precomputed), posts it and arrives at the
// split cluster barrier, and only then updates the rest of its rows; every other CTA
// arrives as soon as it has its copy.  So the barrier waits only for the next block, not
// for the whole update.  The permutation of the right-hand sides (the LU's row
// interchanges) is composed once per CTA into an index map: x = b[sigma] before L
// (forward), x[sigma] = v after L^H (adjoint).

// kind of block step s (KIND of diag_block_solve) and its block index
template <bool ADJ> __device__ __forceinline__ void solve_step(int s, int nblk, int& kind, int& bI) {
  if (s < nblk) { kind = ADJ ? 2 : 0; bI = s; }
  else { kind = ADJ ? 3 : 1; bI = 2 * nblk - 1 - s; }
}

// one warp solves the block entries x[0 .. bw) of one vector in place; rd: reciprocals of
// the diagonal (KIND 1, 2)
template <typename C, int KIND>
__device__ __forceinline__ void block_solve_slot(const C* blk, const C* rd, int bw, C* x, int lane) {
  C xl = lane < bw ? x[lane] : czero<C>();
  if (KIND == 0 || KIND == 2) {
#pragma unroll 4
    for (int q = 0; q < bw; ++q) {
      C m = (KIND == 0) ? blk[lane * 33 + q] : cconj(blk[q * 33 + lane]);
      if (KIND == 2 && lane == q) xl = cmul(xl, rd[q]);
      C xq = shfl_c(xl, q);
      if (lane > q && lane < bw) xl = cfms(xl, m, xq);
    }
  } else {
#pragma unroll 4
    for (int q = bw - 1; q >= 0; --q) {
      C m = (KIND == 1) ? blk[lane * 33 + q] : cconj(blk[q * 33 + lane]);
      if (KIND == 1 && lane == q) xl = cmul(xl, rd[q]);
      C xq = shfl_c(xl, q);
      if (lane < q) xl = cfms(xl, m, xq);
    }
  }
  if (lane < bw) x[lane] = xl;
}

constexpr int kXbStride = 33;  // padded: the g vectors of one row read different banks

// rows of block b2 take the contribution of block bI at this step?
__device__ __forceinline__ bool step_updates(int kind, int bI, int b2) {
  return (kind == 0 || kind == 2) ? (b2 > bI) : (b2 < bI);
}

// x_i -= sum_jj M(i, jb + jj) xb[q][jj] for the local rows li in [l0, l1) that step (kind,
// bI) updates, skipping local block `skip`; work item = (row, vector) so that one block's
// 32 rows still spread over the CTA
template <typename C>
__device__ __forceinline__ void cluster_update_rows(const C* __restrict__ LU, int64_t n, int kind, int bI, int bw,
                                                    int P, int rank, int g, int ln, C* xl, const C* xb, int l0, int l1,
                                                    int skip) {
  const bool ct = (kind >= 2);
  const int64_t jb = (int64_t)bI * 32;
  const int rows = l1 - l0;
  for (int w = threadIdx.x; w < rows * g; w += blockDim.x) {
    const int li = l0 + w / g, q = w % g;  // the g vectors of a row on neighbouring threads
    const int lb = li >> 5;
    if (lb == skip) continue;
    const int b2 = rank + lb * P;
    if (!step_updates(kind, bI, b2)) continue;
    const int64_t i = (int64_t)b2 * 32 + (li & 31);
    if (i >= n) continue;
    C acc = czero<C>();
    const C* xq = xb + q * kXbStride;
    if (ct) {
      const C* col = LU + i * n + jb;  // M(i, j) = conj(LU[j, i]): row i of LU^H is column i of LU
#pragma unroll 8
      for (int jj = 0; jj < bw; ++jj) acc = cfma(acc, cconj(col[jj]), xq[jj]);
    } else {
      const C* row = LU + i + jb * n;
#pragma unroll 8
      for (int jj = 0; jj < bw; ++jj) acc = cfma(acc, row[(int64_t)jj * n], xq[jj]);
    }
    xl[(int64_t)q * ln + li] = csub(xl[(int64_t)q * ln + li], acc);
  }
}

template <typename C, bool ADJ>
__device__ __forceinline__ void cluster_solve_block(const C* __restrict__ LU, int64_t n, int kind, int bI, int P,
                                                    int g, int ln, C* xl, C* blk, C* rd, C* post) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t jb = (int64_t)bI * 32;
  const int bw = (int)((jb + 32 < n) ? 32 : n - jb);
  load_diag_block(LU, n, jb, bw, blk);
  __syncthreads();
  if (warp == 0 && lane < bw) {
    const C dgl = blk[lane * 33 + lane];
    rd[lane] = crecip(kind == 2 ? cconj(dgl) : dgl);
  }
  __syncthreads();
  if (warp < g) {
    C* x = xl + (int64_t)warp * ln + (bI / P) * 32;
    switch (kind) {
      case 0: block_solve_slot<C, 0>(blk, rd, bw, x, lane); break;
      case 1: block_solve_slot<C, 1>(blk, rd, bw, x, lane); break;
      case 2: block_solve_slot<C, 2>(blk, rd, bw, x, lane); break;
      default: block_solve_slot<C, 3>(blk, rd, bw, x, lane); break;
    }
    __syncwarp();
    post[warp * 32 + lane] = lane < bw ? x[lane] : czero<C>();
  }
}

template <typename T, bool ADJ>
__global__ void __launch_bounds__(512) solve_cluster_kernel(BatchDesc d, const typename cplx_t<T>::type* __restrict__ LUall,
                                                            const int32_t* __restrict__ ipiv_all,
                                                            typename cplx_t<T>::type* __restrict__ Xall, int64_t nrhs,
                                                            int64_t xstride, int group, int ln, int upper_only) {
  using C = typename cplx_t<T>::type;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char solve_smem[];
  C* xl = reinterpret_cast<C*>(solve_smem);                          // g x ln, vector-major
  int* sig = reinterpret_cast<int*>(xl + (int64_t)group * ln);       // n
  int* spv = sig + d.n;                                              // n: the pivots
  __shared__ C blk[32 * 33];
  __shared__ C rd[32];
  __shared__ C pub[2][32 * kSG];
  __shared__ C xb[2][kXbStride * kSG];
  const int P = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int64_t n = d.order(blockIdx.z);
  const int nblk = (int)((n + 31) / 32);
  const C* LU = LUall + d.offset(blockIdx.z);
  const int32_t* ipiv = ipiv_all + blockIdx.z * d.n;
  C* X = Xall + d.xoffset(blockIdx.z, xstride);
  const int64_t r0 = blockIdx.y * (int64_t)group;
  const int g = (int)((r0 + group <= nrhs) ? group : nrhs - r0);
  const int tid = threadIdx.x;
  // sigma: the row interchanges composed in order (x = b[sigma] applies them to b); the
  // identity when the right-hand sides went through the factorization (upper_only)
  for (int64_t i = tid; i < n; i += blockDim.x) { sig[i] = (int)i; spv[i] = upper_only ? (int)i : ipiv[i]; }
  __syncthreads();
  if (tid == 0 && !upper_only)
    for (int64_t j = 0; j < n; ++j) {
      const int p = spv[j];
      if (p != j) { const int t = sig[j]; sig[j] = sig[p]; sig[p] = t; }
    }
  __syncthreads();
  const int nlb = (nblk - rank + P - 1) / P;
  const int nloc = nlb * 32;
  for (int w = tid; w < nloc * g; w += blockDim.x) {
    const int li = w % nloc, q = w / nloc;
    const int64_t i = (int64_t)(rank + (li >> 5) * P) * 32 + (li & 31);
    if (i < n) xl[(int64_t)q * ln + li] = X[(ADJ ? i : sig[i]) + (r0 + q) * n];
  }
  __syncthreads();
  const int nsteps = 2 * nblk;
  const int s0 = upper_only ? nblk : 0;  // upper_only: the U steps alone
  int kind, bI;
  solve_step<ADJ>(s0, nblk, kind, bI);
  if (bI % P == rank) cluster_solve_block<C, ADJ>(LU, n, kind, bI, P, g, ln, xl, blk, rd, pub[s0 & 1]);
  cluster_arrive();
  cluster_wait();
  for (int s = s0; s < nsteps; ++s) {
    solve_step<ADJ>(s, nblk, kind, bI);
    const int bw = (int)(((int64_t)bI * 32 + 32 < n) ? 32 : n - (int64_t)bI * 32);
    C* xs = xb[s & 1];
    const C* src = cl.map_shared_rank(&pub[s & 1][0], (unsigned)(bI % P));
    for (int e = tid; e < 32 * g; e += blockDim.x) xs[(e >> 5) * kXbStride + (e & 31)] = src[e];
    __syncthreads();
    const bool last = (s + 1 == nsteps);
    int nkind = 0, nbI = 0, skip = -1;
    if (!last) {
      solve_step<ADJ>(s + 1, nblk, nkind, nbI);
      if (nbI % P == rank) {
        // the next block first: its rows, its solve, its slot
        const int lb = nbI / P;
        if (step_updates(kind, bI, nbI))
          cluster_update_rows<C>(LU, n, kind, bI, bw, P, rank, g, ln, xl, xs, lb * 32, lb * 32 + 32, -1);
        __syncthreads();
        cluster_solve_block<C, ADJ>(LU, n, nkind, nbI, P, g, ln, xl, blk, rd, pub[(s + 1) & 1]);
        skip = lb;
      }
    }
    cluster_arrive();  // step s + 1 posted (or nothing to post)
    cluster_update_rows<C>(LU, n, kind, bI, bw, P, rank, g, ln, xl, xs, 0, nloc, skip);
    cluster_wait();
  }
  __syncthreads();
  for (int w = tid; w < nloc * g; w += blockDim.x) {
    const int li = w % nloc, q = w / nloc;
    const int64_t i = (int64_t)(rank + (li >> 5) * P) * 32 + (li & 31);
    if (i < n) X[(ADJ ? sig[i] : i) + (r0 + q) * n] = xl[(int64_t)q * ln + li];
  }
}

// ------------------------------ Y = A X (FP64) --------------------------------
constexpr int kGemvRows = 128;
constexpr int kGemvNR = 8;

// partial[js][b][r][i] = sum_{j in chunk js} A_b[i, j] X_b[j, r]  (ADJ: A^H)
template <bool ADJ>
__global__ void __launch_bounds__(kGemvRows) zgemm_partial_kernel(BatchDesc d, const double2* __restrict__ Aall,
                                                                  const double2* __restrict__ Xall, int64_t nrhs,
                                                                  int64_t xstride, int64_t jchunk, int r0,
                                                                  double2* __restrict__ part) {
  const int64_t n = d.n;
  const int64_t i = blockIdx.x * (int64_t)kGemvRows + threadIdx.x;
  const int64_t js = blockIdx.y;
  const int64_t b = blockIdx.z;
  const double2* A = Aall + b * d.stride;
  const double2* X = Xall + b * xstride;
  const int64_t ja = js * jchunk, jbnd = (ja + jchunk < n) ? ja + jchunk : n;
  const int g = (int)((r0 + kGemvNR <= nrhs) ? kGemvNR : nrhs - r0);
  double2 acc[kGemvNR];
#pragma unroll
  for (int r = 0; r < kGemvNR; ++r) acc[r] = make_double2(0.0, 0.0);
  if (i < n) {
    for (int64_t j = ja; j < jbnd; ++j) {
      double2 a = ADJ ? cconj(__ldg(A + j + i * n)) : __ldg(A + i + j * n);
#pragma unroll
      for (int r = 0; r < kGemvNR; ++r)
        if (r < g) acc[r] = cfma(acc[r], a, __ldg(X + j + (r0 + r) * n));
    }
    double2* P = part + ((js * d.batch + b) * nrhs) * n;
#pragma unroll
    for (int r = 0; r < kGemvNR; ++r)
      if (r < g) P[(r0 + r) * n + i] = acc[r];
  }
}

__global__ void zgemm_reduce_kernel(BatchDesc d, int64_t nrhs, int64_t nsplit, const double2* __restrict__ part,
                                    double2* __restrict__ Yall, int64_t ystride, const double2* __restrict__ Ball,
                                    int subtract_from_b) {
  const int64_t n = d.n;
  const int64_t per = nrhs * n;
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= per * d.batch) return;
  const int64_t b = q / per, e = q % per;
  double2 s = make_double2(0.0, 0.0);
  for (int64_t js = 0; js < nsplit; ++js) {
    double2 v = part[(js * d.batch + b) * per + e];
    s.x += v.x;
    s.y += v.y;
  }
  if (subtract_from_b) {
    double2 bb = Ball[b * ystride + e];
    s = make_double2(bb.x - s.x, bb.y - s.y);
  }
  Yall[b * ystride + e] = s;
}

int64_t gemm_split(int64_t n, int64_t batch) {
  int64_t rows = (n + kGemvRows - 1) / kGemvRows;
  int64_t want = (4 * 152 + rows * batch - 1) / (rows * batch);
  int64_t maxs = (n + 63) / 64;
  if (want < 1) want = 1;
  if (want > maxs) want = maxs;
  return want;
}

__global__ void z_to_c_kernel(const double2* __restrict__ s, float2* __restrict__ d, int64_t count) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) d[q] = make_float2((float)s[q].x, (float)s[q].y);
}

__global__ void c_to_z_kernel(const float2* __restrict__ s, double2* __restrict__ d, int64_t count) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) d[q] = make_double2((double)s[q].x, (double)s[q].y);
}

__global__ void ir_update_kernel(double2* __restrict__ X, const float2* __restrict__ Cc, int64_t count) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) { X[q].x += (double)Cc[q].x; X[q].y += (double)Cc[q].y; }
}

// out[col] = max_i |re| + |im|  over column col of an n x ncols array
__global__ void col_inf_norm_kernel(int64_t n, const double2* __restrict__ X, double* __restrict__ out) {
  const int64_t col = blockIdx.x;
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double2 v = X[i + col * n];
    double a = fabs(v.x) + fabs(v.y);
    m = a > m ? a : m;
  }
  __shared__ double red[8];
  for (int off = 16; off > 0; off >>= 1) { double o = __shfl_down_sync(0xffffffffu, m, off); m = o > m ? o : m; }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = red[w] > r ? red[w] : r;
    out[col] = r;
  }
}


// the FP32 copy of matrix b (column stride n, matrix stride stride32; a grouped batch: at the
// matrix's own element offset) and, in the same pass
// over A, out[b] = max_i sum_j |re|+|im| (|.|_inf, order independent via atomicMax on the bits
// of a non-negative double; out zeroed first).  128 rows x 8 column slices per CTA, the
// slices' partial row sums added in a fixed order.
__global__ void __launch_bounds__(1024) convert_norm_kernel(BatchDesc d, const double2* __restrict__ A,
                                                            float2* __restrict__ A32, int64_t stride32,
                                                            unsigned long long* __restrict__ out) {
  __shared__ double part[8][128];
  const int64_t i = blockIdx.x * (int64_t)128 + threadIdx.x;
  const int64_t b = blockIdx.y;
  // a grouped batch: the FP32 copies sit at the same element offsets as the matrices
  const int64_t n = d.order(b);
  const double2* Ab = A + d.offset(b);
  float2* Cb = A32 + (d.offsets ? d.offsets[b] : b * stride32);
  const int64_t j0 = (n * threadIdx.y) / 8, j1 = (n * (threadIdx.y + 1)) / 8;
  double s = 0.0;
  if (i < n) {
#pragma unroll 4
    for (int64_t j = j0; j < j1; ++j) {
      const double2 v = Ab[i + j * n];
      Cb[i + j * n] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
      s += fabs(v.x) + fabs(v.y);
    }
  }
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && i < n) {
    double t = 0.0;
    for (int y = 0; y < 8; ++y) t += part[y][threadIdx.x];
    atomicMax(out + b, (unsigned long long)__double_as_longlong(t));
  }
}

}  // namespace

void convert_with_norms(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, float2* A32,
                        int64_t stride32, double* out) {
  cudaMemsetAsync(out, 0, sizeof(double) * d.batch, st);
  dim3 grid((unsigned)((d.n + 127) / 128), (unsigned)d.batch);
  MH_LAUNCH(lc, st, "convert", convert_norm_kernel<<<grid, dim3(128, 8), 0, st>>>(d, A, A32, stride32,
                                                                                (unsigned long long*)out));
}


// CTAs per cluster for a panel of m rows in a batch of `batch` matrices: enough to hold
// the panel in shared memory, and more (up to 8) while all `batch` clusters still fit on
// the GPU at once (clusters are placed within one GPC, so this is taken from the
// occupancy query, not from the SM count), at most `cap` beyond the minimum (the
// launch-shape table's cluster bound); 0 when the panel does not fit the largest cluster
// the GPU can schedule (panel_kernel then runs).
template <typename T>
int panel_cluster_size(int64_t m, int64_t batch, int cap_ctas, int width = kNB) {
  using C = typename cplx_t<T>::type;
  constexpr int cap = PanelRows<T>::value;
  struct Table { int resident[17]; };
  // clusters resident at once at the largest chunk: a full-width panel fills one SM's shared
  // memory, a half-width one (two-level panels) half of it
  auto make_table = [](int w) {
    Table t{};
    // the attribute always allows the full-width panel; the query uses this width's size
    cudaFuncSetAttribute(panel_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         cap * kNB * (int)sizeof(C));
    cudaFuncSetAttribute(panel_cluster_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    const int smem = cap * w * (int)sizeof(C);
    for (int p = 1; p <= 16; ++p) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)p, 1, 1);
      cfg.blockDim = dim3(kPanelThreads, 1, 1);
      cfg.dynamicSmemBytes = (size_t)smem;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)p;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int num = 0;
      if (cudaOccupancyMaxActiveClusters(&num, panel_cluster_kernel<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        num = 0;
      }
      t.resident[p] = num;  // clusters of p CTAs resident at once, at the largest chunk
    }
    return t;
  };
  static const Table tab_full = make_table(kNB);
  static const Table tab_half = make_table(kNB / 2);
  static const int sms = [] {
    int dev = 0, v = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v;
  }();
  const Table& tab = width < kNB ? tab_half : tab_full;
  int64_t need = (m + cap - 1) / cap;
  if (need < 1) need = 1;
  if (need > 16 || tab.resident[need] <= 0) return 0;
  const int64_t lim = m / kNB > 1 ? m / kNB : 1;  // keeps every chunk >= 32 rows (CTA 0 holds the diagonal block)
  int64_t p = need;
  // more CTAs per matrix while all clusters stay resident and every CTA keeps an SM of its own
  // (the panel is FP64-bound per SM)
  for (int64_t q = need + 1; q <= 8 && q <= lim && q <= cap_ctas; ++q)
    if (tab.resident[q] >= batch && q * batch <= sms) p = q;
  return (int)p;
}

// true when the full-width panel of m rows runs its clusters for all `batch` matrices at once
// (its rows need at most as many CTAs per matrix as fit every cluster on the GPU); a panel that
// does not fit runs in waves, and the FP64 tensor-core path factors it in two halves instead
template <typename T>
bool panel_fits_one_wave(int64_t m, int64_t batch) {
  constexpr int cap = PanelRows<T>::value;
  const int64_t need = (m + cap - 1) / cap;
  static int resident[17] = {-1};
  if (resident[0] < 0) {
    using C = typename cplx_t<T>::type;
    cudaFuncSetAttribute(panel_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap * kNB * (int)sizeof(C));
    cudaFuncSetAttribute(panel_cluster_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int p = 1; p <= 16; ++p) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)p, 1, 1);
      cfg.blockDim = dim3(kPanelThreads, 1, 1);
      cfg.dynamicSmemBytes = (size_t)cap * kNB * sizeof(C);
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)p;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int num = 0;
      if (cudaOccupancyMaxActiveClusters(&num, panel_cluster_kernel<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        num = 0;
      }
      resident[p] = num;
    }
    resident[0] = 0;
  }
  return need <= 16 && resident[need] >= batch;
}

template <typename T>
int lu_factor_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, typename cplx_t<T>::type* A,
                      int32_t* ipiv, int32_t* info, void* emu_ws, int* emu_flag) {
  const int64_t n = d.n;
  if (n <= 0 || d.batch <= 0) return 0;
  // appended right-hand sides need the rectangular trailing update of the FP64 tensor-core path
  if (d.extra > 0 && (sizeof(T) != 8 || !emu_ws || d.orders)) return -1;
  cudaMemsetAsync(info, 0, sizeof(int32_t) * d.batch, st);
  {
    constexpr int TM = GemmTile<T>::TM;
    constexpr size_t gsmem = 2 * sizeof(typename cplx_t<T>::type) * GemmTile<T>::KC * (TM + 1);
    cudaFuncSetAttribute(gemm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsmem);
    if (sizeof(T) == 8)
      cudaFuncSetAttribute(gemm3m_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kG3Smem);
  }
  const int cap_ctas = sizeof(T) == 8 ? lc.tile(n).cluster_f64 : lc.tile(n).cluster_f32;
  // the panel at k0 of `width` columns on a cluster of P CTAs
  auto cluster_panel = [&](int64_t k0, int width, int P) {
    const int chunk = (int)((n - k0 + P - 1) / P);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P, (unsigned)d.batch, 1);
    cfg.blockDim = dim3(kPanelThreads, 1, 1);
    cfg.dynamicSmemBytes = (size_t)chunk * width * sizeof(typename cplx_t<T>::type);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)P;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MH_LAUNCH(lc, st, sizeof(T) == 8 ? "lu_panel_f64" : "lu_panel_f32",
              cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T>, d, A, ipiv, info, k0, chunk, width));
  };
  for (int64_t k = 0; k < n; k += kNB) {
    const int64_t kb = (k + kNB < n) ? kNB : n - k;
    // Two-level panel (FP64 with the tensor-core update, tall panels): two 16-column halves
    // on the CUDA cores, the left half's update of the right half (K = 16) on the tensor
    // cores -- half the panel's FP64 work, and half its shared memory per row
    int Pl = 0, P16 = 0;
    if constexpr (sizeof(T) == 8) {
      if (emu_ws && kb == kNB && !d.orders && !panel_fits_one_wave<T>(n - k, d.batch)) {
        Pl = panel_cluster_size<T>(n - k, d.batch, cap_ctas, kNB / 2);
        P16 = panel_cluster_size<T>(n - k - kNB / 2, d.batch, cap_ctas, kNB / 2);
      }
    }
    if (Pl > 0 && P16 > 0) {
      if constexpr (sizeof(T) == 8) {
        const int H = kNB / 2;
        cluster_panel(k, H, Pl);
        dim3 sg(1u, (unsigned)d.batch);
        MH_LAUNCH(lc, st, "lu_laswp_f64", laswp_cols_kernel<T><<<sg, 256, 0, st>>>(d, A, ipiv, k, H, k + H, k + kNB));
        MH_LAUNCH(lc, st, "lu_trsm16_f64", trsm16_kernel<T><<<(unsigned)d.batch, 256, 0, st>>>(d, A, k));
        ozaki_trailing_update(st, lc, d, A, k, H, emu_ws, emu_flag, H);
        cluster_panel(k + H, H, P16);
        MH_LAUNCH(lc, st, "lu_laswp_f64", laswp_cols_kernel<T><<<sg, 256, 0, st>>>(d, A, ipiv, k + H, H, k, k + H));
      }
    } else {
      const int P = panel_cluster_size<T>(n - k, d.batch, cap_ctas);
      if (P > 0) {
        cluster_panel(k, kNB, P);
      } else {
        MH_LAUNCH(lc, st, sizeof(T) == 8 ? "lu_panel_f64" : "lu_panel_f32",
                  panel_kernel<T><<<(unsigned)d.batch, 512, 0, st>>>(d, A, ipiv, info, k));
      }
    }
    if (n + d.extra - kb > 0) {
      dim3 sg((unsigned)((n + d.extra - kb + kSwpCols - 1) / kSwpCols), (unsigned)d.batch);
      MH_LAUNCH(lc, st, sizeof(T) == 8 ? "lu_laswp_f64" : "lu_laswp_f32",
                laswp_kernel<T><<<sg, 256, 0, st>>>(d, A, ipiv, k, (int)kb));
    }
    const int64_t rest = n - k - kb;              // trailing rows
    const int64_t rest_c = n + d.extra - k - kb;  // columns right of the panel
    if (rest_c <= 0) continue;
    bool trsm_done = false;
    if constexpr (sizeof(T) == 8) {  // FP64 with the tensor-core update: U12 on the tensor cores too
      if (emu_ws && kb == kNB) {
        ozaki_trsm(st, lc, d, A, k, emu_ws, emu_flag);
        trsm_done = true;
      }
    }
    if (!trsm_done) {
      dim3 tg((unsigned)((rest_c + 127) / 128), (unsigned)d.batch);
      MH_LAUNCH(lc, st, sizeof(T) == 8 ? "lu_trsm_f64" : "lu_trsm_f32", trsm_kernel<T><<<tg, 128, 0, st>>>(d, A, k));
    }
    if (rest <= 0) continue;
    if (emu_ws) {
      if constexpr (sizeof(T) == 8) {  // FP64 update on the BF16 tensor cores (mh_ozaki.cu)
        ozaki_trailing_update(st, lc, d, A, k, (int)kb, emu_ws, emu_flag);
      } else {  // FP32 update on the BF16 tensor cores (mh_bf16x3.cu)
        bx3_trailing_update(st, lc, d, A, k, (int)kb, emu_ws, emu_flag);
      }
      continue;
    }
    if constexpr (sizeof(T) == 8) {  // FP64: three real products per complex multiply-add
      dim3 gg((unsigned)((rest + kG3TM - 1) / kG3TM), (unsigned)((rest + kG3TM - 1) / kG3TM), (unsigned)d.batch);
      MH_LAUNCH(lc, st, "lu_gemm_f64", gemm3m_kernel<<<gg, 256, kG3Smem, st>>>(d, A, k));
    } else {
      constexpr int TM = GemmTile<T>::TM;
      dim3 gg((unsigned)((rest + TM - 1) / TM), (unsigned)((rest + TM - 1) / TM), (unsigned)d.batch);
      constexpr size_t gsmem = 2 * sizeof(typename cplx_t<T>::type) * GemmTile<T>::KC * (TM + 1);
      MH_LAUNCH(lc, st, "lu_gemm_f32", gemm_kernel<T><<<gg, 256, gsmem, st>>>(d, A, k));
    }
  }
  return 0;
}

// Cluster size for the solve: the fewest CTAs whose shares of the vectors fit in shared
// memory, raised (up to 8) while every (matrix, group) cluster is still resident at once.
// Returns false when even 8 CTAs cannot hold the vectors (the one-CTA kernel then runs).
template <typename T>
bool solve_on_cluster(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const typename cplx_t<T>::type* LU,
                      const int32_t* ipiv, typename cplx_t<T>::type* X, int64_t nrhs, int64_t xstride, bool adjoint,
                      bool upper_only) {
  using C = typename cplx_t<T>::type;
  const int64_t n = d.n;
  const int g = (int)(nrhs < kSG ? nrhs : kSG);
  const int64_t ngroups = (nrhs + g - 1) / g;
  const int64_t nblk = (n + 31) / 32;
  const size_t max_dyn = 190 * 1024;
  auto dyn_bytes = [&](int p) {
    const int64_t ln = (nblk + p - 1) / p * 32;
    return (size_t)ln * g * sizeof(C) + 2 * sizeof(int) * (size_t)n;
  };
  const void* fn = adjoint ? (const void*)solve_cluster_kernel<T, true> : (const void*)solve_cluster_kernel<T, false>;
  static const bool attr_set = [] {
    cudaFuncSetAttribute(solve_cluster_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 190 * 1024);
    cudaFuncSetAttribute(solve_cluster_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 190 * 1024);
    return true;
  }();
  (void)attr_set;
  auto make_cfg = [&](int p, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)p, (unsigned)ngroups, (unsigned)d.batch);
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = dyn_bytes(p);
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)p;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
  };
  int need = 0;
  for (int p = 1; p <= 8 && p <= nblk; ++p)
    if (dyn_bytes(p) <= max_dyn) { need = p; break; }
  if (need == 0) return false;
  int P = need;
  const int64_t clusters = ngroups * d.batch;
  for (int p = need + 1; p <= 8 && p <= nblk; ++p) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = make_cfg(p, attr);
    int num = 0;
    if (cudaOccupancyMaxActiveClusters(&num, fn, &cfg) != cudaSuccess) { cudaGetLastError(); break; }
    if (num >= clusters) P = p;
  }
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = make_cfg(P, attr);
  const int ln = (int)((nblk + P - 1) / P * 32);
  lc.pre(st);
  if (adjoint) cudaLaunchKernelEx(&cfg, solve_cluster_kernel<T, true>, d, LU, ipiv, X, nrhs, xstride, g, ln, 0);
  else cudaLaunchKernelEx(&cfg, solve_cluster_kernel<T, false>, d, LU, ipiv, X, nrhs, xstride, g, ln, (int)upper_only);
  lc.post(st, sizeof(T) == 8 ? "lu_solve_f64" : "lu_solve_f32");
  return true;
}

template <typename T>
void lu_solve_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const typename cplx_t<T>::type* LU,
                      const int32_t* ipiv, typename cplx_t<T>::type* X, int64_t nrhs, int64_t xstride,
                      bool adjoint, bool upper_only) {
  using C = typename cplx_t<T>::type;
  const int64_t n = d.n;
  if (n <= 0 || nrhs <= 0 || d.batch <= 0) return;
  upper_only = upper_only && !adjoint;
  if (solve_on_cluster<T>(st, lc, d, LU, ipiv, X, nrhs, xstride, adjoint, upper_only)) return;
  const size_t max_smem = 200 * 1024;
  const size_t blk_bytes = sizeof(C) * 32 * 33;
  int64_t group = (int64_t)((max_smem - blk_bytes) / (sizeof(C) * n));
  // Enough CTAs to occupy every SM twice: each CTA streams the factor once for
  // its group of right-hand sides, so fewer RHS per CTA trades factor re-reads
  // (from L2 / HBM) for parallelism.
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want_ctas = 2 * (int64_t)sms;
  const int64_t g_par = (nrhs * d.batch + want_ctas - 1) / want_ctas;
  if (group > g_par) group = g_par;
  if (group < 1) group = 1;
  if (group > nrhs) group = nrhs;
  const size_t smem = blk_bytes + sizeof(C) * n * group;
  dim3 grid((unsigned)((nrhs + group - 1) / group), (unsigned)d.batch);
  lc.pre(st);
  if (adjoint) {
    cudaFuncSetAttribute(solve_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
    solve_kernel<T, true><<<grid, 512, smem, st>>>(d, LU, ipiv, X, nrhs, xstride, (int)group, 0);
  } else {
    cudaFuncSetAttribute(solve_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
    solve_kernel<T, false><<<grid, 512, smem, st>>>(d, LU, ipiv, X, nrhs, xstride, (int)group, (int)upper_only);
  }
  lc.post(st, sizeof(T) == 8 ? "lu_solve_f64" : "lu_solve_f32");
}

// Random complex matrices (entries uniform in [-1, 1] x [-1, 1] from a counter-based hash)
// on which the autotuner times factorizations; every column needs partial pivoting.
template <typename T>
__global__ void fill_random_kernel(BatchDesc d, typename cplx_t<T>::type* __restrict__ A, uint64_t seed) {
  const int64_t count = d.n * d.n;
  const int64_t b = blockIdx.y;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(b * count + q + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const T re = (T)((double)(z >> 40) * (2.0 / 16777216.0) - 1.0);
    const T im = (T)((double)(z & 0xFFFFFFull) * (2.0 / 16777216.0) - 1.0);
    A[b * d.stride + q] = cmk(re, im);
  }
}

template <typename T>
void fill_random_matrices(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, typename cplx_t<T>::type* A,
                          uint64_t seed) {
  if (d.n <= 0 || d.batch <= 0) return;
  const int64_t blocks = std::min<int64_t>((d.n * d.n + 255) / 256, 1216);
  MH_LAUNCH(lc, st, "fill_random",
            fill_random_kernel<T><<<dim3((unsigned)blocks, (unsigned)d.batch), 256, 0, st>>>(d, A, seed));
}
template void fill_random_matrices<double>(cudaStream_t, LaunchCounter, const BatchDesc&, double2*, uint64_t);
template void fill_random_matrices<float>(cudaStream_t, LaunchCounter, const BatchDesc&, float2*, uint64_t);

template int lu_factor_batched<double>(cudaStream_t, LaunchCounter, const BatchDesc&, double2*, int32_t*, int32_t*,
                                       void*, int*);
template int lu_factor_batched<float>(cudaStream_t, LaunchCounter, const BatchDesc&, float2*, int32_t*, int32_t*,
                                      void*, int*);
template void lu_solve_batched<double>(cudaStream_t, LaunchCounter, const BatchDesc&, const double2*,
                                       const int32_t*, double2*, int64_t, int64_t, bool, bool);
template void lu_solve_batched<float>(cudaStream_t, LaunchCounter, const BatchDesc&, const float2*, const int32_t*,
                                      float2*, int64_t, int64_t, bool, bool);

size_t zgemm_work_elems(int64_t n, int64_t nrhs, int64_t batch) {
  const size_t fp64 = (size_t)gemm_split(n, batch) * (size_t)batch * (size_t)nrhs * (size_t)n;
  const size_t tc = (tc_zgemv_workspace_bytes(n, batch) + sizeof(double2) - 1) / sizeof(double2);
  return fp64 > tc ? fp64 : tc;
}

void zgemm_nn_tc_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                         int64_t nrhs, int64_t xstride, double2* Y, double2* work, int* timeout_flag) {
  tc_zgemv(st, lc, d, A, X, nrhs, xstride, Y, nullptr, work, timeout_flag);
}

void residual_tc_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                         const double2* B, int64_t nrhs, int64_t xstride, double2* R, double2* work,
                         int* timeout_flag) {
  tc_zgemv(st, lc, d, A, X, nrhs, xstride, R, B, work, timeout_flag);
}

static void zgemm_impl(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                       int64_t nrhs, int64_t xstride, double2* Y, double2* work, const double2* B, bool adjoint) {
  const int64_t n = d.n;
  if (n <= 0 || nrhs <= 0 || d.batch <= 0) return;
  const int64_t ns = gemm_split(n, d.batch);
  const int64_t jchunk = (n + ns - 1) / ns;
  dim3 grid((unsigned)((n + kGemvRows - 1) / kGemvRows), (unsigned)ns, (unsigned)d.batch);
  for (int r0 = 0; r0 < nrhs; r0 += kGemvNR) {
    lc.pre(st);
    if (adjoint) zgemm_partial_kernel<true><<<grid, kGemvRows, 0, st>>>(d, A, X, nrhs, xstride, jchunk, r0, work);
    else zgemm_partial_kernel<false><<<grid, kGemvRows, 0, st>>>(d, A, X, nrhs, xstride, jchunk, r0, work);
    lc.post(st, "zgemm_rhs");
  }
  const int64_t tot = nrhs * n * d.batch;
  MH_LAUNCH(lc, st, "zgemm_rhs_reduce",
            zgemm_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(d, nrhs, ns, work, Y, xstride, B,
                                                                                B != nullptr));
}

void zgemm_nn_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                      int64_t nrhs, int64_t xstride, double2* Y, double2* work) {
  zgemm_impl(st, lc, d, A, X, nrhs, xstride, Y, work, nullptr, false);
}

void zgemm_adj_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                       int64_t nrhs, int64_t xstride, double2* Y, double2* work) {
  zgemm_impl(st, lc, d, A, X, nrhs, xstride, Y, work, nullptr, true);
}

void residual_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                      const double2* B, int64_t nrhs, int64_t xstride, double2* R, double2* work, bool adjoint) {
  zgemm_impl(st, lc, d, A, X, nrhs, xstride, R, work, B, adjoint);
}

void convert_z_to_c(cudaStream_t st, LaunchCounter lc, const double2* src, float2* dst, int64_t count) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "convert", z_to_c_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(src, dst, count));
}


void ir_update(cudaStream_t st, LaunchCounter lc, int64_t count, double2* X, const float2* Cc) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "ir_update", ir_update_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(X, Cc, count));
}

void widen_c_to_z(cudaStream_t st, LaunchCounter lc, const float2* src, double2* dst, int64_t count) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "convert", c_to_z_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(src, dst, count));
}

void inf_norms_batched(cudaStream_t st, LaunchCounter lc, int64_t n, int64_t ncols, const double2* X, double* out) {
  if (ncols <= 0) return;
  MH_LAUNCH(lc, st, "ir_norms", col_inf_norm_kernel<<<(unsigned)ncols, 256, 0, st>>>(n, X, out));
}


}  // namespace mh
