// mh_internal.cuh -- shared declarations of libmarinehydro_cuda.so (not part of the C-ABI).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/marinehydro_gb300.h"

namespace mh {

// ---------------------------------------------------------------------------
// constants (values as Julia evaluates them in the reference)
// ---------------------------------------------------------------------------
constexpr double kPi = 3.141592653589793;
constexpr double kFourPi = 12.566370614359172;        // 4pi
constexpr double kMinusInv4Pi = -0.07957747154594767;  // -1/4pi

// Per-panel record staged in shared memory by the assembly kernels (32 doubles,
// 256 B, 16-byte aligned so it moves with double2 loads).
struct __align__(16) PanelRec {
  double T[9];      // Birk local frame, column-major (s, t, n)      rankine_vectorized.jl:80-89
  double qgc[3];    // Birk area centroid                             :118-122
  double lc[8];     // local corners (x, y) relative to qgc           :125-127
  double c[3];      // mesh center (element center)                   meshes.jl:42-51
  double n[3];      // mesh normal
  double area;      // mesh area
  double radius;    // mesh radius
  double edge[4];   // lengths of the local edges, corner k to corner k+1 (Birk integral)
};
static_assert(sizeof(PanelRec) == 256, "PanelRec layout");

// ---------------------------------------------------------------------------
// complex helpers (interleaved re, im)
// ---------------------------------------------------------------------------
template <typename T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };

__host__ __device__ inline double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline float2 cmk(float r, float i) { return make_float2(r, i); }

// ---------------------------------------------------------------------------
// host-side kernel launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
// Counts kernel launches and, when profiling is on, brackets each launch with a
// pair of CUDA events attributed to a named kernel group (see mh_profile_*).
struct Profiler;

// Launch shapes of the batched LU that depend on the matrix order, chosen per order
// bucket by mh_autotune (or set with mh_tile_table_set).  The defaults are the
// hand-picked shapes the table starts from.
struct TileChoice {
  int oz_group = 8;     // reserved: the Ozaki (FP64 tensor-core) update is a persistent kernel
  int bx_group = 4;     // 128-column tiles per CTA of the BF16x3 (FP32) update, 1..8
  int cluster_f64 = 8;  // largest thread-block cluster of the FP64 LU panel, 1..8
  int cluster_f32 = 8;  // largest thread-block cluster of the FP32 LU panel, 1..8
};
constexpr int kMaxTileEntries = 16;
struct TileTable {
  int n_entries = 0;                  // 0: defaults for every order
  int64_t n_max[kMaxTileEntries];     // ascending bucket bounds (inclusive); the last covers the rest
  TileChoice c[kMaxTileEntries];
  TileChoice lookup(int64_t n) const {
    for (int q = 0; q < n_entries; ++q)
      if (n <= n_max[q] || q == n_entries - 1) return c[q];
    return TileChoice{};
  }
};

struct LaunchCounter {
  int64_t* count;
  Profiler* prof;
  const TileTable* tiles = nullptr;
  void pre(cudaStream_t st) const;
  void post(cudaStream_t st, const char* group) const;
  TileChoice tile(int64_t n) const { return tiles ? tiles->lookup(n) : TileChoice{}; }
};

#define MH_LAUNCH(lc, st, group, ...) \
  do {                                \
    (lc).pre(st);                     \
    __VA_ARGS__;                      \
    (lc).post((st), (group));         \
  } while (0)

// assembly (mh_assembly.cu)
void launch_panel_geometry(cudaStream_t st, LaunchCounter lc, int64_t n, const double* V, const double* C,
                           const double* N, const double* A, const double* R, PanelRec* out);
// loads panel_geometry_kernel's module on the current device now (lazy loading would do it
// at the first launch)
cudaError_t load_panel_geometry_kernel();

struct AssemblyParams {
  int64_t n;
  const PanelRec* P;
  const double* V;        // n x 12 raw vertices (Delhommeau Rankine near field)
  uint32_t gfs;
  int direct;
  int include_identity;
  int has_fixed;
  double fixed[3];
  double k;
  double quad_rtol, quad_atol;
  // learned surrogate (MH_GF_SURROGATE): packed BF16-rounded MLP parameters, and the list
  // of pairs outside its training box that the exact kernel recomputes
  const float* mlp;
  int4* fb_list;                 // (i, j, wavenumber index, 0), i <= j
  unsigned long long* fb_state;  // [0] entries appended by the current launch, [1] sticky overflow,
                                 // [2] sticky tensor-core wait timeout
  int64_t fb_cap;
};

// Static (wavenumber-independent) part into real n x n arrays SR, DR (identity included when asked).
void launch_assemble_static(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double* SR, double* DR);
// S = SR + S_wave(k), D = DR + D_wave(k) (complex); SR/DR may be null (no static part).
// batch: `nk` wavenumbers ks[b], output b at S + b*sstride (complex elements).
void launch_assemble_wave(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* SR,
                          const double* DR, int nk, const double* ks_dev, double2* S, double2* D, int64_t sstride,
                          int wave_identity);
// The exact term's check of surrogate-assembled matrices: n_samples pairs per matrix drawn from
// (seed, first_matrix + b, sample); acc[2 b] += sum |assembled - exact|^2 over S and D entries,
// acc[2 b + 1] += sum |assembled|^2 (acc zeroed by the caller)
void launch_surrogate_judge(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* SR,
                            const double* DR, int nk, const double* ks_dev, const double2* S, const double2* D,
                            int64_t sstride, int64_t n_samples, uint64_t seed, int64_t first_matrix,
                            int wave_identity, double* acc);
// learned surrogate (mh_surrogate.cu)
void launch_surrogate_points(cudaStream_t st, LaunchCounter lc, const float* mlp, int64_t m, const double* r,
                             const double* z, double rtol, double atol, double2* out);
// training samples [offset, offset + count) of the M samples of `seed`: inputs X (u, v),
// scaled targets Y8 (8 floats per sample, 6 used), optionally (r, z) in FP64 into R2
void launch_surrogate_samples(cudaStream_t st, LaunchCounter lc, uint64_t seed, int64_t M, int64_t offset,
                              int64_t count, double rtol, double atol, float2* X, float* Y8, double* R2);
// floats of the per-step activation buffer for a batch of B samples
int64_t mlp_act_floats(int B);
// one Adam step (t >= 1) over samples ((base + b) mod M) * prime mod M, b < B; the mean
// squared error of the batch is added to *loss
void launch_mlp_train_step(cudaStream_t st, LaunchCounter lc, float* theta, float* qparams, float* grad, float* m1,
                           float* m2, const float2* X, const float* Y8, int64_t M, int64_t base, int64_t prime, int B,
                           float* acts, double* loss, float lr, int t);
// mean squared error into *loss and its gradient into grad (accumulated) for the BF16
// parameters qparams over samples ((base + b) mod M) * prime mod M, b < B
void launch_mlp_loss_grad(cudaStream_t st, LaunchCounter lc, const float* qparams, const float2* X, const float* Y8,
                          int64_t M, int64_t base, int64_t prime, int B, float* acts, double* loss, float* grad);
// out = BF16-rounded copy of the packed parameters (padding zeroed)
void launch_round_bf16(cudaStream_t st, LaunchCounter lc, const float* in, float* out);
// point evaluators
void launch_wu_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* hh, const double* vv, double2* out);
// J0, J1, Y0, Y1 (NaN for Y below x = 3) at m points: out 4 doubles per point
void launch_bessel01_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* x, double* out);
// exp(-|x|), log|x|, 1/|x|, sqrt|x| as the Wu term evaluates them on the integer pipe (mh_fixpoint.cuh)
void launch_fixpoint_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* x, double* out);
void launch_exact_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* r, const double* z, double rtol,
                         double atol, double2* out);

// dense linear algebra (mh_lu.cu)
struct BatchDesc {
  int64_t n;        // order (a grouped batch: the largest order)
  int64_t batch;    // number of matrices
  int64_t stride;   // complex elements between matrices (uniform batches)
  // A grouped batch holds matrices of different orders (the many-body batch factors every
  // body's matrices in one launch per panel step): device arrays of each matrix's order,
  // the element offset of the matrix and of its block of right-hand sides.  Null for a
  // uniform batch.  Pivot indices keep the stride n per matrix either way.
  const int64_t* orders = nullptr;
  const int64_t* offsets = nullptr;
  const int64_t* xoffsets = nullptr;
  // Columns stored after each matrix's n columns (same leading dimension n) that the
  // factorization carries along: right-hand sides appended to the matrix receive the row
  // interchanges and the elimination, so that after lu_factor_batched they hold L^-1 P b and
  // only the upper triangular solve remains.  Uniform batches with the tensor-core FP64
  // update only (the trailing update is rectangular, n - k - kb rows by n + extra - k - kb
  // columns); 0 otherwise.
  int64_t extra = 0;
  __device__ __forceinline__ int64_t order(int64_t b) const { return orders ? orders[b] : n; }
  __device__ __forceinline__ int64_t offset(int64_t b) const { return offsets ? offsets[b] : b * stride; }
  __device__ __forceinline__ int64_t xoffset(int64_t b, int64_t xstride) const {
    return xoffsets ? xoffsets[b] : b * xstride;
  }
};
template <typename T>
int lu_factor_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, typename cplx_t<T>::type* A,
                      int32_t* ipiv, int32_t* info, void* emu_ws = nullptr, int* emu_flag = nullptr);
// d.batch random complex matrices for timing factorizations (mh_autotune)
template <typename T>
void fill_random_matrices(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, typename cplx_t<T>::type* A,
                          uint64_t seed);
// FP64 trailing update A22 -= L21 U12 of panel step k on the BF16 tensor cores (mh_ozaki.cu);
// emu_ws: ozaki_workspace_bytes(n, batch) bytes; *timeout_flag set if a completion wait gave up
size_t ozaki_workspace_bytes(int64_t n, int64_t batch, int64_t extra = 0);
// FP32 trailing update of the mixed-precision factors on the BF16 tensor cores, three-way
// split (mh_bf16x3.cu); ws: bx3_workspace_bytes(n, batch) bytes
size_t bx3_workspace_bytes(int64_t n, int64_t batch);
void bx3_trailing_update(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, float2* A, int64_t k, int kb,
                         void* ws, int* timeout_flag);
// kb: the panel's width (32; 16 for the update inside a two-level panel), cols: at most this
// many columns right of the panel are updated
void ozaki_trailing_update(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, double2* A, int64_t k, int kb,
                           void* ws, int* timeout_flag, int64_t cols = INT64_MAX);
// U12 = L11^-1 A12 of panel step k (a full 32-column panel) as an exact-digit product on the
// tensor cores (mh_ozaki.cu); same workspace as the trailing update
void ozaki_trsm(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, double2* A, int64_t k, void* ws,
                int* timeout_flag);
// upper_only: X already holds L^-1 P b (right-hand sides carried through the factorization,
// BatchDesc::extra): only U x = y is solved, without the interchanges
template <typename T>
void lu_solve_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const typename cplx_t<T>::type* LU,
                      const int32_t* ipiv, typename cplx_t<T>::type* X, int64_t nrhs, int64_t xstride,
                      bool adjoint, bool upper_only = false);
// Y_b = A_b X_b (n x n times n x nrhs), batched, FP64; partial sums in `work`
void zgemm_nn_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                      int64_t nrhs, int64_t xstride, double2* Y, double2* work);
size_t zgemm_work_elems(int64_t n, int64_t nrhs, int64_t batch);
// Y_b = A_b^H X_b
void zgemm_adj_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                       int64_t nrhs, int64_t xstride, double2* Y, double2* work);
void convert_z_to_c(cudaStream_t st, LaunchCounter lc, const double2* src, float2* dst, int64_t count);
// R = B - A X (FP64), then C = (float) R ; returns nothing, norms into `norms` (per rhs: |R|_inf, |X|_inf)
void residual_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                      const double2* B, int64_t nrhs, int64_t xstride, double2* R, double2* work, bool adjoint);
// The same products on the BF16 tensor cores, FP64-accurate (mh_zgemv_tc.cu); A X only (no
// adjoint), `work` as for zgemm_nn_batched; *timeout_flag set if a completion wait gave up.
size_t tc_zgemv_workspace_bytes(int64_t n, int64_t batch);
void tc_zgemv(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
              int64_t nrhs, int64_t xstride, double2* Y, const double2* B, void* ws, int* timeout_flag);
void zgemm_nn_tc_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                         int64_t nrhs, int64_t xstride, double2* Y, double2* work, int* timeout_flag);
void residual_tc_batched(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, const double2* X,
                         const double2* B, int64_t nrhs, int64_t xstride, double2* R, double2* work,
                         int* timeout_flag);
void ir_update(cudaStream_t st, LaunchCounter lc, int64_t count, double2* X, const float2* C);
void widen_c_to_z(cudaStream_t st, LaunchCounter lc, const float2* src, double2* dst, int64_t count);
// FP32 copy of each matrix (matrix stride stride32) and its |.|_inf norm into out[b], one pass over A
void convert_with_norms(cudaStream_t st, LaunchCounter lc, const BatchDesc& d, const double2* A, float2* A32,
                        int64_t stride32, double* out);
void inf_norms_batched(cudaStream_t st, LaunchCounter lc, int64_t n, int64_t ncols, const double2* X,
                       double* out);

// epilogue (mh_epilogue.cu)
struct EpilogueGeom {
  int64_t n;
  int64_t n_hull;    // panels n_hull..n-1 form a lid: zero boundary condition, no pressure in the forces
  const double* C;   // centers n x 3
  const double* N;   // normals n x 3
  const double* A;   // areas
  const double* dofs;  // n_dofs x n x 3
};
void launch_build_rhs(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                      double gacc, int n_rad, const int32_t* rad_idx_dev, int n_beta, const double* betas_dev,
                      double2* Bmat, int64_t bstride);
void launch_forces(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                   double rho, double gacc, int nrhs, const double2* Phi, int64_t pstride, int n_inf,
                   const int32_t* inf_idx_dev, int n_beta, const double* betas_dev, double2* F /*nw x n_inf x nrhs*/,
                   double2* FK /*nw x n_inf x n_beta*/);

// adjoint (mh_adjoint.cu)
void launch_static_adjoint(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* RS,
                           const double* RD, double* gc, double* gn, double* ga, double* gv);
// weights W^S = c lS rS^T, W^D = -c lD rD^T (n x nh each); egd_values: the packed exact
// values of launch_egd_pair_values at k when p.gfs holds MH_GF_EXACT_DELHOMMEAU
void launch_wave_adjoint(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, const double2* lS,
                         const double2* rS, const double2* lD, const double2* rD, int nh, double2 c,
                         const double2* egd_values, double* gc, double* gn, double* ga, double* RS, double* RD);
// G and dG/dr of the exact term for the egd_packed_pairs(n) unordered pairs at wavenumber k
// (2 complex values per pair, pair (i <= j) at index j (j + 1)/2 + i)
int64_t egd_packed_pairs(int64_t n);
void launch_egd_pair_values(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, double2* out);
// dS/dk, dD/dk of the exact wave part from those values (n x n complex, no static part)
void launch_egd_dk(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double k, const double2* values,
                   double2* dS, double2* dD);
// out = alpha U V^H for n x nh complex U, V (an n x n complex matrix)
void launch_outer_adj(cudaStream_t st, LaunchCounter lc, int64_t n, int nh, const double2* U, const double2* V,
                      double alpha, double2* out);
// cw: n_inf x n_rad complex cotangent factors c[q, r] of one frequency (device);
// gd: n_dofs x n x 3, indexed by the dof indices in rad / inf
// (cw: n_inf x (n_rad + n_beta); the heading columns follow the radiating ones)
void launch_rhs_adjoint(cudaStream_t st, LaunchCounter lc, int64_t n, const double* N, const double* A,
                        const double* C, const double* dofs, const int32_t* rad, int n_rad, const int32_t* inf,
                        int n_inf, int n_beta, const double* betas, double omega, double rho, double gacc,
                        const double2* cw, const double2* phi, const double2* t, double* gc, double* gn, double* ga,
                        double* gd);
void launch_force_weights(cudaStream_t st, LaunchCounter lc, int64_t n, const double* N, const double* A,
                          const double* dofs, const int32_t* inf, int n_inf, int n_rad, const double2* cw,
                          double omega, double rho, double2* wconj);
void launch_conj(cudaStream_t st, LaunchCounter lc, int64_t count, double2* x);
// dS/dk, dD/dk of the Wu wave part at the wavenumber *k_dev (n x n complex, no static part)
void launch_wave_dk(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* k_dev, double2* dS,
                    double2* dD);
// d(boundary conditions)/d omega of launch_build_rhs, same layout
void launch_build_drhs(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                       double gacc, int n_rad, const int32_t* rad_idx_dev, int n_beta, const double* betas_dev,
                       double2* dB, int64_t bstride);
// y += alpha x (complex vectors of `count` entries, real alpha)
void launch_zaxpy(cudaStream_t st, LaunchCounter lc, int64_t count, double alpha, const double2* x, double2* y);

// profiling (mh_profile.cu)
Profiler* profiler_create();
void profiler_destroy(Profiler* p);
void profiler_enable(Profiler* p, bool on);
bool profiler_on(const Profiler* p);
void profiler_reset(Profiler* p);
int profiler_read(Profiler* p, int64_t capacity, char* names, double* total_ms, int64_t* launches, int64_t* n);
int probe_fma_peaks(cudaStream_t st, double* fp64_tflops, double* fp32_tflops);
// one bounded mbarrier wait that nothing satisfies (the timeout path of the tensor-core kernels)
int probe_wait_timeout(cudaStream_t st, uint32_t polls, int* timed_out);

// misc
void launch_combine_real_to_complex(cudaStream_t st, LaunchCounter lc, int64_t count, const double* re,
                                    double2* out);

}  // namespace mh
