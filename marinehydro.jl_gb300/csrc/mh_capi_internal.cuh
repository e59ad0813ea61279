// mh_capi_internal.cuh -- the state and helpers that the C-ABI translation units share
// (mh_capi.cu: contexts, meshes, assembly, solves, the sweep; mh_capi_batch.cu: the
// many-body graph; mh_capi_diff.cu: derivatives; mh_capi_tuning.cu: the launch-shape
// table and autotuner; mh_capi_surrogate.cu: the learned wave term).  Not part of the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "mh_internal.cuh"
#include "mh_mlp.cuh"

using namespace mh;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};


struct BodyPlan {
  mh_mesh* m = nullptr;
  int64_t n = 0, nw = 0, w_off = 0, out_off = 0;
  int64_t m0 = 0;                 // index of the body's first matrix in the grouped factorization
  int cls = 0;                    // its size class
  int stream = 0;
  double cost = 0.0;
  double *SR = nullptr, *DR = nullptr, *params = nullptr, *dofs = nullptr, *norms = nullptr;
  double2 *S = nullptr, *D = nullptr, *B = nullptr, *X = nullptr, *B0 = nullptr, *R = nullptr, *work = nullptr;
  double2 *F = nullptr, *FK = nullptr;
  float2 *LU32 = nullptr, *X32 = nullptr;
  int32_t *ipiv = nullptr, *info = nullptr;
  void* oz = nullptr;       // tensor-core update workspace (FP64_TC: Ozaki digits; MIXED: BF16 terms)
  int* ozflag = nullptr;    // its timeout flag
  int4* fb_list = nullptr;  // learned surrogate: pairs queued for the exact kernel
  unsigned long long* fb_state = nullptr;  // queue count, overflow and timeout flags
  int64_t fb_cap = 0;
  double* judge = nullptr;   // surrogate judge sums, 2 per frequency (device)
  double* hjudge = nullptr;  // and their pinned copy
  double2 *hF = nullptr, *hFK = nullptr;
  int32_t* hinfo = nullptr;
  double *hnorms = nullptr, *hparams = nullptr, *hdofs = nullptr;
  size_t nparams = 0;
};

struct BatchCache {
  std::vector<double> key;
  std::vector<BodyPlan> bodies;
  void* arena = nullptr;
  char* pinned = nullptr;
  // The grouped factorization: every body's matrices (M in all, stored body after body; the
  // bodies' D, X, LU32, X32 point into these arrays) factored and solved together per size
  // class (bodies whose orders lie within a factor of two), one launch per kernel and panel
  // step for the whole class.
  struct SizeClass {
    int64_t m_start = 0, count = 0, n_max = 0;
    int stream = 0;
    std::vector<int64_t> bodies;
    void* oz = nullptr;      // tensor-core update workspace of the class
    int* ozflag = nullptr;
  };
  std::vector<SizeClass> classes;
  int64_t M = 0, n_max = 0;
  double2 *D_all = nullptr, *X_all = nullptr;
  float2 *LU32_all = nullptr, *X32_all = nullptr;
  int32_t *ipiv_all = nullptr, *info_all = nullptr, *hinfo_all = nullptr;
  int64_t *orders = nullptr, *offsets = nullptr, *xoffsets = nullptr;  // device
  std::vector<int64_t> h_orders, h_offsets, h_xoffsets;
  double *anorm_all = nullptr, *hanorm_all = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_kernels = 0;
  std::vector<int64_t> order;  // bodies, longest first
  int device = 0;
  ~BatchCache() {
    cudaSetDevice(device);
    if (exec) cudaGraphExecDestroy(exec);
    if (arena) cudaFree(arena);
    if (pinned) cudaFreeHost(pinned);
  }
};

struct mh_context {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  std::string err;
  double quad_rtol = 1e-12, quad_atol = 1e-14;
  std::vector<DevBuf> ws;  // workspace slots, grown on demand
  double* pinned = nullptr;  // small pinned staging buffer for scalars / norms
  size_t pinned_bytes = 0;
  Profiler* prof = nullptr;
  std::vector<cudaStream_t> side;  // extra streams of the many-body batch schedule
  BatchCache* batch = nullptr;
  float* mlp = nullptr;  // learned surrogate parameters (BF16-rounded), device
  // the exact term's check of surrogate results (mh_surrogate_set_judge): pairs sampled per
  // matrix (0: off), stream seed, tolerance on the sampled relative error; the estimates and
  // re-run flags of the last surrogate sweep or batch, one per frequency-solve
  int64_t judge_samples = 0;
  uint64_t judge_seed = 0;
  double judge_tol = 0.0;
  std::vector<double> judge_err;
  std::vector<int32_t> judge_rerun;
  TileTable tiles;       // launch shapes of the batched LU per matrix-order bucket (mh_autotune)
  LaunchCounter lc() { return LaunchCounter{&launches, prof, &tiles}; }
};

struct mh_mesh {
  mh_context* ctx = nullptr;
  int64_t n = 0;
  int64_t n_hull = 0;   // panels n_hull..n-1 are an irregular-frequency lid (mh_mesh_set_lid)
  double* V = nullptr;  // n x 12
  double* C = nullptr;  // n x 3
  double* N = nullptr;  // n x 3
  double* A = nullptr;  // n
  double* R = nullptr;  // n
  PanelRec* P = nullptr;
  // cached wavenumber-independent part
  double* SR = nullptr;
  double* DR = nullptr;
  bool st_valid = false;
  uint32_t st_gfs = 0;
  int st_direct = 0, st_ident = 0, st_has_fixed = 0;
  double st_fixed[3] = {0, 0, 0};
};

namespace mh {
namespace capi {

// One NVTX range per C-ABI call, so that timeline tools and ncu's --nvtx filters see the
// library's phases (assembly, solves, sweeps) by name.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

enum Slot {
  kSlotS = 0, kSlotD, kSlotSR, kSlotDR, kSlotB, kSlotX, kSlotWork, kSlotIpiv, kSlotInfo, kSlotLU32, kSlotX32,
  kSlotR, kSlotSmall, kSlotF, kSlotFK, kSlotDofs, kSlotIdx, kSlotNorm, kSlotA64, kSlotIn, kSlotRS, kSlotRD,
  kSlotGrad, kSlotLam, kSlotT, kSlotFb, kSlotFbState, kSlotOzaki, kSlotBx3, kSlotTcFlag, kSlotAnorm, kSlotCw,
  kSlotY, kSlotEgd, kSlotJudge, kSlotCount
};

int fail(mh_context* ctx, int code, const char* fmt, ...);

#define MH_CUDA(ctx, call)                                                                       \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return fail((ctx), e_ == cudaErrorMemoryAllocation ? MH_ERR_NOMEM : MH_ERR_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                            \
  } while (0)

#define MH_TRY(x)            \
  do {                       \
    int rc_ = (x);           \
    if (rc_ != MH_OK) return rc_; \
  } while (0)

int ws_get(mh_context* ctx, int slot, size_t bytes, void** out);

template <typename P>
int ws_get_t(mh_context* ctx, int slot, size_t count, P** out) {
  void* v = nullptr;
  MH_TRY(ws_get(ctx, slot, std::max<size_t>(count, 1) * sizeof(P), &v));
  *out = static_cast<P*>(v);
  return MH_OK;
}

int pinned_get(mh_context* ctx, size_t bytes, double** out);
int set_device(mh_context* ctx);
int check_launch(mh_context* ctx, const char* what);
int sync(mh_context* ctx, const char* what);
int copy_in(mh_context* ctx, void* dst, const void* src, size_t bytes, int mem);
int copy_out(mh_context* ctx, void* dst, const void* src, size_t bytes, int mem);
int put_out(mh_context* ctx, void* dst, const void* src_host, size_t bytes, int mem);
AssemblyParams make_params(mh_context* ctx, const mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                           const double* fixed);
int check_gfs(mh_context* ctx, uint32_t gfs);
int prepare_surrogate(mh_context* ctx, AssemblyParams& p, int64_t nk);
int check_surrogate(mh_context* ctx, const AssemblyParams& p);
int compute_static(mh_context* ctx, const mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                   const double* fixed, double* SR, double* DR);
int ensure_static_cache(mh_context* ctx, mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                        const double* fixed);
int factor_mixed(mh_context* ctx, const BatchDesc& d, const double2* Adev, float2** LU32_out, double** anrm_out);
int refine_mixed(mh_context* ctx, const BatchDesc& d, const double2* Adev, const float2* LU32, const double* anrm,
                 double2* X, int64_t nrhs, int64_t xstride, bool adjoint, bool* converged, double2** B0_out);
int check_pivots(mh_context* ctx, const BatchDesc& d, int64_t first_index);
int solve_core(mh_context* ctx, const BatchDesc& d, double2* Adev, double2* X, int64_t nrhs, int64_t xstride,
               int precision, bool adjoint);

// The substitution kernel keeps one right-hand side (n complex doubles) plus a
// 32 x 33 block in shared memory (<= 227 KB per CTA).
constexpr int64_t kMaxOrder = 12000;

constexpr uint32_t kStaticKinds = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE |
                                  MH_GF_DELHOMMEAU_RANKINE | MH_GF_DELHOMMEAU_RANKINE_REFLECTED;
constexpr uint32_t kWaveKinds = MH_GF_WU | MH_GF_EXACT_DELHOMMEAU | MH_GF_SURROGATE;
constexpr uint32_t kAllKinds = kStaticKinds | kWaveKinds;

}  // namespace capi
}  // namespace mh

using namespace mh::capi;
