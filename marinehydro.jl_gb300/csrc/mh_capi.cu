// mh_capi.cu -- the C-ABI of libmarinehydro_cuda.so (declared in include/marinehydro_gb300.h).
//
// Owns the contexts (device, stream, workspaces, launch counter, last error) and
// mesh handles (device copies of one body's panels, the per-panel Birk frames and
// the cached wavenumber-independent matrices), and orchestrates the kernels of
// mh_assembly.cu, mh_lu.cu and mh_epilogue.cu.
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

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct BodyPlan {
  mh_mesh* m = nullptr;
  int64_t n = 0, nw = 0, w_off = 0, out_off = 0;
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

namespace {

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
  kSlotCount
};

int fail(mh_context* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

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

int ws_get(mh_context* ctx, int slot, size_t bytes, void** out) {
  if ((int)ctx->ws.size() < kSlotCount) ctx->ws.resize(kSlotCount);
  DevBuf& b = ctx->ws[slot];
  if (b.bytes < bytes) {
    if (b.p) MH_CUDA(ctx, cudaFreeAsync(b.p, ctx->stream));
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes + bytes / 8 + 256;
    MH_CUDA(ctx, cudaMallocAsync(&b.p, want, ctx->stream));
    b.bytes = want;
  }
  *out = b.p;
  return MH_OK;
}

template <typename P>
int ws_get_t(mh_context* ctx, int slot, size_t count, P** out) {
  void* v = nullptr;
  MH_TRY(ws_get(ctx, slot, std::max<size_t>(count, 1) * sizeof(P), &v));
  *out = static_cast<P*>(v);
  return MH_OK;
}

int pinned_get(mh_context* ctx, size_t bytes, double** out) {
  if (ctx->pinned_bytes < bytes) {
    if (ctx->pinned) {
      MH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaFreeHost(ctx->pinned);
    }
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    MH_CUDA(ctx, cudaMallocHost(&ctx->pinned, bytes));
    ctx->pinned_bytes = bytes;
  }
  *out = ctx->pinned;
  return MH_OK;
}

int set_device(mh_context* ctx) {
  MH_CUDA(ctx, cudaSetDevice(ctx->device));
  return MH_OK;
}

int check_launch(mh_context* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, MH_ERR_CUDA, "%s: kernel launch failed: %s", what, cudaGetErrorString(e));
  return MH_OK;
}

int sync(mh_context* ctx, const char* what) {
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(ctx, MH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return MH_OK;
}

// copy `bytes` from a caller buffer (host or device) into device memory `dst`
int copy_in(mh_context* ctx, void* dst, const void* src, size_t bytes, int mem) {
  if (bytes == 0) return MH_OK;
  MH_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, mem == MH_MEM_HOST ? cudaMemcpyHostToDevice
                                                                   : cudaMemcpyDeviceToDevice, ctx->stream));
  return MH_OK;
}

int copy_out(mh_context* ctx, void* dst, const void* src, size_t bytes, int mem) {
  if (!dst || bytes == 0) return MH_OK;  // NULL destination skips
  MH_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, mem == MH_MEM_HOST ? cudaMemcpyDeviceToHost
                                                                   : cudaMemcpyDeviceToDevice, ctx->stream));
  return MH_OK;
}

// host-side result -> caller buffer (host memcpy or H2D); NULL destination skips
int put_out(mh_context* ctx, void* dst, const void* src_host, size_t bytes, int mem) {
  if (!dst || bytes == 0) return MH_OK;
  if (mem == MH_MEM_HOST) {
    std::memcpy(dst, src_host, bytes);
    return MH_OK;
  }
  MH_CUDA(ctx, cudaMemcpyAsync(dst, src_host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return sync(ctx, "result upload");
}

// The substitution kernel keeps one right-hand side (n complex doubles) plus a
// 32 x 33 block in shared memory (<= 227 KB per CTA).
constexpr int64_t kMaxOrder = 12000;

constexpr uint32_t kStaticKinds = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE |
                                  MH_GF_DELHOMMEAU_RANKINE | MH_GF_DELHOMMEAU_RANKINE_REFLECTED;
constexpr uint32_t kWaveKinds = MH_GF_WU | MH_GF_EXACT_DELHOMMEAU | MH_GF_SURROGATE;
constexpr uint32_t kAllKinds = kStaticKinds | kWaveKinds;

AssemblyParams make_params(mh_context* ctx, const mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                           const double* fixed) {
  AssemblyParams p;
  p.n = m->n;
  p.P = m->P;
  p.V = m->V;
  p.gfs = gfs;
  p.direct = direct ? 1 : 0;
  p.include_identity = include_identity ? 1 : 0;
  p.has_fixed = fixed ? 1 : 0;
  for (int c = 0; c < 3; ++c) p.fixed[c] = fixed ? fixed[c] : 0.0;
  p.k = 0.0;
  p.quad_rtol = ctx->quad_rtol;
  p.quad_atol = ctx->quad_atol;
  p.mlp = nullptr;
  p.fb_list = nullptr;
  p.fb_state = nullptr;
  p.fb_cap = 0;
  return p;
}

// Green-function sets: at most one wave term; the learned surrogate needs its parameters
int check_gfs(mh_context* ctx, uint32_t gfs) {
  if (gfs == 0 || (gfs & ~kAllKinds)) return fail(ctx, MH_ERR_ARG, "bad Green-function set 0x%x", gfs);
  if ((gfs & MH_GF_SURROGATE) && (gfs & (MH_GF_WU | MH_GF_EXACT_DELHOMMEAU)))
    return fail(ctx, MH_ERR_ARG, "the learned surrogate replaces the wave term: do not combine it with GFWu or "
                                 "ExactGuevelDelhommeau");
  if ((gfs & MH_GF_SURROGATE) && !ctx->mlp)
    return fail(ctx, MH_ERR_ARG, "no surrogate parameters on this context (mh_surrogate_train / mh_surrogate_set)");
  return MH_OK;
}

// surrogate mode: parameters and the queue of pairs outside the training box
// (nk: wavenumbers per assembly launch; every launch queues its nk * n self pairs)
int prepare_surrogate(mh_context* ctx, AssemblyParams& p, int64_t nk) {
  if (!(p.gfs & MH_GF_SURROGATE)) return MH_OK;
  p.mlp = ctx->mlp;
  p.fb_cap = std::max<int64_t>((int64_t)1 << 20, p.n * (nk + 64));
  MH_TRY(ws_get_t(ctx, kSlotFb, (size_t)p.fb_cap, &p.fb_list));
  MH_TRY(ws_get_t(ctx, kSlotFbState, 4, &p.fb_state));
  MH_CUDA(ctx, cudaMemsetAsync(p.fb_state, 0, 4 * sizeof(unsigned long long), ctx->stream));
  return MH_OK;
}

// after a synchronisation: did any surrogate launch queue more pairs than the list holds?
int check_surrogate(mh_context* ctx, const AssemblyParams& p) {
  if (!(p.gfs & MH_GF_SURROGATE)) return MH_OK;
  unsigned long long st[3] = {0, 0, 0};
  MH_CUDA(ctx, cudaMemcpyAsync(st, p.fb_state, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  MH_TRY(sync(ctx, "surrogate state"));
  if (st[2])
    return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the surrogate assembly gave up");
  if (st[1])
    return fail(ctx, MH_ERR_UNSUPPORTED, "more than %lld panel pairs per launch lie outside the surrogate's training "
                                         "box; use ExactGuevelDelhommeau for this mesh", (long long)p.fb_cap);
  return MH_OK;
}

// Static part into (SR, DR); returns MH_OK
int compute_static(mh_context* ctx, const mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                   const double* fixed, double* SR, double* DR) {
  AssemblyParams p = make_params(ctx, m, gfs & kStaticKinds, direct, include_identity, fixed);
  launch_assemble_static(ctx->stream, ctx->lc(), p, SR, DR);
  return check_launch(ctx, "static assembly");
}

int ensure_static_cache(mh_context* ctx, mh_mesh* m, uint32_t gfs, int direct, int include_identity,
                        const double* fixed) {
  uint32_t st = gfs & kStaticKinds;
  bool same = m->st_valid && m->st_gfs == st && m->st_direct == (direct != 0) &&
              m->st_ident == (include_identity != 0) && m->st_has_fixed == (fixed != nullptr);
  if (same && fixed)
    same = m->st_fixed[0] == fixed[0] && m->st_fixed[1] == fixed[1] && m->st_fixed[2] == fixed[2];
  if (same) return MH_OK;
  const size_t nn = (size_t)m->n * (size_t)m->n;
  if (!m->SR) {
    MH_CUDA(ctx, cudaMallocAsync((void**)&m->SR, nn * sizeof(double), ctx->stream));
    MH_CUDA(ctx, cudaMallocAsync((void**)&m->DR, nn * sizeof(double), ctx->stream));
  }
  MH_TRY(compute_static(ctx, m, gfs, direct, include_identity, fixed, m->SR, m->DR));
  m->st_valid = true;
  m->st_gfs = st;
  m->st_direct = direct != 0;
  m->st_ident = include_identity != 0;
  m->st_has_fixed = fixed != nullptr;
  for (int c = 0; c < 3; ++c) m->st_fixed[c] = fixed ? fixed[c] : 0.0;
  return MH_OK;
}

// --- dense solve core on device arrays ------------------------------------------
// FP32 copy of the batch `Adev` (left intact for the FP64 residuals), factored in place;
// the matrices' |.|_inf norms (for the refinement's stopping test) come from the same pass.
int factor_mixed(mh_context* ctx, const BatchDesc& d, const double2* Adev, float2** LU32_out, double** anrm_out) {
  const int64_t n = d.n, nn = n * n;
  int32_t *ipiv, *info;
  float2* LU32;
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)(n * d.batch), &ipiv));
  MH_TRY(ws_get_t(ctx, kSlotInfo, (size_t)d.batch, &info));
  MH_TRY(ws_get_t(ctx, kSlotLU32, (size_t)(nn * d.batch), &LU32));
  double* anrm;
  MH_TRY(ws_get_t(ctx, kSlotAnorm, (size_t)d.batch, &anrm));
  BatchDesc d32 = d;
  d32.stride = nn;
  convert_with_norms(ctx->stream, ctx->lc(), d, Adev, LU32, nn, anrm);
  *anrm_out = anrm;
  // the trailing updates on the BF16 tensor cores (three-way split, FP32 accuracy)
  unsigned char* ws;
  const size_t wsb = bx3_workspace_bytes(n, d.batch);
  MH_TRY(ws_get_t(ctx, kSlotBx3, wsb + 256, &ws));
  int* flag = reinterpret_cast<int*>(ws + wsb);
  MH_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
  lu_factor_batched<float>(ctx->stream, ctx->lc(), d32, LU32, ipiv, info, ws, flag);
  MH_TRY(check_launch(ctx, "lu factor fp32"));
  int hflag = 0;
  MH_CUDA(ctx, cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MH_TRY(sync(ctx, "lu factor fp32"));
  if (hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  *LU32_out = LU32;
  return MH_OK;
}

// Solve A x = b (or A^H x = b) with the FP32 factors of factor_mixed and FP64 iterative
// refinement under LAPACK zcgesv's stopping rule: accept x when
// |b - A x|_inf <= sqrt(n) eps |A|_inf |x|_inf for every column, at most 30 sweeps.
// X holds b on entry and x on exit; *converged reports whether every column met the test
// (when it did not, X holds the last iterate and the caller falls back to FP64).
int refine_mixed(mh_context* ctx, const BatchDesc& d, const double2* Adev, const float2* LU32, const double* anrm,
                 double2* X, int64_t nrhs, int64_t xstride, bool adjoint, bool* converged, double2** B0_out) {
  const int64_t n = d.n, nn = n * n;
  int32_t* ipiv;
  float2* X32;
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)(n * d.batch), &ipiv));
  MH_TRY(ws_get_t(ctx, kSlotX32, (size_t)(xstride * d.batch), &X32));
  BatchDesc d32 = d;
  d32.stride = nn;
  double2 *B0, *R, *work;
  MH_TRY(ws_get_t(ctx, kSlotB, (size_t)(xstride * d.batch), &B0));
  MH_TRY(ws_get_t(ctx, kSlotR, (size_t)(xstride * d.batch), &R));
  MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, d.batch), &work));
  MH_CUDA(ctx, cudaMemcpyAsync(B0, X, sizeof(double2) * xstride * d.batch, cudaMemcpyDeviceToDevice, ctx->stream));
  if (B0_out) *B0_out = B0;
  // x0 = LU32 \ b
  convert_z_to_c(ctx->stream, ctx->lc(), B0, X32, xstride * d.batch);
  lu_solve_batched<float>(ctx->stream, ctx->lc(), d32, LU32, ipiv, X32, nrhs, xstride, adjoint);
  widen_c_to_z(ctx->stream, ctx->lc(), X32, X, xstride * d.batch);
  const int64_t ncols = nrhs * d.batch;
  double* norms;
  MH_TRY(ws_get_t(ctx, kSlotNorm, (size_t)(2 * ncols + d.batch), &norms));
  double* anrm_d = norms + 2 * ncols;
  MH_CUDA(ctx, cudaMemcpyAsync(anrm_d, anrm, sizeof(double) * d.batch, cudaMemcpyDeviceToDevice, ctx->stream));
  double* hn;
  MH_TRY(pinned_get(ctx, sizeof(double) * (2 * ncols + d.batch) + 64, &hn));
  int* tcflag;  // the FP64-accurate residuals run on the tensor cores (forward solves)
  MH_TRY(ws_get_t(ctx, kSlotTcFlag, 4, &tcflag));
  MH_CUDA(ctx, cudaMemsetAsync(tcflag, 0, sizeof(int), ctx->stream));
  const double cte = std::sqrt((double)n) * 2.220446049250313e-16;
  *converged = false;
  for (int it = 0; it <= 30; ++it) {
    if (adjoint) residual_batched(ctx->stream, ctx->lc(), d, Adev, X, B0, nrhs, xstride, R, work, true);
    else residual_tc_batched(ctx->stream, ctx->lc(), d, Adev, X, B0, nrhs, xstride, R, work, tcflag);
    for (int64_t b = 0; b < d.batch; ++b) {
      inf_norms_batched(ctx->stream, ctx->lc(), n, nrhs, R + b * xstride, norms + b * nrhs);
      inf_norms_batched(ctx->stream, ctx->lc(), n, nrhs, X + b * xstride, norms + ncols + b * nrhs);
    }
    MH_TRY(check_launch(ctx, "refinement"));
    MH_CUDA(ctx, cudaMemcpyAsync(hn, norms, sizeof(double) * (2 * ncols + d.batch), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    int* hflag = reinterpret_cast<int*>(hn + 2 * ncols + d.batch);
    MH_CUDA(ctx, cudaMemcpyAsync(hflag, tcflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MH_TRY(sync(ctx, "refinement norms"));
    if (*hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the refinement residual gave up");
    bool ok = true;
    for (int64_t c = 0; c < ncols && ok; ++c) {
      const double anrm = hn[2 * ncols + c / nrhs];
      const double rn = hn[c], xn = hn[ncols + c];
      if (!(rn <= cte * anrm * xn)) ok = false;  // also false for NaN
    }
    if (ok) { *converged = true; break; }
    if (it == 30) break;
    // c = LU32 \ r ; x += c
    convert_z_to_c(ctx->stream, ctx->lc(), R, X32, xstride * d.batch);
    lu_solve_batched<float>(ctx->stream, ctx->lc(), d32, LU32, ipiv, X32, nrhs, xstride, adjoint);
    ir_update(ctx->stream, ctx->lc(), xstride * d.batch, X, X32);
  }
  return MH_OK;
}

// Reads the per-matrix pivot status of the last factorization; MH_ERR_SINGULAR on a zero pivot.
int check_pivots(mh_context* ctx, const BatchDesc& d, int64_t first_index) {
  int32_t* info;
  MH_TRY(ws_get_t(ctx, kSlotInfo, (size_t)d.batch, &info));
  std::vector<int32_t> hinfo(d.batch);
  MH_CUDA(ctx, cudaMemcpyAsync(hinfo.data(), info, sizeof(int32_t) * d.batch, cudaMemcpyDeviceToHost, ctx->stream));
  MH_TRY(sync(ctx, "lu"));
  for (int64_t b = 0; b < d.batch; ++b)
    if (hinfo[b] != 0)
      return fail(ctx, MH_ERR_SINGULAR, "matrix %lld is singular: zero pivot in column %d",
                  (long long)(first_index + b), hinfo[b]);
  return MH_OK;
}

// Factor the batch of matrices `Adev` (overwritten with LU factors in FP64 mode)
// and solve for X (in/out: rhs on entry).  In mixed mode `Adev` is left intact
// (used for the FP64 residuals) and an FP32 copy is factored; when refinement does
// not converge, the FP64 factorization is used instead.
int solve_core(mh_context* ctx, const BatchDesc& d, double2* Adev, double2* X, int64_t nrhs, int64_t xstride,
               int precision, bool adjoint) {
  const int64_t n = d.n;
  int32_t *ipiv, *info;
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)(n * d.batch), &ipiv));
  MH_TRY(ws_get_t(ctx, kSlotInfo, (size_t)d.batch, &info));
  if (precision == MH_PREC_FP64) {
    lu_factor_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, info);
    MH_TRY(check_launch(ctx, "lu factor"));
    lu_solve_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, X, nrhs, xstride, adjoint);
    MH_TRY(check_launch(ctx, "lu solve"));
  } else if (precision == MH_PREC_FP64_TC) {
    unsigned char* ws;
    const size_t wsb = ozaki_workspace_bytes(n, d.batch);
    MH_TRY(ws_get_t(ctx, kSlotOzaki, wsb + 256, &ws));
    int* flag = reinterpret_cast<int*>(ws + wsb);
    MH_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
    lu_factor_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, info, ws, flag);
    MH_TRY(check_launch(ctx, "lu factor (tensor-core update)"));
    lu_solve_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, X, nrhs, xstride, adjoint);
    MH_TRY(check_launch(ctx, "lu solve"));
    int hflag = 0;
    MH_CUDA(ctx, cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MH_TRY(sync(ctx, "tensor-core update"));
    if (hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  } else {
    float2* LU32;
    double* anrm;
    MH_TRY(factor_mixed(ctx, d, Adev, &LU32, &anrm));
    bool converged = false;
    double2* B0 = nullptr;
    MH_TRY(refine_mixed(ctx, d, Adev, LU32, anrm, X, nrhs, xstride, adjoint, &converged, &B0));
    if (!converged) {
      // fall back to the FP64 factorization
      MH_CUDA(ctx, cudaMemcpyAsync(X, B0, sizeof(double2) * xstride * d.batch, cudaMemcpyDeviceToDevice, ctx->stream));
      lu_factor_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, info);
      lu_solve_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, X, nrhs, xstride, adjoint);
      MH_TRY(check_launch(ctx, "lu fp64 fallback"));
    }
  }
  return check_pivots(ctx, d, 0);
}

// ---------------------------------------------------------------------------
// Many-body batch: every body's sweep is enqueued without host synchronisation on
// one of several streams (longest-processing-time order), the whole schedule is
// captured into one CUDA graph, and the instantiated graph is cached for repeated
// calls with the same bodies and options.
// ---------------------------------------------------------------------------
struct BatchOpts {
  uint32_t gfs;
  int direct, precision, ir_sweeps;
  double rho, g;
  int64_t n_dofs, n_rad, n_inf, n_beta, nrhs;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Lay out (or size, when base == nullptr) the device buffers of one body.
size_t layout_body(BodyPlan& b, const BatchOpts& o, char* base) {
  const size_t n = (size_t)b.n, nw = (size_t)b.nw, nn = n * n, nx = n * (size_t)o.nrhs;
  const bool mixed = o.precision == MH_PREC_MIXED;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += align256(std::max<size_t>(bytes, 8));
    return p;
  };
  b.SR = (double*)take(nn * 8);
  b.DR = (double*)take(nn * 8);
  b.S = (double2*)take(nw * nn * 16);
  b.D = (double2*)take(nw * nn * 16);
  b.B = (double2*)take(nw * nx * 16);
  b.X = (double2*)take(nw * nx * 16);
  b.B0 = mixed ? (double2*)take(nw * nx * 16) : nullptr;
  b.R = mixed ? (double2*)take(nw * nx * 16) : nullptr;
  b.work = (double2*)take(zgemm_work_elems(b.n, o.nrhs, b.nw) * 16);
  b.LU32 = mixed ? (float2*)take(nw * nn * 8) : nullptr;
  b.X32 = mixed ? (float2*)take(nw * nx * 8) : nullptr;
  b.ipiv = (int32_t*)take(nw * n * 4);
  b.info = (int32_t*)take(nw * 4);
  b.norms = (double*)take((2 * (size_t)o.nrhs * nw + nw) * 8);
  if (o.precision == MH_PREC_FP64_TC) {
    b.oz = take(ozaki_workspace_bytes(b.n, b.nw));
    b.ozflag = (int*)take(64);
  } else if (mixed) {
    b.oz = take(bx3_workspace_bytes(b.n, b.nw));
    b.ozflag = (int*)take(64);
  }
  if (o.gfs & MH_GF_SURROGATE) {  // every self pair plus room for pairs outside the training box
    b.fb_cap = b.n * (b.nw + 64) + 4096;
    b.fb_list = (int4*)take((size_t)b.fb_cap * sizeof(int4));
    b.fb_state = (unsigned long long*)take(4 * sizeof(unsigned long long));
  }
  b.F = (double2*)take(nw * (size_t)std::max<int64_t>(o.n_inf, 1) * o.nrhs * 16);
  b.FK = (double2*)take(nw * (size_t)std::max<int64_t>(o.n_inf, 1) * std::max<int64_t>(o.n_beta, 1) * 16);
  b.nparams = 2 * nw + (size_t)o.n_beta + (size_t)(o.n_rad + o.n_inf + 1) / 2 + 2;
  b.params = (double*)take(b.nparams * 8);
  b.dofs = (double*)take((size_t)o.n_dofs * n * 3 * 8);
  return off;
}

size_t pinned_body(BodyPlan& b, const BatchOpts& o, char* base) {
  const size_t nw = (size_t)b.nw;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += align256(std::max<size_t>(bytes, 8));
    return p;
  };
  b.hF = (double2*)take(nw * (size_t)std::max<int64_t>(o.n_inf, 1) * o.nrhs * 16);
  b.hFK = (double2*)take(nw * (size_t)std::max<int64_t>(o.n_inf, 1) * std::max<int64_t>(o.n_beta, 1) * 16);
  b.hinfo = (int32_t*)take(nw * 4);
  b.hnorms = (double*)take((2 * (size_t)o.nrhs * nw + nw) * 8);
  b.hparams = (double*)take(b.nparams * 8);
  b.hdofs = (double*)take((size_t)o.n_dofs * (size_t)b.n * 3 * 8);
  return off;
}

// One body's whole sweep, enqueued on `st` with no host synchronisation.
void enqueue_body(mh_context* ctx, LaunchCounter lc, cudaStream_t st, BodyPlan& b, const BatchOpts& o) {
  const int64_t n = b.n, nw = b.nw, nn = n * n, bstride = n * o.nrhs;
  const double* om_d = b.params;
  const double* ks_d = b.params + nw;
  const double* beta_d = b.params + 2 * nw;
  const int32_t* rad_d = (const int32_t*)(b.params + 2 * nw + o.n_beta);
  const int32_t* inf_d = rad_d + o.n_rad;
  const uint32_t st_kinds = o.gfs & kStaticKinds;
  AssemblyParams p = make_params(ctx, b.m, o.gfs, o.direct, 1, nullptr);
  if (b.fb_state) {
    p.mlp = ctx->mlp;
    p.fb_list = b.fb_list;
    p.fb_state = b.fb_state;
    p.fb_cap = b.fb_cap;
    cudaMemsetAsync(b.fb_state, 0, 4 * sizeof(unsigned long long), st);
  }
  if (st_kinds) {
    AssemblyParams ps = make_params(ctx, b.m, st_kinds, o.direct, 1, nullptr);
    launch_assemble_static(st, lc, ps, b.SR, b.DR);
  }
  launch_assemble_wave(st, lc, p, st_kinds ? b.SR : nullptr, st_kinds ? b.DR : nullptr, (int)nw, ks_d, b.S, b.D,
                       nn, st_kinds ? 0 : 1);
  EpilogueGeom eg{n, b.m->n_hull, b.m->C, b.m->N, b.m->A, b.dofs};
  launch_build_rhs(st, lc, eg, (int)nw, om_d, o.g, (int)o.n_rad, rad_d, (int)o.n_beta, beta_d, b.B, bstride);
  BatchDesc d{n, nw, nn};
  if (b.ozflag) cudaMemsetAsync(b.ozflag, 0, sizeof(int), st);
  // S products on the tensor cores (FP64-accurate) outside the plain FP64 path
  auto s_times = [&](const double2* in, double2* out) {
    if (o.precision == MH_PREC_FP64) zgemm_nn_batched(st, lc, d, b.S, in, o.nrhs, bstride, out, b.work);
    else zgemm_nn_tc_batched(st, lc, d, b.S, in, o.nrhs, bstride, out, b.work, b.ozflag);
  };
  if (o.direct) s_times(b.B, b.X);
  else cudaMemcpyAsync(b.X, b.B, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st);
  if (o.precision == MH_PREC_FP64 || o.precision == MH_PREC_FP64_TC) {
    lu_factor_batched<double>(st, lc, d, b.D, b.ipiv, b.info, b.oz, b.ozflag);
    lu_solve_batched<double>(st, lc, d, b.D, b.ipiv, b.X, o.nrhs, bstride, false);
  } else {
    BatchDesc d32{n, nw, nn};
    const int64_t ncols = o.nrhs * nw;
    cudaMemcpyAsync(b.B0, b.X, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st);
    convert_with_norms(st, lc, d, b.D, b.LU32, nn, b.norms + 2 * ncols);
    lu_factor_batched<float>(st, lc, d32, b.LU32, b.ipiv, b.info, b.oz, b.ozflag);
    convert_z_to_c(st, lc, b.B0, b.X32, bstride * nw);
    lu_solve_batched<float>(st, lc, d32, b.LU32, b.ipiv, b.X32, o.nrhs, bstride, false);
    widen_c_to_z(st, lc, b.X32, b.X, bstride * nw);
    for (int it = 0; it < o.ir_sweeps; ++it) {
      residual_tc_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, bstride, b.R, b.work, b.ozflag);
      convert_z_to_c(st, lc, b.R, b.X32, bstride * nw);
      lu_solve_batched<float>(st, lc, d32, b.LU32, b.ipiv, b.X32, o.nrhs, bstride, false);
      ir_update(st, lc, bstride * nw, b.X, b.X32);
    }
    // the residual of the returned x, judged on the host after the graph
    residual_tc_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, bstride, b.R, b.work, b.ozflag);
    for (int64_t w = 0; w < nw; ++w) {
      inf_norms_batched(st, lc, n, o.nrhs, b.R + w * bstride, b.norms + w * o.nrhs);
      inf_norms_batched(st, lc, n, o.nrhs, b.X + w * bstride, b.norms + ncols + w * o.nrhs);
    }
    cudaMemcpyAsync(b.hnorms, b.norms, sizeof(double) * (2 * ncols + nw), cudaMemcpyDeviceToHost, st);
  }
  double2* phi = b.X;
  if (!o.direct) {
    s_times(b.X, b.B);
    phi = b.B;
  }
  if (o.n_inf > 0)
    launch_forces(st, lc, eg, (int)nw, om_d, o.rho, o.g, (int)o.nrhs, phi, bstride, (int)o.n_inf, inf_d,
                  (int)o.n_beta, beta_d, b.F, b.FK);
  cudaMemcpyAsync(b.hinfo, b.info, sizeof(int32_t) * nw, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(b.hF, b.F, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.nrhs,
                  cudaMemcpyDeviceToHost, st);
  if (o.n_beta > 0)
    cudaMemcpyAsync(b.hFK, b.FK, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.n_beta,
                    cudaMemcpyDeviceToHost, st);
}

// Host-side completion of one body after the graph: singular check, refinement
// convergence (extra sweeps or the FP64 fallback on the context stream).
int finish_body(mh_context* ctx, BodyPlan& b, const BatchOpts& o) {
  for (int64_t w = 0; w < b.nw; ++w)
    if (b.hinfo[w] != 0)
      return fail(ctx, MH_ERR_SINGULAR, "body with %lld panels, frequency %lld: zero pivot in column %d",
                  (long long)b.n, (long long)w, b.hinfo[w]);
  if (b.ozflag) {
    int flag = 0;
    MH_CUDA(ctx, cudaMemcpy(&flag, b.ozflag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  }
  if (b.fb_state) {
    unsigned long long fs[3] = {0, 0, 0};
    MH_CUDA(ctx, cudaMemcpy(fs, b.fb_state, sizeof(fs), cudaMemcpyDeviceToHost));
    if (fs[2]) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the surrogate assembly gave up");
    if (fs[1])
      return fail(ctx, MH_ERR_UNSUPPORTED, "body with %lld panels: more than %lld panel pairs lie outside the "
                                           "surrogate's training box; use ExactGuevelDelhommeau for it",
                  (long long)b.n, (long long)b.fb_cap);
  }
  if (o.precision != MH_PREC_MIXED) return MH_OK;
  const int64_t n = b.n, nw = b.nw, nn = n * n, bstride = n * o.nrhs, ncols = o.nrhs * nw;
  const double cte = std::sqrt((double)n) * 2.220446049250313e-16;
  auto converged = [&]() {
    for (int64_t c = 0; c < ncols; ++c) {
      const double anrm = b.hnorms[2 * ncols + c / o.nrhs];
      if (!(b.hnorms[c] <= cte * anrm * b.hnorms[ncols + c])) return false;
    }
    return true;
  };
  if (converged()) return MH_OK;
  cudaStream_t st = ctx->stream;
  const LaunchCounter lc = ctx->lc();
  BatchDesc d{n, nw, nn};
  bool ok = false;
  for (int it = 0; it < 30 && !ok; ++it) {
    convert_z_to_c(st, lc, b.R, b.X32, bstride * nw);
    lu_solve_batched<float>(st, lc, d, b.LU32, b.ipiv, b.X32, o.nrhs, bstride, false);
    ir_update(st, lc, bstride * nw, b.X, b.X32);
    residual_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, bstride, b.R, b.work, false);
    for (int64_t w = 0; w < nw; ++w) {
      inf_norms_batched(st, lc, n, o.nrhs, b.R + w * bstride, b.norms + w * o.nrhs);
      inf_norms_batched(st, lc, n, o.nrhs, b.X + w * bstride, b.norms + ncols + w * o.nrhs);
    }
    MH_CUDA(ctx, cudaMemcpyAsync(b.hnorms, b.norms, sizeof(double) * (2 * ncols + nw), cudaMemcpyDeviceToHost, st));
    MH_TRY(sync(ctx, "batch refinement"));
    ok = converged();
  }
  if (!ok) {
    MH_CUDA(ctx, cudaMemcpyAsync(b.X, b.B0, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st));
    lu_factor_batched<double>(st, lc, d, b.D, b.ipiv, b.info);
    lu_solve_batched<double>(st, lc, d, b.D, b.ipiv, b.X, o.nrhs, bstride, false);
  }
  // forces of the corrected solution
  const double* om_d = b.params;
  const double* beta_d = b.params + 2 * nw;
  const int32_t* inf_d = (const int32_t*)(b.params + 2 * nw + o.n_beta) + o.n_rad;
  EpilogueGeom eg{n, b.m->n_hull, b.m->C, b.m->N, b.m->A, b.dofs};
  double2* phi = b.X;
  if (!o.direct) {
    zgemm_nn_batched(st, lc, d, b.S, b.X, o.nrhs, bstride, b.B, b.work);
    phi = b.B;
  }
  if (o.n_inf > 0)
    launch_forces(st, lc, eg, (int)nw, om_d, o.rho, o.g, (int)o.nrhs, phi, bstride, (int)o.n_inf, inf_d,
                  (int)o.n_beta, beta_d, b.F, b.FK);
  MH_CUDA(ctx, cudaMemcpyAsync(b.hF, b.F, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.nrhs,
                               cudaMemcpyDeviceToHost, st));
  if (o.n_beta > 0)
    MH_CUDA(ctx, cudaMemcpyAsync(b.hFK, b.FK, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.n_beta,
                                 cudaMemcpyDeviceToHost, st));
  MH_CUDA(ctx, cudaMemcpyAsync(b.hinfo, b.info, sizeof(int32_t) * nw, cudaMemcpyDeviceToHost, st));
  MH_TRY(sync(ctx, "batch fallback"));
  for (int64_t w = 0; w < nw; ++w)
    if (b.hinfo[w] != 0) return fail(ctx, MH_ERR_SINGULAR, "singular matrix in the batch");
  return MH_OK;
}

}  // namespace

// ============================================================================
// C-ABI
// ============================================================================
namespace {
// device buffers of one training run, freed on every exit path
struct TrainBufs {
  cudaStream_t st = nullptr;
  std::vector<void*> ptrs;
  ~TrainBufs() {
    for (void* q : ptrs) cudaFreeAsync(q, st);
    if (st) cudaStreamSynchronize(st);
  }
  template <typename T>
  cudaError_t get(T** out, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(count, 1) * sizeof(T), st);
    if (e == cudaSuccess) ptrs.push_back(q);
    *out = static_cast<T*>(q);
    return e;
  }
};

uint64_t gcd_u64(uint64_t a, uint64_t b) {
  while (b) { uint64_t t = a % b; a = b; b = t; }
  return a;
}
}  // namespace

namespace {

// Time one batched factorization of d.batch random matrices of order d.n with the
// context's current launch shapes: the smallest of `reps` runs after one warm-up (ms).
template <typename T>
int time_factorization(mh_context* ctx, const BatchDesc& d, typename cplx_t<T>::type* A, int32_t* ipiv, int32_t* info,
                       void* emu_ws, int* emu_flag, int reps, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
  double best = 1e300;
  for (int r = 0; r <= reps; ++r) {
    fill_random_matrices<T>(ctx->stream, ctx->lc(), d, A, 0x5EEDull + (uint64_t)r);
    if (emu_flag) MH_CUDA(ctx, cudaMemsetAsync(emu_flag, 0, sizeof(int), ctx->stream));
    MH_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    lu_factor_batched<T>(ctx->stream, ctx->lc(), d, A, ipiv, info, emu_ws, emu_flag);
    MH_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    MH_TRY(check_launch(ctx, "autotune factorization"));
    MH_TRY(sync(ctx, "autotune factorization"));
    if (emu_flag) {
      int hflag = 0;
      MH_CUDA(ctx, cudaMemcpy(&hflag, emu_flag, sizeof(int), cudaMemcpyDeviceToHost));
      if (hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
    }
    float t = 0.f;
    MH_CUDA(ctx, cudaEventElapsedTime(&t, e0, e1));
    if (r > 0) best = std::min(best, (double)t);
  }
  *ms = best;
  return MH_OK;
}

}  // namespace

extern "C" {

int mh_abi_version(void) { return MH_ABI_VERSION; }

int mh_create(int device, mh_context** out) {
  if (!out) return MH_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= 0) return MH_ERR_CUDA;
  if (device < 0 || device >= ndev) return MH_ERR_ARG;
  mh_context* ctx = new mh_context();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return MH_ERR_CUDA;
  }
  ctx->stream = ctx->own;
  ctx->prof = profiler_create();
  *out = ctx;
  return MH_OK;
}

int mh_destroy(mh_context* ctx) {
  if (!ctx) return MH_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& b : ctx->ws)
    if (b.p) cudaFreeAsync(b.p, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->mlp) cudaFree(ctx->mlp);
  delete ctx->batch;
  for (cudaStream_t st : ctx->side) cudaStreamDestroy(st);
  if (ctx->own) cudaStreamDestroy(ctx->own);
  profiler_destroy(ctx->prof);
  delete ctx;
  return MH_OK;
}

const char* mh_last_error(const mh_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mh_get_stream(mh_context* ctx, void** stream) {
  if (!ctx || !stream) return MH_ERR_ARG;
  *stream = (void*)ctx->stream;
  return MH_OK;
}

int mh_set_stream(mh_context* ctx, void* stream) {
  if (!ctx) return MH_ERR_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
  return MH_OK;
}

int mh_synchronize(mh_context* ctx) {
  if (!ctx) return MH_ERR_ARG;
  MH_TRY(set_device(ctx));
  return sync(ctx, "synchronize");
}

int64_t mh_launch_count(const mh_context* ctx) { return ctx ? ctx->launches : -1; }

int64_t mh_workspace_bytes(const mh_context* ctx) {
  if (!ctx) return -1;
  int64_t s = 0;
  for (auto& b : ctx->ws) s += (int64_t)b.bytes;
  return s;
}

int mh_set_quadrature_tolerance(mh_context* ctx, double rtol, double atol) {
  if (!ctx) return MH_ERR_ARG;
  if (!(rtol >= 0) || !(atol >= 0) || (rtol == 0 && atol == 0))
    return fail(ctx, MH_ERR_ARG, "quadrature tolerances must be >= 0 and not both zero");
  ctx->quad_rtol = rtol;
  ctx->quad_atol = atol;
  return MH_OK;
}

int mh_mesh_create(mh_context* ctx, int64_t n, const double* vertices, const double* centers, const double* normals,
                   const double* areas, const double* radii, int mem, mh_mesh** out) {
  NvtxRange nvtx_range("mh_mesh_create");
  if (!ctx || !out) return MH_ERR_ARG;
  *out = nullptr;
  if (n <= 0) return fail(ctx, MH_ERR_ARG, "mesh needs at least one panel (got %lld)", (long long)n);
  if (!vertices || !centers || !normals || !areas || !radii)
    return fail(ctx, MH_ERR_ARG, "mesh arrays must not be NULL");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (mem == MH_MEM_HOST) {
    const double* arrs[5] = {vertices, centers, normals, areas, radii};
    const int64_t lens[5] = {12 * n, 3 * n, 3 * n, n, n};
    const char* names[5] = {"vertices", "centers", "normals", "areas", "radii"};
    for (int a = 0; a < 5; ++a)
      for (int64_t q = 0; q < lens[a]; ++q)
        if (!std::isfinite(arrs[a][q]))
          return fail(ctx, MH_ERR_ARG, "mesh %s[%lld] is not finite", names[a], (long long)q);
  }
  MH_TRY(set_device(ctx));
  mh_mesh* m = new mh_mesh();
  m->ctx = ctx;
  m->n = n;
  m->n_hull = n;
  const size_t nb = (size_t)n * sizeof(double);
  // one allocation: V | C | N | A | R | P
  char* base = nullptr;
  size_t bytes = nb * 20 + (size_t)n * sizeof(PanelRec) + 256;
  cudaError_t e = cudaMallocAsync((void**)&base, bytes, ctx->stream);
  if (e != cudaSuccess) {
    delete m;
    return fail(ctx, MH_ERR_NOMEM, "mesh allocation: %s", cudaGetErrorString(e));
  }
  m->V = (double*)base;
  m->C = m->V + 12 * n;
  m->N = m->C + 3 * n;
  m->A = m->N + 3 * n;
  m->R = m->A + n;
  m->P = (PanelRec*)(((uintptr_t)(m->R + n) + 255) & ~(uintptr_t)255);
  int rc = copy_in(ctx, m->V, vertices, nb * 12, mem);
  if (!rc) rc = copy_in(ctx, m->C, centers, nb * 3, mem);
  if (!rc) rc = copy_in(ctx, m->N, normals, nb * 3, mem);
  if (!rc) rc = copy_in(ctx, m->A, areas, nb, mem);
  if (!rc) rc = copy_in(ctx, m->R, radii, nb, mem);
  if (!rc) {
    launch_panel_geometry(ctx->stream, ctx->lc(), n, m->V, m->C, m->N, m->A, m->R, m->P);
    rc = check_launch(ctx, "panel geometry");
  }
  if (rc) {
    cudaFreeAsync(base, ctx->stream);
    delete m;
    return rc;
  }
  *out = m;
  return MH_OK;
}

int mh_mesh_destroy(mh_mesh* m) {
  if (!m) return MH_OK;
  mh_context* ctx = m->ctx;
  cudaSetDevice(ctx->device);
  // a cached batch graph that reads this mesh's buffers goes with it (the cache is keyed by
  // mesh address, which a later mesh may reuse)
  if (ctx->batch) {
    bool uses = false;
    for (const BodyPlan& b : ctx->batch->bodies) uses = uses || b.m == m;
    if (uses) {
      cudaStreamSynchronize(ctx->stream);
      delete ctx->batch;
      ctx->batch = nullptr;
    }
  }
  if (m->SR) cudaFreeAsync(m->SR, ctx->stream);
  if (m->DR) cudaFreeAsync(m->DR, ctx->stream);
  if (m->V) cudaFreeAsync(m->V, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  delete m;
  return MH_OK;
}

int64_t mh_mesh_panels(const mh_mesh* m) { return m ? m->n : -1; }

int mh_mesh_set_lid(mh_mesh* m, int64_t n_hull) {
  if (!m) return MH_ERR_ARG;
  mh_context* ctx = m->ctx;
  if (n_hull < 1 || n_hull > m->n)
    return fail(ctx, MH_ERR_ARG, "n_hull must be in 1..%lld (got %lld)", (long long)m->n, (long long)n_hull);
  if (n_hull < m->n) {
    // Lid panels at the free surface meet the vv = 0 singularity of the wave terms at their
    // self pairs (wu.jl:21-24: dd = 0; the exact term's E1(0)); the reference's lids sit below it.
    MH_TRY(set_device(ctx));
    const int64_t nl = m->n - n_hull;
    std::vector<double> c((size_t)(3 * nl));
    MH_CUDA(ctx, cudaMemcpyAsync(c.data(), m->C + 3 * n_hull, sizeof(double) * 3 * nl, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    MH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < nl; ++i)
      if (!(c[3 * i + 2] < -1e-8))
        return fail(ctx, MH_ERR_ARG, "lid panel %lld has centre z = %g; a lid must lie below the free surface",
                    (long long)(n_hull + i), c[3 * i + 2]);
  }
  m->n_hull = n_hull;
  return MH_OK;
}

int mh_assemble_matrices(mh_context* ctx, mh_mesh* m, double k, uint32_t gfs, int direct, int include_identity,
                         const double* fixed_normal, double* S, double* D, int mem) {
  NvtxRange nvtx_range("mh_assemble_matrices");
  if (!ctx) return MH_ERR_ARG;
  if (!m || m->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh does not belong to this context");
  if (!S || !D) return fail(ctx, MH_ERR_ARG, "S and D must not be NULL");
  MH_TRY(check_gfs(ctx, gfs));
  if ((gfs & kWaveKinds) && !(k > 0) )
    return fail(ctx, MH_ERR_ARG, "wave Green functions need a positive wavenumber (got %g)", k);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  MH_TRY(set_device(ctx));
  const int64_t n = m->n;
  const size_t nn = (size_t)n * (size_t)n;
  const uint32_t st = gfs & kStaticKinds;
  if (st) MH_TRY(ensure_static_cache(ctx, m, gfs, direct, include_identity, fixed_normal));
  double2 *Sd, *Dd;
  if (mem == MH_MEM_DEVICE) {
    Sd = (double2*)S;
    Dd = (double2*)D;
  } else {
    MH_TRY(ws_get_t(ctx, kSlotS, nn, &Sd));
    MH_TRY(ws_get_t(ctx, kSlotD, nn, &Dd));
  }
  double* kd;
  MH_TRY(ws_get_t(ctx, kSlotSmall, 4, &kd));
  double* hk;
  MH_TRY(pinned_get(ctx, 64, &hk));
  hk[0] = k;
  MH_CUDA(ctx, cudaMemcpyAsync(kd, hk, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  AssemblyParams p = make_params(ctx, m, gfs, direct, include_identity, fixed_normal);
  MH_TRY(prepare_surrogate(ctx, p, 1));
  launch_assemble_wave(ctx->stream, ctx->lc(), p, st ? m->SR : nullptr, st ? m->DR : nullptr, 1, kd, Sd, Dd,
                       (int64_t)nn, (!st && include_identity) ? 1 : 0);
  MH_TRY(check_launch(ctx, "wave assembly"));
  if (mem == MH_MEM_HOST) {
    MH_TRY(copy_out(ctx, S, Sd, nn * sizeof(double2), mem));
    MH_TRY(copy_out(ctx, D, Dd, nn * sizeof(double2), mem));
  }
  MH_TRY(sync(ctx, "assemble_matrices"));
  return check_surrogate(ctx, p);
}

int mh_linsolve(mh_context* ctx, int64_t n, int64_t nrhs, const double* A, const double* B, double* X, int precision,
                int mem) {
  NvtxRange nvtx_range("mh_linsolve");
  if (!ctx) return MH_ERR_ARG;
  if (n <= 0 || nrhs <= 0) return fail(ctx, MH_ERR_ARG, "bad sizes n=%lld nrhs=%lld", (long long)n, (long long)nrhs);
  if (!A || !B || !X) return fail(ctx, MH_ERR_ARG, "A, B and X must not be NULL");
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "order %lld exceeds the supported %lld", (long long)n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const size_t nn = (size_t)n * (size_t)n, nx = (size_t)n * (size_t)nrhs;
  double2 *Ad, *Xd;
  MH_TRY(ws_get_t(ctx, kSlotA64, nn, &Ad));
  MH_TRY(ws_get_t(ctx, kSlotX, nx, &Xd));
  MH_TRY(copy_in(ctx, Ad, A, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Xd, B, nx * sizeof(double2), mem));
  BatchDesc d{n, 1, (int64_t)nn};
  MH_TRY(solve_core(ctx, d, Ad, Xd, nrhs, (int64_t)nx, precision, false));
  MH_TRY(copy_out(ctx, X, Xd, nx * sizeof(double2), mem));
  return sync(ctx, "linsolve");
}

int mh_linsolve_adjoint(mh_context* ctx, int64_t n, int64_t nrhs, const double* A, const double* Ybar,
                        double* Lambda, int precision, int mem) {
  NvtxRange nvtx_range("mh_linsolve_adjoint");
  if (!ctx) return MH_ERR_ARG;
  if (n <= 0 || nrhs <= 0) return fail(ctx, MH_ERR_ARG, "bad sizes n=%lld nrhs=%lld", (long long)n, (long long)nrhs);
  if (!A || !Ybar || !Lambda) return fail(ctx, MH_ERR_ARG, "A, Ybar and Lambda must not be NULL");
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "order %lld exceeds the supported %lld", (long long)n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const size_t nn = (size_t)n * (size_t)n, nx = (size_t)n * (size_t)nrhs;
  double2 *Ad, *Xd;
  MH_TRY(ws_get_t(ctx, kSlotA64, nn, &Ad));
  MH_TRY(ws_get_t(ctx, kSlotX, nx, &Xd));
  MH_TRY(copy_in(ctx, Ad, A, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Xd, Ybar, nx * sizeof(double2), mem));
  BatchDesc d{n, 1, (int64_t)nn};
  MH_TRY(solve_core(ctx, d, Ad, Xd, nrhs, (int64_t)nx, precision, true));
  MH_TRY(copy_out(ctx, Lambda, Xd, nx * sizeof(double2), mem));
  return sync(ctx, "linsolve_adjoint");
}

int mh_solve(mh_context* ctx, int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc, int direct,
             double* phi, double* sources, int precision, int mem) {
  NvtxRange nvtx_range("mh_solve");
  if (!ctx) return MH_ERR_ARG;
  if (n <= 0 || nrhs <= 0) return fail(ctx, MH_ERR_ARG, "bad sizes n=%lld nrhs=%lld", (long long)n, (long long)nrhs);
  if (!D || !S || !bc || !phi) return fail(ctx, MH_ERR_ARG, "D, S, bc and phi must not be NULL");
  if (!direct && !sources) return fail(ctx, MH_ERR_ARG, "the indirect method needs a `sources` buffer");
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "order %lld exceeds the supported %lld", (long long)n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const size_t nn = (size_t)n * (size_t)n, nx = (size_t)n * (size_t)nrhs;
  double2 *Ad, *Sd, *Bd, *Xd, *work;
  MH_TRY(ws_get_t(ctx, kSlotA64, nn, &Ad));
  MH_TRY(ws_get_t(ctx, kSlotS, nn, &Sd));
  MH_TRY(ws_get_t(ctx, kSlotIn, nx, &Bd));
  MH_TRY(ws_get_t(ctx, kSlotX, nx, &Xd));
  MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
  MH_TRY(copy_in(ctx, Ad, D, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Sd, S, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Bd, bc, nx * sizeof(double2), mem));
  BatchDesc d{n, 1, (int64_t)nn};
  if (direct) {
    zgemm_nn_batched(ctx->stream, ctx->lc(), d, Sd, Bd, nrhs, (int64_t)nx, Xd, work);
    MH_TRY(check_launch(ctx, "S*bc"));
    MH_TRY(solve_core(ctx, d, Ad, Xd, nrhs, (int64_t)nx, precision, false));
    MH_TRY(copy_out(ctx, phi, Xd, nx * sizeof(double2), mem));
  } else {
    MH_CUDA(ctx, cudaMemcpyAsync(Xd, Bd, nx * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
    MH_TRY(solve_core(ctx, d, Ad, Xd, nrhs, (int64_t)nx, precision, false));
    MH_TRY(copy_out(ctx, sources, Xd, nx * sizeof(double2), mem));
    MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
    zgemm_nn_batched(ctx->stream, ctx->lc(), d, Sd, Xd, nrhs, (int64_t)nx, Bd, work);
    MH_TRY(check_launch(ctx, "S*sources"));
    MH_TRY(copy_out(ctx, phi, Bd, nx * sizeof(double2), mem));
  }
  return sync(ctx, "solve");
}

int mh_hydrodynamic_coefficients(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho,
                                 double g, uint32_t gfs, int direct, int64_t n_dofs, const double* dofs,
                                 int64_t n_rad, const int32_t* rad_idx, int64_t n_inf, const int32_t* inf_idx,
                                 int64_t n_beta, const double* betas, int precision, double* added_mass,
                                 double* radiation_damping, double* diffraction_force, double* froude_krylov_force,
                                 double* excitation_force, int mem) {
  NvtxRange nvtx_range("mh_hydrodynamic_coefficients");
  if (!ctx) return MH_ERR_ARG;
  if (!m || m->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh does not belong to this context");
  if (n_omega <= 0 || !omegas) return fail(ctx, MH_ERR_ARG, "need at least one wave frequency");
  if (n_rad < 0 || n_inf < 0 || n_beta < 0 || n_dofs < 0) return fail(ctx, MH_ERR_ARG, "negative counts");
  if (n_rad + n_beta == 0) return fail(ctx, MH_ERR_ARG, "nothing to solve: no radiating dof and no wave direction");
  if ((n_rad > 0 || n_inf > 0) && (!dofs || n_dofs <= 0)) return fail(ctx, MH_ERR_ARG, "dof fields required");
  MH_TRY(check_gfs(ctx, gfs));
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (!(rho > 0) || !(g > 0)) return fail(ctx, MH_ERR_ARG, "rho and g must be positive");
  for (int64_t w = 0; w < n_omega; ++w)
    if (!(omegas[w] > 0)) return fail(ctx, MH_ERR_ARG, "wave frequencies must be positive (omega[%lld]=%g)", (long long)w, omegas[w]);
  for (int64_t q = 0; q < n_rad; ++q)
    if (rad_idx[q] < 0 || rad_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "radiating dof index out of range");
  for (int64_t q = 0; q < n_inf; ++q)
    if (inf_idx[q] < 0 || inf_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "influenced dof index out of range");
  if (m->n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "mesh of %lld panels exceeds the supported %lld", (long long)m->n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const int64_t n = m->n;
  const size_t nn = (size_t)n * (size_t)n;
  const int64_t nrhs = n_rad + n_beta;
  const uint32_t st = gfs & kStaticKinds;

  // small parameter arrays -> device in one pinned staging block:
  // [omegas | betas | wavenumbers | rad_idx, inf_idx (int32)]
  const size_t n_int_d = (size_t)((n_rad + n_inf + 1) / 2) + 1;
  const size_t nsmall = (size_t)n_omega * 2 + (size_t)n_beta + n_int_d + 8;
  double* hs;
  MH_TRY(pinned_get(ctx, nsmall * sizeof(double), &hs));
  double* small_d;
  MH_TRY(ws_get_t(ctx, kSlotIdx, nsmall, &small_d));
  std::memcpy(hs, omegas, sizeof(double) * n_omega);
  if (n_beta) std::memcpy(hs + n_omega, betas, sizeof(double) * n_beta);
  for (int64_t w = 0; w < n_omega; ++w) hs[n_omega + n_beta + w] = omegas[w] * omegas[w] / g;  // compute_wavenumber
  int32_t* hidx = (int32_t*)(hs + 2 * n_omega + n_beta);
  for (int64_t q = 0; q < n_rad; ++q) hidx[q] = rad_idx[q];
  for (int64_t q = 0; q < n_inf; ++q) hidx[n_rad + q] = inf_idx[q];
  MH_CUDA(ctx, cudaMemcpyAsync(small_d, hs, nsmall * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const double* om_d = small_d;
  const double* beta_d = small_d + n_omega;
  const double* ks_all = small_d + n_omega + n_beta;
  const int32_t* rad_d = (const int32_t*)(small_d + 2 * n_omega + n_beta);
  const int32_t* inf_d = rad_d + n_rad;

  // dof fields
  const double* dofs_d = nullptr;
  if (n_dofs > 0) {
    if (mem == MH_MEM_DEVICE) {
      dofs_d = dofs;
    } else {
      double* dd;
      MH_TRY(ws_get_t(ctx, kSlotDofs, (size_t)(n_dofs * n * 3), &dd));
      MH_TRY(copy_in(ctx, dd, dofs, sizeof(double) * n_dofs * n * 3, MH_MEM_HOST));
      dofs_d = dd;
    }
  }

  // wavenumber-independent part, once for the whole sweep
  double *SR = nullptr, *DR = nullptr;
  if (st) {
    MH_TRY(ws_get_t(ctx, kSlotSR, nn, &SR));
    MH_TRY(ws_get_t(ctx, kSlotDR, nn, &DR));
    MH_TRY(compute_static(ctx, m, gfs, direct, 1, nullptr, SR, DR));
  }

  // chunk the frequencies by memory
  size_t free_b = 0, total_b = 0;
  MH_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
  size_t per_w = nn * sizeof(double2) * 2 + (size_t)n * nrhs * sizeof(double2) * 4;
  if (precision == MH_PREC_MIXED) per_w += nn * sizeof(float2);
  size_t budget = std::min<size_t>(free_b / 2, (size_t)48 << 30);
  int64_t chunk = (int64_t)std::max<size_t>(1, budget / per_w);
  chunk = std::min<int64_t>(chunk, n_omega);

  double2 *S, *D, *B, *X, *work, *F, *FK;
  MH_TRY(ws_get_t(ctx, kSlotS, nn * chunk, &S));
  MH_TRY(ws_get_t(ctx, kSlotD, nn * chunk, &D));
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(n * nrhs * chunk), &B));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(n * nrhs * chunk), &X));
  MH_TRY(ws_get_t(ctx, kSlotF, (size_t)(n_omega * std::max<int64_t>(n_inf, 1) * nrhs), &F));
  MH_TRY(ws_get_t(ctx, kSlotFK, (size_t)(n_omega * std::max<int64_t>(n_inf, 1) * std::max<int64_t>(n_beta, 1)), &FK));

  EpilogueGeom eg{n, m->n_hull, m->C, m->N, m->A, dofs_d};
  AssemblyParams p = make_params(ctx, m, gfs, direct, 1, nullptr);
  MH_TRY(prepare_surrogate(ctx, p, chunk));

  for (int64_t w0 = 0; w0 < n_omega; w0 += chunk) {
    const int64_t nw = std::min<int64_t>(chunk, n_omega - w0);
    launch_assemble_wave(ctx->stream, ctx->lc(), p, SR, DR, (int)nw, ks_all + w0, S, D, (int64_t)nn,
                         st ? 0 : 1);
    MH_TRY(check_launch(ctx, "wave assembly"));
    const int64_t bstride = n * nrhs;
    launch_build_rhs(ctx->stream, ctx->lc(), eg, (int)nw, om_d + w0, g, (int)n_rad, rad_d, (int)n_beta, beta_d, B,
                     bstride);
    MH_TRY(check_launch(ctx, "boundary conditions"));
    BatchDesc d{n, nw, (int64_t)nn};
    MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, nw), &work));
    // S times a block of vectors: FP64 FMAs in the plain path, the FP64-accurate tensor-core
    // product in the others
    int* tcflag;
    MH_TRY(ws_get_t(ctx, kSlotTcFlag, 4, &tcflag));
    auto s_times = [&](const double2* in, double2* out) -> int {
      if (precision == MH_PREC_FP64) {
        zgemm_nn_batched(ctx->stream, ctx->lc(), d, S, in, nrhs, bstride, out, work);
        return check_launch(ctx, "S product");
      }
      MH_CUDA(ctx, cudaMemsetAsync(tcflag + 2, 0, sizeof(int), ctx->stream));
      zgemm_nn_tc_batched(ctx->stream, ctx->lc(), d, S, in, nrhs, bstride, out, work, tcflag + 2);
      MH_TRY(check_launch(ctx, "S product"));
      int hflag = 0;
      MH_CUDA(ctx, cudaMemcpyAsync(&hflag, tcflag + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      MH_TRY(sync(ctx, "S product"));
      if (hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the S product gave up");
      return MH_OK;
    };
    if (direct) {
      MH_TRY(s_times(B, X));
      MH_TRY(solve_core(ctx, d, D, X, nrhs, bstride, precision, false));
    } else {
      MH_CUDA(ctx, cudaMemcpyAsync(X, B, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, ctx->stream));
      MH_TRY(solve_core(ctx, d, D, X, nrhs, bstride, precision, false));
      MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, nw), &work));
      MH_TRY(s_times(X, B));
      std::swap(B, X);
    }
    if (n_inf > 0) {
      launch_forces(ctx->stream, ctx->lc(), eg, (int)nw, om_d + w0, rho, g, (int)nrhs, X, bstride, (int)n_inf, inf_d,
                    (int)n_beta, beta_d, F + w0 * n_inf * nrhs, FK + w0 * n_inf * std::max<int64_t>(n_beta, 1));
      MH_TRY(check_launch(ctx, "forces"));
    }
    if (!direct) std::swap(B, X);
  }
  // pack (n_U = 1): A[i, r, w] = Re F / w^2, B = Im F / w  (problems_and_results.jl:207-208, 325-339);
  // Fd[i, w, b], Fk, Fe = Fd + Fk  (problems_and_results.jl:218-219, 366-380)
  const int64_t ninf1 = std::max<int64_t>(n_inf, 1), nb1 = std::max<int64_t>(n_beta, 1);
  std::vector<double2> hF((size_t)(n_omega * ninf1 * nrhs)), hFK((size_t)(n_omega * ninf1 * nb1));
  if (n_inf > 0) {
    MH_CUDA(ctx, cudaMemcpyAsync(hF.data(), F, sizeof(double2) * hF.size(), cudaMemcpyDeviceToHost, ctx->stream));
    if (n_beta > 0)
      MH_CUDA(ctx, cudaMemcpyAsync(hFK.data(), FK, sizeof(double2) * hFK.size(), cudaMemcpyDeviceToHost, ctx->stream));
  }
  MH_TRY(sync(ctx, "sweep"));
  MH_TRY(check_surrogate(ctx, p));
  std::vector<double> hA((size_t)(n_inf * n_rad * n_omega)), hB(hA.size());
  std::vector<double2> hd((size_t)(n_inf * n_omega * n_beta)), hk(hd.size()), he(hd.size());
  for (int64_t w = 0; w < n_omega; ++w) {
    const double om = omegas[w];
    for (int64_t i = 0; i < n_inf; ++i) {
      for (int64_t r = 0; r < n_rad; ++r) {
        double2 f = hF[(w * n_inf + i) * nrhs + r];
        hA[i + n_inf * (r + n_rad * w)] = f.x / (om * om);
        hB[i + n_inf * (r + n_rad * w)] = f.y / om;
      }
      for (int64_t b = 0; b < n_beta; ++b) {
        double2 fd = hF[(w * n_inf + i) * nrhs + n_rad + b];
        double2 fk = hFK[(w * n_inf + i) * n_beta + b];
        size_t o = (size_t)(i + n_inf * (w + n_omega * b));
        hd[o] = fd;
        hk[o] = fk;
        he[o] = make_double2(fd.x + fk.x, fd.y + fk.y);
      }
    }
  }
  MH_TRY(put_out(ctx, added_mass, hA.data(), hA.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, radiation_damping, hB.data(), hB.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, diffraction_force, hd.data(), hd.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, froude_krylov_force, hk.data(), hk.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, excitation_force, he.data(), he.size() * sizeof(double2), mem));
  return sync(ctx, "sweep outputs");
}

int mh_hydro_frequency_derivative(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho,
                                  double g, uint32_t gfs, int direct, int64_t n_dofs, const double* dofs,
                                  int64_t n_rad, const int32_t* rad_idx, int64_t n_inf, const int32_t* inf_idx,
                                  int64_t n_beta, const double* betas, double* added_mass, double* radiation_damping,
                                  double* diffraction_force, double* froude_krylov_force, double* excitation_force,
                                  double* d_added_mass, double* d_radiation_damping, double* d_diffraction_force,
                                  double* d_froude_krylov_force, double* d_excitation_force, int mem) {
  NvtxRange nvtx_range("mh_hydro_frequency_derivative");
  if (!ctx) return MH_ERR_ARG;
  if (!m || m->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh does not belong to this context");
  if (n_omega <= 0 || !omegas) return fail(ctx, MH_ERR_ARG, "need at least one wave frequency");
  if (n_rad < 0 || n_inf < 0 || n_beta < 0 || n_dofs < 0) return fail(ctx, MH_ERR_ARG, "negative counts");
  if (n_rad + n_beta == 0) return fail(ctx, MH_ERR_ARG, "nothing to solve: no radiating dof and no wave direction");
  if ((n_rad > 0 || n_inf > 0) && (!dofs || n_dofs <= 0)) return fail(ctx, MH_ERR_ARG, "dof fields required");
  MH_TRY(check_gfs(ctx, gfs));
  if (gfs & (MH_GF_EXACT_DELHOMMEAU | MH_GF_SURROGATE))
    return fail(ctx, MH_ERR_UNSUPPORTED, "the frequency derivative covers the Rankine kinds and GFWu (got 0x%x)", gfs);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (!(rho > 0) || !(g > 0)) return fail(ctx, MH_ERR_ARG, "rho and g must be positive");
  for (int64_t w = 0; w < n_omega; ++w)
    if (!(omegas[w] > 0)) return fail(ctx, MH_ERR_ARG, "wave frequencies must be positive (omega[%lld]=%g)", (long long)w, omegas[w]);
  for (int64_t q = 0; q < n_rad; ++q)
    if (rad_idx[q] < 0 || rad_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "radiating dof index out of range");
  for (int64_t q = 0; q < n_inf; ++q)
    if (inf_idx[q] < 0 || inf_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "influenced dof index out of range");
  if (m->n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "mesh of %lld panels exceeds the supported %lld", (long long)m->n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const int64_t n = m->n, nh = m->n_hull;
  const size_t nn = (size_t)n * (size_t)n;
  const int64_t nrhs = n_rad + n_beta, bstride = n * nrhs;
  const uint32_t st = gfs & kStaticKinds;
  cudaStream_t s0 = ctx->stream;

  // [omegas | betas | wavenumbers | rad_idx, inf_idx]
  const size_t n_int_d = (size_t)((n_rad + n_inf + 1) / 2) + 1;
  const size_t nsmall = (size_t)n_omega * 2 + (size_t)n_beta + n_int_d + 8;
  double* hs;
  MH_TRY(pinned_get(ctx, nsmall * sizeof(double), &hs));
  double* small_d;
  MH_TRY(ws_get_t(ctx, kSlotIdx, nsmall, &small_d));
  std::memcpy(hs, omegas, sizeof(double) * n_omega);
  if (n_beta) std::memcpy(hs + n_omega, betas, sizeof(double) * n_beta);
  for (int64_t w = 0; w < n_omega; ++w) hs[n_omega + n_beta + w] = omegas[w] * omegas[w] / g;
  int32_t* hidx = (int32_t*)(hs + 2 * n_omega + n_beta);
  for (int64_t q = 0; q < n_rad; ++q) hidx[q] = rad_idx[q];
  for (int64_t q = 0; q < n_inf; ++q) hidx[n_rad + q] = inf_idx[q];
  MH_CUDA(ctx, cudaMemcpyAsync(small_d, hs, nsmall * sizeof(double), cudaMemcpyHostToDevice, s0));
  const double* om_d = small_d;
  const double* beta_d = small_d + n_omega;
  const double* ks_all = small_d + n_omega + n_beta;
  const int32_t* rad_d = (const int32_t*)(small_d + 2 * n_omega + n_beta);
  const int32_t* inf_d = rad_d + n_rad;

  // dof fields on the device and, for the Froude-Krylov derivative, on the host
  std::vector<double> hdofs((size_t)(n_dofs * n * 3)), hC((size_t)(3 * n)), hN((size_t)(3 * n)), hAr((size_t)n);
  const double* dofs_d = nullptr;
  if (n_dofs > 0) {
    double* dd;
    MH_TRY(ws_get_t(ctx, kSlotDofs, (size_t)(n_dofs * n * 3), &dd));
    MH_TRY(copy_in(ctx, dd, dofs, sizeof(double) * n_dofs * n * 3, mem));
    dofs_d = dd;
    MH_CUDA(ctx, cudaMemcpyAsync(hdofs.data(), dd, sizeof(double) * hdofs.size(), cudaMemcpyDeviceToHost, s0));
  }
  MH_CUDA(ctx, cudaMemcpyAsync(hC.data(), m->C, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s0));
  MH_CUDA(ctx, cudaMemcpyAsync(hN.data(), m->N, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s0));
  MH_CUDA(ctx, cudaMemcpyAsync(hAr.data(), m->A, sizeof(double) * n, cudaMemcpyDeviceToHost, s0));

  double *SR = nullptr, *DR = nullptr;
  if (st) {
    MH_TRY(ws_get_t(ctx, kSlotSR, nn, &SR));
    MH_TRY(ws_get_t(ctx, kSlotDR, nn, &DR));
    MH_TRY(compute_static(ctx, m, gfs, direct, 1, nullptr, SR, DR));
  }
  double2 *S, *D, *dS, *dD, *B, *X, *dB, *R, *T, *P2, *F, *FK, *dF, *work;
  int32_t* ipiv;
  MH_TRY(ws_get_t(ctx, kSlotS, nn, &S));
  MH_TRY(ws_get_t(ctx, kSlotD, nn, &D));
  MH_TRY(ws_get_t(ctx, kSlotA64, nn, &dS));
  MH_TRY(ws_get_t(ctx, kSlotLU32, nn, &dD));
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)bstride, &B));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)bstride, &X));
  MH_TRY(ws_get_t(ctx, kSlotB, (size_t)bstride, &dB));
  MH_TRY(ws_get_t(ctx, kSlotR, (size_t)bstride, &R));
  MH_TRY(ws_get_t(ctx, kSlotT, (size_t)bstride, &T));
  MH_TRY(ws_get_t(ctx, kSlotLam, (size_t)bstride, &P2));
  const int64_t ninf1 = std::max<int64_t>(n_inf, 1), nb1 = std::max<int64_t>(n_beta, 1);
  MH_TRY(ws_get_t(ctx, kSlotF, (size_t)(n_omega * ninf1 * nrhs), &F));
  MH_TRY(ws_get_t(ctx, kSlotFK, (size_t)(n_omega * ninf1 * nb1), &FK));
  MH_TRY(ws_get_t(ctx, kSlotGrad, (size_t)(n_omega * ninf1 * nrhs), &dF));
  MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)n, &ipiv));

  EpilogueGeom eg{n, nh, m->C, m->N, m->A, dofs_d};
  AssemblyParams p = make_params(ctx, m, gfs, direct, 1, nullptr);
  const BatchDesc d{n, 1, (int64_t)nn};
  LaunchCounter lc = ctx->lc();
  auto times = [&](const double2* A, const double2* in, double2* out) {
    zgemm_nn_batched(s0, lc, d, A, in, nrhs, bstride, out, work);
  };
  for (int64_t w = 0; w < n_omega; ++w) {
    const double om = omegas[w];
    launch_assemble_wave(s0, lc, p, SR, DR, 1, ks_all + w, S, D, (int64_t)nn, st ? 0 : 1);
    launch_wave_dk(s0, lc, p, ks_all + w, dS, dD);
    launch_build_rhs(s0, lc, eg, 1, om_d + w, g, (int)n_rad, rad_d, (int)n_beta, beta_d, B, bstride);
    launch_build_drhs(s0, lc, eg, 1, om_d + w, g, (int)n_rad, rad_d, (int)n_beta, beta_d, dB, bstride);
    MH_TRY(check_launch(ctx, "frequency-derivative assembly"));
    // dS/domega = dS/dk dk/domega, likewise D: scale the products by dk/domega = 2 omega / g
    const double dk = 2.0 * om / g;
    if (direct) {
      // phi = D^-1 S b;  dphi = D^-1 (dS b + S db - dD phi)
      times(S, B, X);
      MH_TRY(solve_core(ctx, d, D, X, nrhs, bstride, MH_PREC_FP64, false));
      MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)n, &ipiv));
      times(dS, B, R);
      MH_CUDA(ctx, cudaMemsetAsync(P2, 0, sizeof(double2) * bstride, s0));
      launch_zaxpy(s0, lc, bstride, dk, R, P2);
      times(S, dB, T);
      launch_zaxpy(s0, lc, bstride, 1.0, T, P2);
      times(dD, X, T);
      launch_zaxpy(s0, lc, bstride, -dk, T, P2);
      lu_solve_batched<double>(s0, lc, d, D, ipiv, P2, nrhs, bstride, false);
      MH_TRY(check_launch(ctx, "frequency-derivative solve"));
    } else {
      // sigma = D^-1 b, phi = S sigma;  dsigma = D^-1 (db - dD sigma), dphi = dS sigma + S dsigma
      MH_CUDA(ctx, cudaMemcpyAsync(X, B, sizeof(double2) * bstride, cudaMemcpyDeviceToDevice, s0));
      MH_TRY(solve_core(ctx, d, D, X, nrhs, bstride, MH_PREC_FP64, false));
      MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)n, &ipiv));
      MH_CUDA(ctx, cudaMemcpyAsync(R, dB, sizeof(double2) * bstride, cudaMemcpyDeviceToDevice, s0));
      times(dD, X, T);
      launch_zaxpy(s0, lc, bstride, -dk, T, R);
      lu_solve_batched<double>(s0, lc, d, D, ipiv, R, nrhs, bstride, false);  // dsigma
      times(dS, X, T);
      MH_CUDA(ctx, cudaMemsetAsync(P2, 0, sizeof(double2) * bstride, s0));
      launch_zaxpy(s0, lc, bstride, dk, T, P2);
      times(S, R, T);
      launch_zaxpy(s0, lc, bstride, 1.0, T, P2);                               // dphi
      times(S, X, T);
      MH_CUDA(ctx, cudaMemcpyAsync(X, T, sizeof(double2) * bstride, cudaMemcpyDeviceToDevice, s0));  // phi
      MH_TRY(check_launch(ctx, "frequency-derivative solve"));
    }
    // p = i rho omega phi;  dp = i rho omega (phi / omega + dphi): forces of phi and of phi / omega + dphi
    launch_zaxpy(s0, lc, bstride, 1.0 / om, X, P2);
    if (n_inf > 0) {
      launch_forces(s0, lc, eg, 1, om_d + w, rho, g, (int)nrhs, X, bstride, (int)n_inf, inf_d, (int)n_beta, beta_d,
                    F + w * n_inf * nrhs, FK + w * n_inf * nb1);
      launch_forces(s0, lc, eg, 1, om_d + w, rho, g, (int)nrhs, P2, bstride, (int)n_inf, inf_d, 0, nullptr,
                    dF + w * n_inf * nrhs, nullptr);
      MH_TRY(check_launch(ctx, "forces"));
    }
  }
  std::vector<double2> hF((size_t)(n_omega * ninf1 * nrhs)), hdF(hF.size()), hFK((size_t)(n_omega * ninf1 * nb1));
  if (n_inf > 0) {
    MH_CUDA(ctx, cudaMemcpyAsync(hF.data(), F, sizeof(double2) * hF.size(), cudaMemcpyDeviceToHost, s0));
    MH_CUDA(ctx, cudaMemcpyAsync(hdF.data(), dF, sizeof(double2) * hdF.size(), cudaMemcpyDeviceToHost, s0));
    if (n_beta > 0) MH_CUDA(ctx, cudaMemcpyAsync(hFK.data(), FK, sizeof(double2) * hFK.size(), cudaMemcpyDeviceToHost, s0));
  }
  MH_TRY(sync(ctx, "frequency derivative"));
  // pack; A = Re F / w^2, B = Im F / w (problems_and_results.jl:207-208) and their omega-derivatives;
  // Froude-Krylov: p = rho g e^{kz} e^{i k wbar}, dp/domega = p (z + i wbar) 2 omega / g (waves.jl:259-264)
  std::vector<double> hA((size_t)(n_inf * n_rad * n_omega)), hB(hA.size()), hdA(hA.size()), hdB(hA.size());
  std::vector<double2> hd((size_t)(n_inf * n_omega * n_beta)), hk(hd.size()), he(hd.size()), hdd(hd.size()),
      hdk(hd.size()), hde(hd.size());
  for (int64_t w = 0; w < n_omega; ++w) {
    const double om = omegas[w], k = om * om / g, dk = 2.0 * om / g;
    for (int64_t i = 0; i < n_inf; ++i) {
      for (int64_t r = 0; r < n_rad; ++r) {
        const double2 f = hF[(w * n_inf + i) * nrhs + r], df = hdF[(w * n_inf + i) * nrhs + r];
        const size_t o = (size_t)(i + n_inf * (r + n_rad * w));
        hA[o] = f.x / (om * om);
        hB[o] = f.y / om;
        hdA[o] = df.x / (om * om) - 2.0 * f.x / (om * om * om);
        hdB[o] = df.y / om - f.y / (om * om);
      }
      const double* dof = hdofs.data() + (size_t)inf_idx[i] * n * 3;
      for (int64_t b = 0; b < n_beta; ++b) {
        const double2 fd = hF[(w * n_inf + i) * nrhs + n_rad + b], dfd = hdF[(w * n_inf + i) * nrhs + n_rad + b];
        const double2 fk = hFK[(w * n_inf + i) * n_beta + b];
        const double cb = std::cos(betas[b]), sb = std::sin(betas[b]);
        double dkr = 0.0, dki = 0.0;
        for (int64_t j = 0; j < nh; ++j) {
          const double wbar = hC[3 * j] * cb + hC[3 * j + 1] * sb, z = hC[3 * j + 2];
          const double a = rho * g * std::exp(k * z);
          const double pr = a * std::cos(k * wbar), pi = a * std::sin(k * wbar);
          const double disp = hN[3 * j] * dof[3 * j] + hN[3 * j + 1] * dof[3 * j + 1] + hN[3 * j + 2] * dof[3 * j + 2];
          const double f = -disp * hAr[j];
          // (pr + i pi) (z + i wbar) dk
          dkr += (pr * z - pi * wbar) * dk * f;
          dki += (pr * wbar + pi * z) * dk * f;
        }
        const size_t o = (size_t)(i + n_inf * (w + n_omega * b));
        hd[o] = fd;
        hk[o] = fk;
        he[o] = make_double2(fd.x + fk.x, fd.y + fk.y);
        hdd[o] = dfd;
        hdk[o] = make_double2(dkr, dki);
        hde[o] = make_double2(dfd.x + dkr, dfd.y + dki);
      }
    }
  }
  MH_TRY(put_out(ctx, added_mass, hA.data(), hA.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, radiation_damping, hB.data(), hB.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, diffraction_force, hd.data(), hd.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, froude_krylov_force, hk.data(), hk.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, excitation_force, he.data(), he.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, d_added_mass, hdA.data(), hdA.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, d_radiation_damping, hdB.data(), hdB.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, d_diffraction_force, hdd.data(), hdd.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, d_froude_krylov_force, hdk.data(), hdk.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, d_excitation_force, hde.data(), hde.size() * sizeof(double2), mem));
  return sync(ctx, "frequency-derivative outputs");
}

int mh_wu_wave_terms(mh_context* ctx, int64_t m, const double* hh, const double* vv, double* out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (m <= 0 || !hh || !vv || !out) return fail(ctx, MH_ERR_ARG, "bad wave-term arguments");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  MH_TRY(set_device(ctx));
  double *in, *o;
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(2 * m), &in));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(6 * m), &o));
  MH_TRY(copy_in(ctx, in, hh, sizeof(double) * m, mem));
  MH_TRY(copy_in(ctx, in + m, vv, sizeof(double) * m, mem));
  launch_wu_points(ctx->stream, ctx->lc(), m, in, in + m, (double2*)o);
  MH_TRY(check_launch(ctx, "wu wave terms"));
  MH_TRY(copy_out(ctx, out, o, sizeof(double) * 6 * m, mem));
  return sync(ctx, "wu wave terms");
}

int mh_bessel01_points(mh_context* ctx, int64_t m, const double* x, double* out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (m <= 0 || !x || !out) return fail(ctx, MH_ERR_ARG, "bad Bessel arguments");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  MH_TRY(set_device(ctx));
  double *in, *o;
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)m, &in));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(4 * m), &o));
  MH_TRY(copy_in(ctx, in, x, sizeof(double) * m, mem));
  launch_bessel01_points(ctx->stream, ctx->lc(), m, in, o);
  MH_TRY(check_launch(ctx, "Bessel points"));
  MH_TRY(copy_out(ctx, out, o, sizeof(double) * 4 * m, mem));
  return sync(ctx, "Bessel points");
}

int mh_exact_wave_terms(mh_context* ctx, int64_t m, const double* r, const double* z, double rtol, double atol,
                        double* out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (m <= 0 || !r || !z || !out) return fail(ctx, MH_ERR_ARG, "bad wave-term arguments");
  if (!(rtol >= 0) || !(atol >= 0) || (rtol == 0 && atol == 0))
    return fail(ctx, MH_ERR_ARG, "quadrature tolerances must be >= 0 and not both zero");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  MH_TRY(set_device(ctx));
  double *in, *o;
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(2 * m), &in));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(4 * m), &o));
  MH_TRY(copy_in(ctx, in, r, sizeof(double) * m, mem));
  MH_TRY(copy_in(ctx, in + m, z, sizeof(double) * m, mem));
  launch_exact_points(ctx->stream, ctx->lc(), m, in, in + m, rtol, atol, (double2*)o);
  MH_TRY(check_launch(ctx, "exact wave terms"));
  MH_TRY(copy_out(ctx, out, o, sizeof(double) * 4 * m, mem));
  return sync(ctx, "exact wave terms");
}

int mh_profile_enable(mh_context* ctx, int enable) {
  if (!ctx) return MH_ERR_ARG;
  profiler_enable(ctx->prof, enable != 0);
  return MH_OK;
}

int mh_profile_reset(mh_context* ctx) {
  if (!ctx) return MH_ERR_ARG;
  MH_TRY(set_device(ctx));
  MH_TRY(sync(ctx, "profile reset"));
  profiler_reset(ctx->prof);
  return MH_OK;
}

int mh_profile_read(mh_context* ctx, int64_t capacity, char* names, double* total_ms, int64_t* launches,
                    int64_t* n_groups) {
  if (!ctx || !n_groups || capacity < 0) return MH_ERR_ARG;
  MH_TRY(set_device(ctx));
  MH_CUDA(ctx, cudaDeviceSynchronize());
  profiler_read(ctx->prof, capacity, names, total_ms, launches, n_groups);
  return MH_OK;
}

int mh_probe_fma_peaks(mh_context* ctx, double* fp64_tflops, double* fp32_tflops) {
  if (!ctx) return MH_ERR_ARG;
  MH_TRY(set_device(ctx));
  int rc = probe_fma_peaks(ctx->stream, fp64_tflops, fp32_tflops);
  if (rc) return fail(ctx, rc, "FMA probe failed");
  return MH_OK;
}

int mh_probe_wait_timeout(mh_context* ctx, uint32_t polls) {
  if (!ctx) return MH_ERR_ARG;
  if (polls < 1 || polls > (1u << 20)) return fail(ctx, MH_ERR_ARG, "polls must be 1..2^20 (got %u)", polls);
  MH_TRY(set_device(ctx));
  int timed_out = 0;
  int rc = probe_wait_timeout(ctx->stream, polls, &timed_out);
  if (rc) return fail(ctx, rc, "wait-timeout probe: %s", cudaGetErrorString(cudaGetLastError()));
  if (timed_out) return fail(ctx, MH_ERR_TIMEOUT, "a bounded completion wait gave up after %u polls", polls);
  return MH_OK;
}

int mh_tile_table_set(mh_context* ctx, int64_t n_entries, const int64_t* n_max, const int32_t* choices) {
  if (!ctx) return MH_ERR_ARG;
  if (n_entries < 0 || n_entries > kMaxTileEntries)
    return fail(ctx, MH_ERR_ARG, "a tile table holds 0..%d entries (got %lld)", kMaxTileEntries, (long long)n_entries);
  if (n_entries > 0 && (!n_max || !choices)) return fail(ctx, MH_ERR_ARG, "tile table arrays must not be NULL");
  TileTable t;
  for (int64_t q = 0; q < n_entries; ++q) {
    if (n_max[q] < 1 || (q > 0 && n_max[q] <= n_max[q - 1]))
      return fail(ctx, MH_ERR_ARG, "tile table bucket bounds must be positive and ascending");
    const int32_t* c = choices + 4 * q;
    for (int f = 0; f < 4; ++f)
      if (c[f] < 1 || c[f] > 8) return fail(ctx, MH_ERR_ARG, "tile table entry %lld field %d = %d is outside 1..8",
                                            (long long)q, f, c[f]);
    t.n_max[q] = n_max[q];
    t.c[q].oz_group = c[0];
    t.c[q].bx_group = c[1];
    t.c[q].cluster_f64 = c[2];
    t.c[q].cluster_f32 = c[3];
  }
  t.n_entries = (int)n_entries;
  ctx->tiles = t;
  return MH_OK;
}

int mh_tile_table_get(mh_context* ctx, int64_t capacity, int64_t* n_max, int32_t* choices, int64_t* n_entries) {
  if (!ctx) return MH_ERR_ARG;
  if (!n_entries) return fail(ctx, MH_ERR_ARG, "n_entries must not be NULL");
  const TileTable& t = ctx->tiles;
  *n_entries = t.n_entries;
  if (t.n_entries == 0) return MH_OK;
  if (capacity < t.n_entries || !n_max || !choices)
    return fail(ctx, MH_ERR_ARG, "the tile table has %d entries; capacity %lld", t.n_entries, (long long)capacity);
  for (int q = 0; q < t.n_entries; ++q) {
    n_max[q] = t.n_max[q];
    choices[4 * q + 0] = t.c[q].oz_group;
    choices[4 * q + 1] = t.c[q].bx_group;
    choices[4 * q + 2] = t.c[q].cluster_f64;
    choices[4 * q + 3] = t.c[q].cluster_f32;
  }
  return MH_OK;
}

int mh_autotune(mh_context* ctx, int precision, int64_t n_sizes, const int64_t* sizes, int64_t batch, int reps,
                double* ms_best, double* ms_default) {
  NvtxRange nvtx_range("mh_autotune");
  if (!ctx) return MH_ERR_ARG;
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC)
    return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (n_sizes < 1 || n_sizes > kMaxTileEntries || !sizes)
    return fail(ctx, MH_ERR_ARG, "autotune needs 1..%d matrix orders", kMaxTileEntries);
  for (int64_t q = 0; q < n_sizes; ++q)
    if (sizes[q] < 32 || sizes[q] > kMaxOrder || (q > 0 && sizes[q] <= sizes[q - 1]))
      return fail(ctx, MH_ERR_ARG, "autotune orders must ascend within 32..%lld", (long long)kMaxOrder);
  if (batch < 1 || batch > 64) return fail(ctx, MH_ERR_ARG, "autotune batch must be 1..64 (got %lld)", (long long)batch);
  if (reps < 1 || reps > 20) return fail(ctx, MH_ERR_ARG, "autotune reps must be 1..20 (got %d)", reps);
  MH_TRY(set_device(ctx));
  const TileTable saved = ctx->tiles;
  // candidates: the cluster bound of the panel and, for the tensor-core updates, the
  // column tiles per CTA; the first candidate is the default shape
  std::vector<TileChoice> cands;
  const int caps[3] = {8, 4, 2}, groups[4] = {4, 1, 2, 8};
  for (int cap : caps) {
    if (precision == MH_PREC_FP64) {
      TileChoice c;
      c.cluster_f64 = cap;
      cands.push_back(c);
      continue;
    }
    for (int gr : groups) {
      TileChoice c;
      if (precision == MH_PREC_MIXED) {
        c.bx_group = gr;
        c.cluster_f32 = cap;
      } else {
        c.oz_group = gr;
        c.cluster_f64 = cap;
      }
      cands.push_back(c);
    }
  }
  TileTable out;
  out.n_entries = (int)n_sizes;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  MH_CUDA(ctx, cudaEventCreate(&e0));
  MH_CUDA(ctx, cudaEventCreate(&e1));
  int rc = MH_OK;
  for (int64_t q = 0; q < n_sizes && rc == MH_OK; ++q) {
    const int64_t n = sizes[q], nn = n * n;
    out.n_max[q] = q + 1 < n_sizes ? (int64_t)std::sqrt((double)sizes[q] * (double)sizes[q + 1]) : INT64_MAX;
    TileChoice base = saved.lookup(n);
    const BatchDesc d{n, batch, nn};
    int32_t *ipiv = nullptr, *info = nullptr;
    rc = ws_get_t(ctx, kSlotIpiv, (size_t)(n * batch), &ipiv);
    if (!rc) rc = ws_get_t(ctx, kSlotInfo, (size_t)batch, &info);
    double2* A64 = nullptr;
    float2* A32 = nullptr;
    unsigned char* ws = nullptr;
    int* flag = nullptr;
    if (!rc && precision == MH_PREC_MIXED) {
      rc = ws_get_t(ctx, kSlotLU32, (size_t)(nn * batch), &A32);
      const size_t wsb = bx3_workspace_bytes(n, batch);
      if (!rc) rc = ws_get_t(ctx, kSlotBx3, wsb + 256, &ws);
      if (!rc) flag = reinterpret_cast<int*>(ws + wsb);
    } else if (!rc) {
      rc = ws_get_t(ctx, kSlotD, (size_t)(nn * batch), &A64);
      if (!rc && precision == MH_PREC_FP64_TC) {
        const size_t wsb = ozaki_workspace_bytes(n, batch);
        rc = ws_get_t(ctx, kSlotOzaki, wsb + 256, &ws);
        if (!rc) flag = reinterpret_cast<int*>(ws + wsb);
      }
    }
    double best_t = 1e300, def_t = 1e300;
    TileChoice best_c = cands[0];
    for (size_t ci = 0; ci < cands.size() && !rc; ++ci) {
      TileChoice c = base;
      if (precision == MH_PREC_MIXED) {
        c.bx_group = cands[ci].bx_group;
        c.cluster_f32 = cands[ci].cluster_f32;
      } else {
        c.oz_group = precision == MH_PREC_FP64_TC ? cands[ci].oz_group : c.oz_group;
        c.cluster_f64 = cands[ci].cluster_f64;
      }
      ctx->tiles.n_entries = 1;
      ctx->tiles.n_max[0] = INT64_MAX;
      ctx->tiles.c[0] = c;
      double t = 0.0;
      rc = precision == MH_PREC_MIXED
               ? time_factorization<float>(ctx, d, A32, ipiv, info, ws, flag, reps, e0, e1, &t)
               : time_factorization<double>(ctx, d, A64, ipiv, info, ws, flag, reps, e0, e1, &t);
      if (rc) break;
      if (ci == 0) def_t = t;
      if (t < best_t) {
        best_t = t;
        best_c = c;
      }
    }
    if (rc) break;
    // keep the default shape unless another one is faster by more than the timing noise
    if (best_t > 0.98 * def_t) {
      best_t = def_t;
      best_c = base;
      if (precision == MH_PREC_MIXED) {
        best_c.bx_group = cands[0].bx_group;
        best_c.cluster_f32 = cands[0].cluster_f32;
      } else {
        if (precision == MH_PREC_FP64_TC) best_c.oz_group = cands[0].oz_group;
        best_c.cluster_f64 = cands[0].cluster_f64;
      }
    }
    out.c[q] = best_c;
    if (ms_best) ms_best[q] = best_t;
    if (ms_default) ms_default[q] = def_t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tiles = rc ? saved : out;
  return rc;
}

int mh_batch_hydrodynamic_coefficients(mh_context* ctx, int64_t n_bodies, mh_mesh* const* meshes,
                                       const int64_t* n_omega, const double* omegas, double rho, double g,
                                       uint32_t gfs, int direct, int64_t n_dofs, const double* const* dofs,
                                       int64_t n_rad, const int32_t* rad_idx, int64_t n_inf, const int32_t* inf_idx,
                                       int64_t n_beta, const double* betas, int precision, int n_streams,
                                       double* added_mass, double* radiation_damping, double* diffraction_force,
                                       double* froude_krylov_force, double* excitation_force, int mem) {
  NvtxRange nvtx_range("mh_batch_hydrodynamic_coefficients");
  if (!ctx) return MH_ERR_ARG;
  if (n_bodies <= 0 || !meshes || !n_omega || !omegas) return fail(ctx, MH_ERR_ARG, "need at least one body");
  if (n_rad < 0 || n_inf < 0 || n_beta < 0 || n_dofs < 0) return fail(ctx, MH_ERR_ARG, "negative counts");
  if (n_rad + n_beta == 0) return fail(ctx, MH_ERR_ARG, "nothing to solve: no radiating dof and no wave direction");
  if ((n_rad > 0 || n_inf > 0) && (!dofs || n_dofs <= 0)) return fail(ctx, MH_ERR_ARG, "dof fields required");
  MH_TRY(check_gfs(ctx, gfs));
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (!(rho > 0) || !(g > 0)) return fail(ctx, MH_ERR_ARG, "rho and g must be positive");
  for (int64_t q = 0; q < n_rad; ++q)
    if (rad_idx[q] < 0 || rad_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "radiating dof index out of range");
  for (int64_t q = 0; q < n_inf; ++q)
    if (inf_idx[q] < 0 || inf_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "influenced dof index out of range");
  int64_t total_w = 0;
  for (int64_t b = 0; b < n_bodies; ++b) {
    if (!meshes[b] || meshes[b]->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh %lld does not belong to this context", (long long)b);
    if (n_omega[b] <= 0) return fail(ctx, MH_ERR_ARG, "body %lld has no wave frequency", (long long)b);
    if (meshes[b]->n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "body %lld exceeds %lld panels", (long long)b, (long long)kMaxOrder);
    total_w += n_omega[b];
  }
  for (int64_t w = 0; w < total_w; ++w)
    if (!(omegas[w] > 0)) return fail(ctx, MH_ERR_ARG, "wave frequencies must be positive");
  MH_TRY(set_device(ctx));
  const int S = n_streams > 0 ? (int)std::min(n_streams, 16) : 4;
  BatchOpts o{gfs, direct ? 1 : 0, precision, 2, rho, g, n_dofs, n_rad, n_inf, n_beta, n_rad + n_beta};

  // cache key: everything the captured graph bakes in
  // with profiling on, the schedule runs uncaptured on one stream so that every launch is
  // timed by its own events (kernel shares of the batch); the graph is not built
  const bool profiling = profiler_on(ctx->prof);
  std::vector<double> key = {(double)n_bodies, (double)gfs, (double)o.direct, (double)precision, (double)S, rho, g,
                             (double)n_dofs, (double)n_rad, (double)n_inf, (double)n_beta, ctx->quad_rtol,
                             ctx->quad_atol, profiling ? 1.0 : 0.0};
  for (int64_t b = 0; b < n_bodies; ++b) {
    key.push_back((double)(uintptr_t)meshes[b]);
    key.push_back((double)n_omega[b]);
    key.push_back((double)meshes[b]->n_hull);  // the lid split is baked into the epilogue launches
  }
  for (int64_t q = 0; q < n_rad; ++q) key.push_back(rad_idx[q]);
  for (int64_t q = 0; q < n_inf; ++q) key.push_back(inf_idx[q]);
  for (int q = 0; q < ctx->tiles.n_entries; ++q) {  // launch shapes are baked into the graph
    const TileChoice& t = ctx->tiles.c[q];
    key.insert(key.end(), {(double)ctx->tiles.n_max[q], (double)t.oz_group, (double)t.bx_group,
                           (double)t.cluster_f64, (double)t.cluster_f32});
  }
  BatchCache* bc = ctx->batch;
  if (!bc || bc->key != key) {
    delete bc;
    ctx->batch = nullptr;
    bc = new BatchCache();
    bc->device = ctx->device;
    bc->key = key;
    bc->bodies.resize(n_bodies);
    int64_t w_off = 0;
    for (int64_t b = 0; b < n_bodies; ++b) {
      BodyPlan& p = bc->bodies[b];
      p.m = meshes[b];
      p.n = meshes[b]->n;
      p.nw = n_omega[b];
      p.w_off = w_off;
      w_off += p.nw;
      const double n = (double)p.n;
      p.cost = (double)p.nw * (precision == MH_PREC_FP64 ? n * n * n : n * n * n / 20.0 + 60.0 * n * n);
    }
    // longest processing time first onto the least-loaded stream
    std::vector<int64_t> order(n_bodies);
    for (int64_t b = 0; b < n_bodies; ++b) order[b] = b;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t c) { return bc->bodies[a].cost > bc->bodies[c].cost; });
    std::vector<double> load(S, 0.0);
    for (int64_t b : order) {
      int best = 0;
      for (int q = 1; q < S; ++q) if (load[q] < load[best]) best = q;
      bc->bodies[b].stream = best;
      load[best] += bc->bodies[b].cost;
    }
    size_t dev_bytes = 0, host_bytes = 0;
    std::vector<size_t> doff(n_bodies), hoff(n_bodies);
    for (int64_t b = 0; b < n_bodies; ++b) {
      doff[b] = dev_bytes;
      dev_bytes += layout_body(bc->bodies[b], o, nullptr);
      hoff[b] = host_bytes;
      host_bytes += pinned_body(bc->bodies[b], o, nullptr);
    }
    size_t free_b = 0, total_b = 0;
    MH_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    if (dev_bytes > (size_t)(0.8 * (double)free_b)) {
      delete bc;
      return fail(ctx, MH_ERR_NOMEM, "batch needs %.1f GB of device memory, %.1f GB free", dev_bytes / 1e9,
                  free_b / 1e9);
    }
    MH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (cudaMalloc(&bc->arena, dev_bytes) != cudaSuccess || cudaMallocHost((void**)&bc->pinned, host_bytes) != cudaSuccess) {
      delete bc;
      return fail(ctx, MH_ERR_NOMEM, "batch allocation of %.1f GB failed", dev_bytes / 1e9);
    }
    for (int64_t b = 0; b < n_bodies; ++b) {
      layout_body(bc->bodies[b], o, (char*)bc->arena + doff[b]);
      pinned_body(bc->bodies[b], o, bc->pinned + hoff[b]);
    }
    while ((int)ctx->side.size() < S - 1) {
      cudaStream_t st;
      MH_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      ctx->side.push_back(st);
    }
    bc->order = order;
    if (profiling) {
      ctx->batch = bc;
    } else {
      // capture the schedule
      cudaStream_t s0 = ctx->stream;
      std::vector<cudaEvent_t> ev(S);
      for (auto& e : ev) MH_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      LaunchCounter cap{&bc->graph_kernels, nullptr, &ctx->tiles};
      MH_CUDA(ctx, cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
      cudaEventRecord(ev[0], s0);
      for (int q = 1; q < S; ++q) cudaStreamWaitEvent(ctx->side[q - 1], ev[0], 0);
      for (int64_t b : order) {
        BodyPlan& p = bc->bodies[b];
        enqueue_body(ctx, cap, p.stream == 0 ? s0 : ctx->side[p.stream - 1], p, o);
      }
      for (int q = 1; q < S; ++q) {
        cudaEventRecord(ev[q], ctx->side[q - 1]);
        cudaStreamWaitEvent(s0, ev[q], 0);
      }
      cudaGraph_t graph = nullptr;
      cudaError_t ce = cudaStreamEndCapture(s0, &graph);
      for (auto& e : ev) cudaEventDestroy(e);
      if (ce != cudaSuccess || !graph) {
        delete bc;
        return fail(ctx, MH_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
      }
      ce = cudaGraphInstantiate(&bc->exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        delete bc;
        return fail(ctx, MH_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ce));
      }
      ctx->batch = bc;
    }
  }
  // per-call parameters -> the bodies' device buffers (outside the graph)
  for (int64_t b = 0; b < n_bodies; ++b) {
    BodyPlan& p = bc->bodies[b];
    double* hp = p.hparams;
    std::memcpy(hp, omegas + p.w_off, sizeof(double) * p.nw);
    for (int64_t w = 0; w < p.nw; ++w) hp[p.nw + w] = omegas[p.w_off + w] * omegas[p.w_off + w] / g;
    if (n_beta) std::memcpy(hp + 2 * p.nw, betas, sizeof(double) * n_beta);
    int32_t* hi = (int32_t*)(hp + 2 * p.nw + n_beta);
    for (int64_t q = 0; q < n_rad; ++q) hi[q] = rad_idx[q];
    for (int64_t q = 0; q < n_inf; ++q) hi[n_rad + q] = inf_idx[q];
    MH_CUDA(ctx, cudaMemcpyAsync(p.params, hp, sizeof(double) * p.nparams, cudaMemcpyHostToDevice, ctx->stream));
    if (n_dofs > 0) {
      const size_t db = sizeof(double) * n_dofs * p.n * 3;
      if (mem == MH_MEM_HOST) {
        std::memcpy(p.hdofs, dofs[b], db);
        MH_CUDA(ctx, cudaMemcpyAsync(p.dofs, p.hdofs, db, cudaMemcpyHostToDevice, ctx->stream));
      } else {
        MH_CUDA(ctx, cudaMemcpyAsync(p.dofs, dofs[b], db, cudaMemcpyDeviceToDevice, ctx->stream));
      }
    }
  }
  if (bc->exec) {
    MH_CUDA(ctx, cudaGraphLaunch(bc->exec, ctx->stream));
    ctx->launches += bc->graph_kernels;
  } else {
    for (int64_t b : bc->order) enqueue_body(ctx, ctx->lc(), ctx->stream, bc->bodies[b], o);
  }
  MH_TRY(sync(ctx, "batch graph"));
  for (auto& p : bc->bodies) MH_TRY(finish_body(ctx, p, o));
  // pack per body (n_U = 1), bodies concatenated along the frequency axis
  std::vector<double> hA((size_t)(n_inf * n_rad * total_w)), hB(hA.size());
  std::vector<double2> hd((size_t)(n_inf * total_w * n_beta)), hk(hd.size()), he(hd.size());
  for (auto& p : bc->bodies) {
    for (int64_t w = 0; w < p.nw; ++w) {
      const double om = omegas[p.w_off + w];
      for (int64_t i = 0; i < n_inf; ++i) {
        for (int64_t r = 0; r < n_rad; ++r) {
          double2 f = p.hF[(w * n_inf + i) * o.nrhs + r];
          hA[(size_t)(n_inf * n_rad * p.w_off) + i + n_inf * (r + n_rad * w)] = f.x / (om * om);
          hB[(size_t)(n_inf * n_rad * p.w_off) + i + n_inf * (r + n_rad * w)] = f.y / om;
        }
        for (int64_t bb = 0; bb < n_beta; ++bb) {
          double2 fd = p.hF[(w * n_inf + i) * o.nrhs + n_rad + bb];
          double2 fk = p.hFK[(w * n_inf + i) * n_beta + bb];
          size_t q = (size_t)(n_inf * n_beta * p.w_off) + (size_t)(i + n_inf * (w + p.nw * bb));
          hd[q] = fd;
          hk[q] = fk;
          he[q] = make_double2(fd.x + fk.x, fd.y + fk.y);
        }
      }
    }
  }
  MH_TRY(put_out(ctx, added_mass, hA.data(), hA.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, radiation_damping, hB.data(), hB.size() * sizeof(double), mem));
  MH_TRY(put_out(ctx, diffraction_force, hd.data(), hd.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, froude_krylov_force, hk.data(), hk.size() * sizeof(double2), mem));
  MH_TRY(put_out(ctx, excitation_force, he.data(), he.size() * sizeof(double2), mem));
  return sync(ctx, "batch outputs");
}

int mh_batch_release(mh_context* ctx) {
  if (!ctx) return MH_ERR_ARG;
  MH_TRY(set_device(ctx));
  MH_TRY(sync(ctx, "batch release"));
  delete ctx->batch;
  ctx->batch = nullptr;
  return MH_OK;
}

}  // extern "C"

namespace {

// Reverse-mode product of the zero-speed radiation sweep: J = sum over omega, influenced q
// and radiating r of abar[q, r, w] A[q, r, w] + bbar[q, r, w] B[q, r, w] (host cotangents,
// n_inf x n_rad x n_omega, column-major) and its gradient with respect to every panel's
// centre, normal, area, Birk corners and the dof fields.  The gradient of the dof fields
// stays on the device (n_dofs x n x 3, *gd_out, workspace memory).
int hydro_vjp_core(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                   uint32_t gfs, int64_t n_dofs, const double* dofs, int64_t n_rad, const int32_t* rad_idx,
                   int64_t n_inf, const int32_t* inf_idx, const double* abar, const double* bbar, int64_t n_beta,
                   const double* betas, const double* fbar, int precision, double* J, double* grad_centers,
                   double* grad_normals, double* grad_areas, double* grad_vertices, const double** gd_out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (!m || m->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh does not belong to this context");
  if (n_omega <= 0 || !omegas) return fail(ctx, MH_ERR_ARG, "need at least one wave frequency");
  if (n_rad < 0 || n_beta < 0 || n_rad + n_beta <= 0 || n_inf <= 0 || (n_rad && !rad_idx) || !inf_idx ||
      (n_beta && (!betas || !fbar)))
    return fail(ctx, MH_ERR_ARG, "need influenced dofs and radiating dofs or headings");
  if (n_rad > 64 || n_inf > 64 || n_beta > 64) return fail(ctx, MH_ERR_ARG, "at most 64 dofs and 64 headings each");
  if (m->n_hull != m->n) return fail(ctx, MH_ERR_UNSUPPORTED, "the adjoint does not cover meshes with a lid");
  if (!dofs || n_dofs <= 0) return fail(ctx, MH_ERR_ARG, "dof fields required");
  const uint32_t allowed = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE | MH_GF_WU;
  if (gfs == 0 || (gfs & ~allowed))
    return fail(ctx, MH_ERR_UNSUPPORTED, "the adjoint covers the Birk Rankine family and GFWu (got 0x%x)", gfs);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC) return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (!(rho > 0) || !(g > 0)) return fail(ctx, MH_ERR_ARG, "rho and g must be positive");
  for (int64_t q = 0; q < n_rad; ++q)
    if (rad_idx[q] < 0 || rad_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "radiating dof index out of range");
  for (int64_t q = 0; q < n_inf; ++q)
    if (inf_idx[q] < 0 || inf_idx[q] >= n_dofs) return fail(ctx, MH_ERR_ARG, "influenced dof index out of range");
  for (int64_t w = 0; w < n_omega; ++w)
    if (!(omegas[w] > 0)) return fail(ctx, MH_ERR_ARG, "wave frequencies must be positive");
  if (m->n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "mesh exceeds %lld panels", (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const int64_t n = m->n, nr = n_rad, ni = n_inf, nb = n_beta, ncol = n_rad + n_beta;
  const size_t nn = (size_t)n * n;
  cudaStream_t st = ctx->stream;
  const LaunchCounter lc = ctx->lc();
  // frequencies are processed in chunks sized by free memory, like the sweep: assembly,
  // factorization and both solves run batched over a chunk, the adjoint kernels per frequency
  size_t free_b = 0, total_b = 0;
  MH_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
  size_t per_w = nn * sizeof(double2) * 2 + (size_t)n * ncol * sizeof(double2) * 6;
  if (precision == MH_PREC_MIXED) per_w += nn * sizeof(float2) + (size_t)n * ncol * sizeof(double2) * 3;
  const size_t budget = std::min<size_t>(free_b / 2, (size_t)48 << 30);
  const int64_t chunk = std::min<int64_t>(n_omega, (int64_t)std::max<size_t>(1, budget / per_w));
  const int64_t bstride = n * ncol;
  double *SR, *DR, *RS, *RD, *grad, *small, *dofs_d;
  double2 *S, *D, *B, *X, *lam, *t, *work, *F, *FK, *cw;
  int32_t *ipiv, *info;
  MH_TRY(ws_get_t(ctx, kSlotSR, nn, &SR));
  MH_TRY(ws_get_t(ctx, kSlotDR, nn, &DR));
  MH_TRY(ws_get_t(ctx, kSlotRS, nn, &RS));
  MH_TRY(ws_get_t(ctx, kSlotRD, nn, &RD));
  MH_TRY(ws_get_t(ctx, kSlotS, nn * chunk, &S));
  MH_TRY(ws_get_t(ctx, kSlotD, nn * chunk, &D));
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(bstride * chunk), &B));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(bstride * chunk), &X));
  MH_TRY(ws_get_t(ctx, kSlotLam, (size_t)(bstride * chunk), &lam));
  MH_TRY(ws_get_t(ctx, kSlotT, (size_t)(bstride * chunk), &t));
  MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, ncol, chunk), &work));
  MH_TRY(ws_get_t(ctx, kSlotF, (size_t)(ni * ncol * n_omega), &F));
  MH_TRY(ws_get_t(ctx, kSlotFK, (size_t)(ni * std::max<int64_t>(nb, 1) * n_omega), &FK));
  MH_TRY(ws_get_t(ctx, kSlotCw, (size_t)(ni * ncol * n_omega), &cw));  // not kSlotNorm: the refinement owns it
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)(n * chunk), &ipiv));
  MH_TRY(ws_get_t(ctx, kSlotInfo, (size_t)chunk, &info));
  MH_TRY(ws_get_t(ctx, kSlotGrad, (size_t)((19 + 3 * n_dofs) * n), &grad));
  void* oz_ws = nullptr;  // FP64 LU update on the tensor cores (MH_PREC_FP64_TC)
  int* oz_flag = nullptr;
  if (precision == MH_PREC_FP64_TC) {
    unsigned char* w;
    const size_t wsb = ozaki_workspace_bytes(n, chunk);
    MH_TRY(ws_get_t(ctx, kSlotOzaki, wsb + 256, &w));
    oz_ws = w;
    oz_flag = reinterpret_cast<int*>(w + wsb);
    MH_CUDA(ctx, cudaMemsetAsync(oz_flag, 0, sizeof(int), st));
  }
  // small device block: [omegas | wavenumbers | headings | radiating, influenced dof indices (int32)]
  const size_t nsmall = (size_t)(2 * n_omega + nb) + (size_t)(nr + ni + 1) / 2 + 2;
  MH_TRY(ws_get_t(ctx, kSlotIdx, nsmall, &small));
  if (mem == MH_MEM_DEVICE) {
    dofs_d = (double*)dofs;
  } else {
    MH_TRY(ws_get_t(ctx, kSlotDofs, (size_t)(n_dofs * n * 3), &dofs_d));
    MH_TRY(copy_in(ctx, dofs_d, dofs, sizeof(double) * n_dofs * n * 3, MH_MEM_HOST));
  }
  double* gc = grad;
  double* gn = grad + 3 * n;
  double* ga = grad + 6 * n;
  double* gv = grad + 7 * n;
  double* gd = grad + 19 * n;
  MH_CUDA(ctx, cudaMemsetAsync(grad, 0, sizeof(double) * (19 + 3 * n_dofs) * n, st));
  MH_CUDA(ctx, cudaMemsetAsync(RS, 0, sizeof(double) * nn, st));
  MH_CUDA(ctx, cudaMemsetAsync(RD, 0, sizeof(double) * nn, st));
  const uint32_t stk = gfs & kStaticKinds;
  AssemblyParams pst = make_params(ctx, m, stk, 1, 1, nullptr);
  if (stk) {
    launch_assemble_static(st, lc, pst, SR, DR);
    MH_TRY(check_launch(ctx, "static assembly"));
  }
  AssemblyParams p = make_params(ctx, m, gfs, 1, 1, nullptr);
  // host staging in pageable memory (the mixed solver owns the pinned block)
  std::vector<double> hsmall(nsmall, 0.0);
  for (int64_t w = 0; w < n_omega; ++w) {
    hsmall[w] = omegas[w];
    hsmall[n_omega + w] = omegas[w] * omegas[w] / g;
  }
  for (int64_t b = 0; b < nb; ++b) hsmall[2 * n_omega + b] = betas[b];
  int32_t* hidx = (int32_t*)(hsmall.data() + 2 * n_omega + nb);
  for (int64_t q = 0; q < nr; ++q) hidx[q] = rad_idx[q];
  for (int64_t q = 0; q < ni; ++q) hidx[nr + q] = inf_idx[q];
  MH_CUDA(ctx, cudaMemcpyAsync(small, hsmall.data(), sizeof(double) * nsmall, cudaMemcpyHostToDevice, st));
  // cotangent factors per frequency, n_inf x (n_rad + n_beta): c = abar / w^2 - i bbar / w for the
  // radiating columns (A = Re F / w^2, B = Im F / w), c = conj(fbar) for the headings
  // (J = Re fbar Re Fe + Im fbar Im Fe = Re(conj(fbar) Fe))
  std::vector<double2> hcw((size_t)(ni * ncol * n_omega));
  for (int64_t w = 0; w < n_omega; ++w) {
    for (int64_t r = 0; r < nr; ++r)
      for (int64_t q = 0; q < ni; ++q) {
        const size_t o = (size_t)(q + ni * (r + nr * w));
        hcw[(size_t)(w * ni * ncol + r * ni + q)] = make_double2(abar[o] / (omegas[w] * omegas[w]), -bbar[o] / omegas[w]);
      }
    for (int64_t b = 0; b < nb; ++b)
      for (int64_t q = 0; q < ni; ++q) {
        const size_t o = (size_t)(q + ni * (w + n_omega * b));
        hcw[(size_t)(w * ni * ncol + (nr + b) * ni + q)] = make_double2(fbar[2 * o], -fbar[2 * o + 1]);
      }
  }
  MH_CUDA(ctx, cudaMemcpyAsync(cw, hcw.data(), sizeof(double2) * hcw.size(), cudaMemcpyHostToDevice, st));
  const int64_t nb1 = std::max<int64_t>(nb, 1);
  std::vector<double2> hF((size_t)(ni * ncol * n_omega)), hFK((size_t)(ni * nb1 * n_omega));
  const double* om_d = small;
  const double* ks_d = small + n_omega;
  const double* beta_d = small + 2 * n_omega;
  const int32_t* rad_d = (const int32_t*)(small + 2 * n_omega + nb);
  const int32_t* inf_d = rad_d + nr;
  EpilogueGeom eg{n, m->n_hull, m->C, m->N, m->A, dofs_d};
  for (int64_t w0 = 0; w0 < n_omega; w0 += chunk) {
    const int64_t nw = std::min<int64_t>(chunk, n_omega - w0);
    BatchDesc d{n, nw, (int64_t)nn};
    launch_assemble_wave(st, lc, p, stk ? SR : nullptr, stk ? DR : nullptr, (int)nw, ks_d + w0, S, D, (int64_t)nn,
                         stk ? 0 : 1);
    launch_build_rhs(st, lc, eg, (int)nw, om_d + w0, g, (int)nr, rad_d, (int)nb, beta_d, B, bstride);
    // phi = D^-1 S b, forces, and mu = D^-H conj(w) for the force weights w
    auto forces_and_weights = [&]() {
      launch_forces(st, lc, eg, (int)nw, om_d + w0, rho, g, (int)ncol, X, bstride, (int)ni, inf_d, (int)nb, beta_d,
                    F + w0 * ni * ncol, FK + w0 * ni * nb1);
      for (int64_t w = 0; w < nw; ++w)
        launch_force_weights(st, lc, n, m->N, m->A, dofs_d, inf_d, (int)ni, (int)ncol, cw + (w0 + w) * ni * ncol,
                             omegas[w0 + w], rho, lam + w * bstride);
    };
    bool done = false;
    if (precision == MH_PREC_MIXED) {
      // FP32 factors, both solves refined to FP64 backward error; any column that does not
      // converge sends the whole chunk to the FP64 factorization below (D is left intact)
      float2* LU32;
      double* anrm;
      MH_TRY(factor_mixed(ctx, d, D, &LU32, &anrm));
      zgemm_nn_batched(st, lc, d, S, B, ncol, bstride, X, work);
      bool ok_fwd = false, ok_adj = false;
      MH_TRY(refine_mixed(ctx, d, D, LU32, anrm, X, ncol, bstride, false, &ok_fwd, nullptr));
      if (ok_fwd) {
        forces_and_weights();
        MH_TRY(refine_mixed(ctx, d, D, LU32, anrm, lam, ncol, bstride, true, &ok_adj, nullptr));
      }
      done = ok_fwd && ok_adj;
    }
    if (!done) {
      zgemm_nn_batched(st, lc, d, S, B, ncol, bstride, X, work);
      lu_factor_batched<double>(st, lc, d, D, ipiv, info, oz_ws, oz_flag);
      lu_solve_batched<double>(st, lc, d, D, ipiv, X, ncol, bstride, false);   // X = phi
      forces_and_weights();
      lu_solve_batched<double>(st, lc, d, D, ipiv, lam, ncol, bstride, true);  // mu = D^-H conj(w)
    }
    MH_TRY(check_launch(ctx, "gradient solves"));
    MH_TRY(check_pivots(ctx, d, w0));
    zgemm_adj_batched(st, lc, d, S, lam, ncol, bstride, t, work);              // S^H mu
    launch_conj(st, lc, nw * bstride, t);                                      // t = S^T lam
    launch_conj(st, lc, nw * bstride, lam);                                    // lam = D^-T w
    for (int64_t w = 0; w < nw; ++w) {
      const double om = omegas[w0 + w], k = om * om / g;
      // wave-term gradient (GFWu only) and the frequency-summed Rankine weights, the
      // cotangent factors already in lam; the wave kernel takes up to four columns at a time
      for (int64_t c0 = 0; c0 < ncol; c0 += 4) {
        const int64_t off = w * bstride + c0 * n;
        launch_wave_adjoint(st, lc, p, k, lam + off, B + off, X + off, (int)std::min<int64_t>(4, ncol - c0),
                            make_double2(1.0, 0.0), gc, gn, ga, RS, RD);
      }
      launch_rhs_adjoint(st, lc, n, m->N, m->A, m->C, dofs_d, rad_d, (int)nr, inf_d, (int)ni, (int)nb, beta_d, om,
                         rho, g, cw + (w0 + w) * ni * ncol, X + w * bstride, t + w * bstride, gc, gn, ga, gd);
    }
    MH_TRY(check_launch(ctx, "gradient frequencies"));
  }
  MH_CUDA(ctx, cudaMemcpyAsync(hF.data(), F, sizeof(double2) * hF.size(), cudaMemcpyDeviceToHost, st));
  if (nb) MH_CUDA(ctx, cudaMemcpyAsync(hFK.data(), FK, sizeof(double2) * hFK.size(), cudaMemcpyDeviceToHost, st));
  if (stk) launch_static_adjoint(st, lc, pst, RS, RD, gc, gn, ga, gv);
  MH_TRY(check_launch(ctx, "static adjoint"));
  MH_TRY(sync(ctx, "forces"));
  if (oz_flag) {
    int flag = 0;
    MH_CUDA(ctx, cudaMemcpy(&flag, oz_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  }
  double Jsum = 0.0;
  for (int64_t w = 0; w < n_omega; ++w) {
    const double om = omegas[w];
    for (int64_t q = 0; q < ni; ++q) {
      for (int64_t r = 0; r < nr; ++r) {
        const double2 f = hF[(w * ni + q) * ncol + r];  // influenced q, right-hand side r
        const size_t o = (size_t)(q + ni * (r + nr * w));
        Jsum += abar[o] * f.x / (om * om) + bbar[o] * f.y / om;
      }
      for (int64_t b = 0; b < nb; ++b) {  // excitation = diffraction + Froude-Krylov
        const double2 fd = hF[(w * ni + q) * ncol + nr + b], fk = hFK[(w * ni + q) * nb1 + b];
        const size_t o = (size_t)(q + ni * (w + n_omega * b));
        Jsum += fbar[2 * o] * (fd.x + fk.x) + fbar[2 * o + 1] * (fd.y + fk.y);
      }
    }
  }
  if (J) *J = Jsum;
  MH_TRY(copy_out(ctx, grad_centers, gc, sizeof(double) * 3 * n, mem));
  MH_TRY(copy_out(ctx, grad_normals, gn, sizeof(double) * 3 * n, mem));
  MH_TRY(copy_out(ctx, grad_areas, ga, sizeof(double) * n, mem));
  MH_TRY(copy_out(ctx, grad_vertices, gv, sizeof(double) * 12 * n, mem));
  *gd_out = gd;
  return MH_OK;
}

}  // namespace

extern "C" {

int mh_hydro_gradient(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                      uint32_t gfs, int64_t n_dofs, const double* dofs, int64_t n_obj, const int32_t* obj_idx,
                      int precision, double* J, double* grad_centers, double* grad_normals, double* grad_areas,
                      double* grad_vertices, double* grad_dofs, int mem) {
  NvtxRange nvtx_range("mh_hydro_gradient");
  if (!ctx) return MH_ERR_ARG;
  if (n_obj <= 0 || n_obj > 4 || !obj_idx) return fail(ctx, MH_ERR_ARG, "objective needs 1..4 dofs");
  if (n_omega <= 0 || !omegas) return fail(ctx, MH_ERR_ARG, "need at least one wave frequency");
  // J = sum_w sum_h A_hh + B_hh: identity cotangents on the diagonal
  std::vector<double> bar((size_t)(n_obj * n_obj * n_omega), 0.0);
  for (int64_t w = 0; w < n_omega; ++w)
    for (int64_t h = 0; h < n_obj; ++h) bar[(size_t)(h + n_obj * (h + n_obj * w))] = 1.0;
  const double* gd = nullptr;
  MH_TRY(hydro_vjp_core(ctx, m, n_omega, omegas, rho, g, gfs, n_dofs, dofs, n_obj, obj_idx, n_obj, obj_idx,
                        bar.data(), bar.data(), 0, nullptr, nullptr, precision, J, grad_centers, grad_normals,
                        grad_areas, grad_vertices, &gd, mem));
  for (int64_t h = 0; h < n_obj; ++h)
    MH_TRY(copy_out(ctx, grad_dofs ? grad_dofs + 3 * m->n * h : nullptr, gd + (size_t)obj_idx[h] * m->n * 3,
                    sizeof(double) * 3 * m->n, mem));
  return sync(ctx, "gradient");
}

int mh_hydro_vjp(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                 uint32_t gfs, int64_t n_dofs, const double* dofs, int64_t n_rad, const int32_t* rad_idx,
                 int64_t n_inf, const int32_t* inf_idx, int64_t n_beta, const double* betas,
                 const double* added_mass_bar, const double* radiation_damping_bar, const double* excitation_force_bar,
                 int precision, double* J, double* grad_centers, double* grad_normals, double* grad_areas,
                 double* grad_vertices, double* grad_dofs, int mem) {
  NvtxRange nvtx_range("mh_hydro_vjp");
  if (!ctx) return MH_ERR_ARG;
  if (n_omega <= 0 || !omegas || n_rad < 0 || n_beta < 0 || n_rad + n_beta <= 0 || n_inf <= 0 || n_rad > 64 ||
      n_inf > 64 || n_beta > 64)
    return fail(ctx, MH_ERR_ARG, "need a frequency, 1..64 influenced dofs and 1..64 radiating dofs or headings");
  if ((n_rad && (!added_mass_bar || !radiation_damping_bar)) || (n_beta && (!excitation_force_bar || !betas)))
    return fail(ctx, MH_ERR_ARG, "cotangents must not be NULL");
  if (!m || m->ctx != ctx) return fail(ctx, MH_ERR_ARG, "mesh does not belong to this context");
  const size_t nrb = (size_t)(n_inf * n_rad * n_omega), nfb = (size_t)(2 * n_inf * n_omega * n_beta);
  std::vector<double> ab(nrb), bb(nrb), fb(nfb);
  auto get = [&](double* dst, const double* src, size_t count) -> int {
    if (!count) return MH_OK;
    if (mem == MH_MEM_DEVICE) {
      MH_TRY(set_device(ctx));
      MH_CUDA(ctx, cudaMemcpy(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost));
    } else {
      std::memcpy(dst, src, sizeof(double) * count);
    }
    return MH_OK;
  };
  MH_TRY(get(ab.data(), added_mass_bar, nrb));
  MH_TRY(get(bb.data(), radiation_damping_bar, nrb));
  MH_TRY(get(fb.data(), excitation_force_bar, nfb));
  std::vector<double> hb((size_t)std::max<int64_t>(n_beta, 1));
  MH_TRY(get(hb.data(), betas, (size_t)n_beta));
  const double* gd = nullptr;
  MH_TRY(hydro_vjp_core(ctx, m, n_omega, omegas, rho, g, gfs, n_dofs, dofs, n_rad, rad_idx, n_inf, inf_idx,
                        ab.data(), bb.data(), n_beta, hb.data(), fb.data(), precision, J, grad_centers, grad_normals,
                        grad_areas, grad_vertices, &gd, mem));
  MH_TRY(copy_out(ctx, grad_dofs, gd, sizeof(double) * 3 * m->n * n_dofs, mem));
  return sync(ctx, "vector-Jacobian product");
}

int mh_surrogate_param_count(void) { return kMlpParams; }

int mh_surrogate_set(mh_context* ctx, const float* params) {
  if (!ctx) return MH_ERR_ARG;
  if (!params) return fail(ctx, MH_ERR_ARG, "params must not be NULL");
  MH_TRY(set_device(ctx));
  if (!ctx->mlp) MH_CUDA(ctx, cudaMalloc((void**)&ctx->mlp, sizeof(float) * kMlpParamsPadded));
  float* tmp;
  MH_CUDA(ctx, cudaMallocAsync((void**)&tmp, sizeof(float) * kMlpParamsPadded, ctx->stream));
  MH_CUDA(ctx, cudaMemsetAsync(tmp, 0, sizeof(float) * kMlpParamsPadded, ctx->stream));
  MH_CUDA(ctx, cudaMemcpyAsync(tmp, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, ctx->stream));
  launch_round_bf16(ctx->stream, ctx->lc(), tmp, ctx->mlp);
  MH_CUDA(ctx, cudaFreeAsync(tmp, ctx->stream));
  MH_TRY(check_launch(ctx, "surrogate parameters"));
  return sync(ctx, "surrogate parameters");
}

int mh_surrogate_wave_terms(mh_context* ctx, int64_t m, const double* r, const double* z, double* out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (m <= 0 || !r || !z || !out) return fail(ctx, MH_ERR_ARG, "bad wave-term arguments");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (!ctx->mlp) return fail(ctx, MH_ERR_ARG, "no surrogate parameters on this context");
  MH_TRY(set_device(ctx));
  double *in, *o;
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(2 * m), &in));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(6 * m), &o));
  MH_TRY(copy_in(ctx, in, r, sizeof(double) * m, mem));
  MH_TRY(copy_in(ctx, in + m, z, sizeof(double) * m, mem));
  launch_surrogate_points(ctx->stream, ctx->lc(), ctx->mlp, m, in, in + m, ctx->quad_rtol, ctx->quad_atol,
                          (double2*)o);
  MH_TRY(check_launch(ctx, "surrogate wave terms"));
  MH_TRY(copy_out(ctx, out, o, sizeof(double) * 6 * m, mem));
  return sync(ctx, "surrogate wave terms");
}


int mh_surrogate_loss_grad(mh_context* ctx, const float* params, int64_t m, const float* inputs, const float* targets,
                           float* grad, double* loss) {
  if (!ctx) return MH_ERR_ARG;
  if (!params || m <= 0 || m > (1 << 20) || !inputs || !targets || !grad)
    return fail(ctx, MH_ERR_ARG, "bad loss/gradient arguments (1 <= m <= 2^20)");
  MH_TRY(set_device(ctx));
  TrainBufs tb;
  tb.st = ctx->stream;
  float *theta, *q, *g, *Y8, *acts;
  float2* X;
  double* dl;
  MH_CUDA(ctx, tb.get(&theta, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&q, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&g, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&X, (size_t)m));
  MH_CUDA(ctx, tb.get(&Y8, (size_t)(8 * m)));
  MH_CUDA(ctx, tb.get(&acts, (size_t)mlp_act_floats((int)m)));
  MH_CUDA(ctx, tb.get(&dl, 1));
  cudaStream_t st = ctx->stream;
  std::vector<float> hy((size_t)(8 * m), 0.0f);
  for (int64_t i = 0; i < m; ++i)
    for (int c = 0; c < kMlpOut; ++c) hy[8 * i + c] = targets[kMlpOut * i + c];
  MH_CUDA(ctx, cudaMemsetAsync(theta, 0, sizeof(float) * kMlpParamsPadded, st));
  MH_CUDA(ctx, cudaMemcpyAsync(theta, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, st));
  MH_CUDA(ctx, cudaMemcpyAsync(X, inputs, sizeof(float2) * m, cudaMemcpyHostToDevice, st));
  MH_CUDA(ctx, cudaMemcpyAsync(Y8, hy.data(), sizeof(float) * 8 * m, cudaMemcpyHostToDevice, st));
  MH_CUDA(ctx, cudaMemsetAsync(g, 0, sizeof(float) * kMlpParamsPadded, st));
  MH_CUDA(ctx, cudaMemsetAsync(dl, 0, sizeof(double), st));
  launch_round_bf16(st, ctx->lc(), theta, q);
  launch_mlp_loss_grad(st, ctx->lc(), q, X, Y8, m, 0, 1, (int)m, acts, dl, g);
  MH_TRY(check_launch(ctx, "surrogate loss/gradient"));
  std::vector<float> hg((size_t)kMlpParamsPadded);
  MH_CUDA(ctx, cudaMemcpyAsync(hg.data(), g, sizeof(float) * kMlpParamsPadded, cudaMemcpyDeviceToHost, st));
  double hl = 0.0;
  MH_CUDA(ctx, cudaMemcpyAsync(&hl, dl, sizeof(double), cudaMemcpyDeviceToHost, st));
  MH_TRY(sync(ctx, "surrogate loss/gradient"));
  for (int i = 0; i < kMlpParams; ++i) grad[i] = hg[i];
  if (loss) *loss = hl;
  return MH_OK;
}

int mh_surrogate_train(mh_context* ctx, int64_t n_samples, uint64_t seed, int epochs, int batch, double lr,
                       float* params_out, double* report) {
  NvtxRange nvtx_range("mh_surrogate_train");
  if (!ctx) return MH_ERR_ARG;
  if (n_samples < 1024 || n_samples > ((int64_t)1 << 27)) return fail(ctx, MH_ERR_ARG, "n_samples must be in [1024, 2^27]");
  if (epochs <= 0 || batch <= 0 || batch > (1 << 16) || !(lr > 0)) return fail(ctx, MH_ERR_ARG, "bad training settings");
  MH_TRY(set_device(ctx));
  cudaStream_t st = ctx->stream;
  const LaunchCounter lc = ctx->lc();
  TrainBufs tb;
  tb.st = st;
  const int64_t M = n_samples;
  const int64_t n_val = std::min<int64_t>(100000, std::max<int64_t>(1024, M / 10));
  float2 *X, *Xv;
  float *Y8, *Yv, *theta, *q, *g, *m1, *m2, *acts;
  double *loss, *Rv, *out_s, *out_w, *out_e;
  MH_CUDA(ctx, tb.get(&X, (size_t)M));
  MH_CUDA(ctx, tb.get(&Y8, (size_t)(8 * M)));
  MH_CUDA(ctx, tb.get(&Xv, (size_t)n_val));
  MH_CUDA(ctx, tb.get(&Yv, (size_t)(8 * n_val)));
  MH_CUDA(ctx, tb.get(&Rv, (size_t)(2 * n_val)));
  MH_CUDA(ctx, tb.get(&out_s, (size_t)(6 * n_val)));
  MH_CUDA(ctx, tb.get(&out_w, (size_t)(6 * n_val)));
  MH_CUDA(ctx, tb.get(&out_e, (size_t)(4 * n_val)));
  MH_CUDA(ctx, tb.get(&theta, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&q, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&g, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&m1, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&m2, kMlpParamsPadded));
  MH_CUDA(ctx, tb.get(&acts, (size_t)mlp_act_floats(batch)));
  MH_CUDA(ctx, tb.get(&loss, 1));
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  struct EvGuard {
    cudaEvent_t a, b, c;
    ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); cudaEventDestroy(c); }
  } evg{e0, e1, e2};
  // training and validation samples (exact kernel at the context's quadrature tolerances)
  MH_CUDA(ctx, cudaEventRecord(e0, st));
  // targets are FP32: quadrature to 1e-10 relative is ample for them
  const double srtol = std::max(ctx->quad_rtol, 1e-10), satol = std::max(ctx->quad_atol, 1e-13);
  const int64_t chunk = (int64_t)1 << 18;
  for (int64_t off = 0; off < M; off += chunk) {
    launch_surrogate_samples(st, lc, seed, M, off, std::min(chunk, M - off), srtol, satol, X, Y8, nullptr);
    MH_TRY(check_launch(ctx, "surrogate samples"));
  }
  const uint64_t vseed = seed ^ 0x5DEECE66Dull;
  launch_surrogate_samples(st, lc, vseed, n_val, 0, n_val, srtol, satol, Xv, Yv, Rv);
  MH_TRY(check_launch(ctx, "surrogate validation samples"));
  MH_CUDA(ctx, cudaEventRecord(e1, st));
  // Glorot-uniform initialisation from a seeded 64-bit Mersenne twister (raw bits -> [0, 1))
  std::vector<float> h0((size_t)kMlpParamsPadded, 0.0f);
  {
    std::mt19937_64 gen(seed);
    auto uni = [&]() { return (double)(gen() >> 11) * (1.0 / 9007199254740992.0); };
    const int offs[4] = {kMlpW1, kMlpW2, kMlpW3, kMlpW4};
    const int fo[4] = {kMlpH, kMlpH, kMlpH, kMlpOut}, fi[4] = {kMlpIn, kMlpH, kMlpH, kMlpH};
    for (int l = 0; l < 4; ++l) {
      const double a = std::sqrt(6.0 / (fo[l] + fi[l]));
      for (int i = 0; i < fo[l] * fi[l]; ++i) h0[offs[l] + i] = (float)((2.0 * uni() - 1.0) * a);
    }
  }
  MH_CUDA(ctx, cudaMemcpyAsync(theta, h0.data(), sizeof(float) * kMlpParamsPadded, cudaMemcpyHostToDevice, st));
  MH_CUDA(ctx, cudaMemsetAsync(g, 0, sizeof(float) * kMlpParamsPadded, st));
  MH_CUDA(ctx, cudaMemsetAsync(m1, 0, sizeof(float) * kMlpParamsPadded, st));
  MH_CUDA(ctx, cudaMemsetAsync(m2, 0, sizeof(float) * kMlpParamsPadded, st));
  launch_round_bf16(st, lc, theta, q);
  // epochs over a fresh multiplicative permutation of the samples each time
  const int64_t steps = (M + batch - 1) / batch;
  const int64_t total = steps * epochs;
  static const uint64_t primes[] = {1000003ull, 2000003ull, 3000017ull, 4000037ull, 5000011ull, 6000011ull,
                                    7000003ull, 8000009ull, 9000011ull, 10000019ull, 11000027ull, 12000017ull};
  double last_loss = 0.0;
  int64_t t = 0;
  for (int e = 0; e < epochs; ++e) {
    uint64_t prime = primes[e % 12];
    while (gcd_u64(prime, (uint64_t)M) != 1) prime += 2;
    MH_CUDA(ctx, cudaMemsetAsync(loss, 0, sizeof(double), st));
    for (int64_t sidx = 0; sidx < steps; ++sidx, ++t) {
      const int64_t base = sidx * batch;
      const int B = (int)std::min<int64_t>(batch, M - base);
      const double cosf_ = 0.5 * (1.0 + std::cos(3.141592653589793 * (double)t / (double)total));
      const float lr_t = (float)(lr * (0.01 + 0.99 * cosf_));
      launch_mlp_train_step(st, lc, theta, q, g, m1, m2, X, Y8, M, base, (int64_t)prime, B, acts, loss, lr_t,
                            (int)(t + 1));
    }
    MH_TRY(check_launch(ctx, "surrogate training"));
    double hl = 0.0;
    MH_CUDA(ctx, cudaMemcpyAsync(&hl, loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    MH_TRY(sync(ctx, "surrogate epoch"));
    last_loss = hl / (double)steps;
  }
  MH_CUDA(ctx, cudaEventRecord(e2, st));
  // install on the context and validate: surrogate vs exact vs Wu at the validation points
  if (!ctx->mlp) MH_CUDA(ctx, cudaMalloc((void**)&ctx->mlp, sizeof(float) * kMlpParamsPadded));
  MH_CUDA(ctx, cudaMemcpyAsync(ctx->mlp, q, sizeof(float) * kMlpParamsPadded, cudaMemcpyDeviceToDevice, st));
  std::vector<double> hr((size_t)(2 * n_val));
  MH_CUDA(ctx, cudaMemcpyAsync(hr.data(), Rv, sizeof(double) * 2 * n_val, cudaMemcpyDeviceToHost, st));
  MH_TRY(sync(ctx, "surrogate validation points"));
  std::vector<double> rz((size_t)(2 * n_val));
  for (int64_t i = 0; i < n_val; ++i) {
    rz[i] = hr[2 * i];
    rz[n_val + i] = hr[2 * i + 1];
  }
  double* rzd;
  MH_CUDA(ctx, tb.get(&rzd, (size_t)(2 * n_val)));
  MH_CUDA(ctx, cudaMemcpyAsync(rzd, rz.data(), sizeof(double) * 2 * n_val, cudaMemcpyHostToDevice, st));
  launch_surrogate_points(st, lc, ctx->mlp, n_val, rzd, rzd + n_val, ctx->quad_rtol, ctx->quad_atol, (double2*)out_s);
  launch_wu_points(st, lc, n_val, rzd, rzd + n_val, (double2*)out_w);
  launch_exact_points(st, lc, n_val, rzd, rzd + n_val, ctx->quad_rtol, ctx->quad_atol, (double2*)out_e);
  MH_TRY(check_launch(ctx, "surrogate validation"));
  std::vector<double> hs((size_t)(6 * n_val)), hw((size_t)(6 * n_val)), he((size_t)(4 * n_val));
  MH_CUDA(ctx, cudaMemcpyAsync(hs.data(), out_s, sizeof(double) * 6 * n_val, cudaMemcpyDeviceToHost, st));
  MH_CUDA(ctx, cudaMemcpyAsync(hw.data(), out_w, sizeof(double) * 6 * n_val, cudaMemcpyDeviceToHost, st));
  MH_CUDA(ctx, cudaMemcpyAsync(he.data(), out_e, sizeof(double) * 4 * n_val, cudaMemcpyDeviceToHost, st));
  std::vector<float> hq((size_t)kMlpParamsPadded);
  MH_CUDA(ctx, cudaMemcpyAsync(hq.data(), q, sizeof(float) * kMlpParamsPadded, cudaMemcpyDeviceToHost, st));
  MH_TRY(sync(ctx, "surrogate validation"));
  // errors relative to max(|G|, |G_r|) scale of each point: |G - G_exact| / |G_exact|
  double s_max = 0, w_max = 0, s_rms = 0, w_rms = 0, sr_max = 0, wr_max = 0;
  for (int64_t i = 0; i < n_val; ++i) {
    const double gx = he[4 * i], gy = he[4 * i + 1], rx = he[4 * i + 2], ry = he[4 * i + 3];
    const double ga = std::hypot(gx, gy), ra = std::hypot(rx, ry);
    const double es = std::hypot(hs[6 * i] - gx, hs[6 * i + 1] - gy) / ga;
    const double ew = std::hypot(hw[6 * i] - gx, hw[6 * i + 1] - gy) / ga;
    const double esr = std::hypot(hs[6 * i + 2] - rx, hs[6 * i + 3] - ry) / std::max(ra, 1e-300);
    const double ewr = std::hypot(hw[6 * i + 2] - rx, hw[6 * i + 3] - ry) / std::max(ra, 1e-300);
    s_max = std::max(s_max, es);
    w_max = std::max(w_max, ew);
    sr_max = std::max(sr_max, esr);
    wr_max = std::max(wr_max, ewr);
    s_rms += es * es;
    w_rms += ew * ew;
  }
  float ms01 = 0, ms12 = 0;
  cudaEventElapsedTime(&ms01, e0, e1);
  cudaEventElapsedTime(&ms12, e1, e2);
  if (params_out) std::memcpy(params_out, hq.data(), sizeof(float) * kMlpParams);
  if (report) {
    report[0] = last_loss;                        // final-epoch mean squared error (scaled targets)
    report[1] = std::sqrt(s_rms / n_val);         // RMS relative error of G, surrogate
    report[2] = s_max;                            // max relative error of G, surrogate
    report[3] = std::sqrt(w_rms / n_val);         // RMS relative error of G, Wu fits
    report[4] = w_max;                            // max relative error of G, Wu fits
    report[5] = sr_max;                           // max relative error of dG/dr, surrogate
    report[6] = wr_max;                           // max relative error of dG/dr, Wu fits
    report[7] = ms01 * 1e-3;                      // seconds: sample generation (exact kernel)
    report[8] = ms12 * 1e-3;                      // seconds: training
    report[9] = (double)n_val;                    // validation points
  }
  return MH_OK;
}

}  // extern "C"




