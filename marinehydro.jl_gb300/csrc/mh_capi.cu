// mh_capi.cu -- the C-ABI of libmarinehydro_cuda.so (declared in include/marinehydro_gb300.h).
//
// Owns the contexts (device, stream, workspaces, launch counter, last error) and
// mesh handles (device copies of one body's panels, the per-panel Birk frames and
// the cached wavenumber-independent matrices), defines the helpers the other C-ABI
// units share (mh_capi_internal.cuh), and orchestrates the kernels of mh_assembly.cu,
// mh_lu.cu and mh_epilogue.cu for assembly, dense solves and the frequency sweep.  The
// many-body batch, the derivatives, the launch-shape tuning and the surrogate have
// their own units (mh_capi_batch.cu, mh_capi_diff.cu, mh_capi_tuning.cu,
// mh_capi_surrogate.cu).
#include "mh_capi_internal.cuh"

namespace mh {
namespace capi {

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

// FP64 factorization with the tensor-core update of matrices that carry their right-hand
// sides as d.extra appended columns: after the factorization those columns hold L^-1 P b, and
// the upper triangular solve overwrites them with the solution.
int solve_core_appended(mh_context* ctx, const BatchDesc& d, double2* Adev) {
  const int64_t n = d.n;
  int32_t *ipiv, *info;
  MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)(n * d.batch), &ipiv));
  MH_TRY(ws_get_t(ctx, kSlotInfo, (size_t)d.batch, &info));
  unsigned char* ws;
  const size_t wsb = ozaki_workspace_bytes(n, d.batch, d.extra);
  MH_TRY(ws_get_t(ctx, kSlotOzaki, wsb + 256, &ws));
  int* flag = reinterpret_cast<int*>(ws + wsb);
  MH_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
  if (lu_factor_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, info, ws, flag) != 0)
    return fail(ctx, MH_ERR_UNSUPPORTED, "appended right-hand sides need the uniform tensor-core FP64 factorization");
  MH_TRY(check_launch(ctx, "lu factor (tensor-core update, appended right-hand sides)"));
  lu_solve_batched<double>(ctx->stream, ctx->lc(), d, Adev, ipiv, Adev + (size_t)n * (size_t)n, d.extra, d.stride,
                           false, true);
  MH_TRY(check_launch(ctx, "upper triangular solve"));
  int hflag = 0;
  MH_CUDA(ctx, cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MH_TRY(sync(ctx, "tensor-core update"));
  if (hflag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  return check_pivots(ctx, d, 0);
}

}  // namespace capi
}  // namespace mh

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

  // FP64 with the tensor-core update: the right-hand sides ride along as appended columns of
  // D (and S keeps the same stride), so the factorization performs the forward substitution
  const bool appended = precision == MH_PREC_FP64_TC;
  const size_t mstride = nn + (appended ? (size_t)n * (size_t)nrhs : 0);

  // chunk the frequencies by memory
  size_t free_b = 0, total_b = 0;
  MH_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
  size_t per_w = mstride * sizeof(double2) * 2 + (size_t)n * nrhs * sizeof(double2) * 4;
  if (precision == MH_PREC_MIXED) per_w += nn * sizeof(float2);
  size_t budget = std::min<size_t>(free_b / 2, (size_t)48 << 30);
  int64_t chunk = (int64_t)std::max<size_t>(1, budget / per_w);
  chunk = std::min<int64_t>(chunk, n_omega);

  double2 *S, *D, *B, *X, *work, *F, *FK;
  MH_TRY(ws_get_t(ctx, kSlotS, mstride * chunk, &S));
  MH_TRY(ws_get_t(ctx, kSlotD, mstride * chunk, &D));
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)(n * nrhs * chunk), &B));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(n * nrhs * chunk), &X));
  MH_TRY(ws_get_t(ctx, kSlotF, (size_t)(n_omega * std::max<int64_t>(n_inf, 1) * nrhs), &F));
  MH_TRY(ws_get_t(ctx, kSlotFK, (size_t)(n_omega * std::max<int64_t>(n_inf, 1) * std::max<int64_t>(n_beta, 1)), &FK));

  EpilogueGeom eg{n, m->n_hull, m->C, m->N, m->A, dofs_d};
  AssemblyParams p = make_params(ctx, m, gfs, direct, 1, nullptr);
  MH_TRY(prepare_surrogate(ctx, p, chunk));
  const bool judging = (gfs & MH_GF_SURROGATE) && ctx->judge_samples > 0;
  double* judge_acc = nullptr;
  if (judging) {
    MH_TRY(ws_get_t(ctx, kSlotJudge, (size_t)(2 * chunk), &judge_acc));
    ctx->judge_err.assign((size_t)n_omega, 0.0);
    ctx->judge_rerun.assign((size_t)n_omega, 0);
  }

  for (int64_t w0 = 0; w0 < n_omega; w0 += chunk) {
    const int64_t nw = std::min<int64_t>(chunk, n_omega - w0);
    launch_assemble_wave(ctx->stream, ctx->lc(), p, SR, DR, (int)nw, ks_all + w0, S, D, (int64_t)mstride,
                         st ? 0 : 1);
    MH_TRY(check_launch(ctx, "wave assembly"));
    if (judging) {
      // the exact term judges each surrogate matrix on sampled pairs; a matrix whose sampled
      // relative error exceeds the tolerance is assembled again with the exact term
      MH_TRY(check_surrogate(ctx, p));
      MH_CUDA(ctx, cudaMemsetAsync(judge_acc, 0, sizeof(double) * 2 * nw, ctx->stream));
      launch_surrogate_judge(ctx->stream, ctx->lc(), p, SR, DR, (int)nw, ks_all + w0, S, D, (int64_t)mstride,
                             ctx->judge_samples, ctx->judge_seed, w0, st ? 0 : 1, judge_acc);
      MH_TRY(check_launch(ctx, "surrogate judge"));
      std::vector<double> hacc((size_t)(2 * nw));
      MH_CUDA(ctx, cudaMemcpyAsync(hacc.data(), judge_acc, sizeof(double) * 2 * nw, cudaMemcpyDeviceToHost,
                                   ctx->stream));
      MH_TRY(sync(ctx, "surrogate judge"));
      const AssemblyParams pe = make_params(ctx, m, (gfs & ~MH_GF_SURROGATE) | MH_GF_EXACT_DELHOMMEAU, direct, 1,
                                            nullptr);
      for (int64_t b = 0; b < nw; ++b) {
        const double err = hacc[2 * b + 1] > 0 ? std::sqrt(hacc[2 * b] / hacc[2 * b + 1]) : 0.0;
        ctx->judge_err[(size_t)(w0 + b)] = err;
        if (!(err <= ctx->judge_tol)) {
          ctx->judge_rerun[(size_t)(w0 + b)] = 1;
          launch_assemble_wave(ctx->stream, ctx->lc(), pe, SR, DR, 1, ks_all + w0 + b, S + b * mstride,
                               D + b * mstride, (int64_t)mstride, st ? 0 : 1);
        }
      }
      MH_TRY(check_launch(ctx, "exact re-assembly"));
    }
    const int64_t bstride = n * nrhs;
    launch_build_rhs(ctx->stream, ctx->lc(), eg, (int)nw, om_d + w0, g, (int)n_rad, rad_d, (int)n_beta, beta_d, B,
                     bstride);
    MH_TRY(check_launch(ctx, "boundary conditions"));
    BatchDesc d{n, nw, (int64_t)mstride};
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
    if (appended) {
      // right-hand sides (S b, or b for the sources) into the appended columns, factor, solve
      // U x = y in place, and the solution back to X
      const double2* rhs = B;
      if (direct) {
        MH_TRY(s_times(B, X));
        rhs = X;
      }
      MH_CUDA(ctx, cudaMemcpy2DAsync(D + nn, mstride * sizeof(double2), rhs, bstride * sizeof(double2),
                                     bstride * sizeof(double2), (size_t)nw, cudaMemcpyDeviceToDevice, ctx->stream));
      BatchDesc da = d;
      da.extra = nrhs;
      MH_TRY(solve_core_appended(ctx, da, D));
      MH_CUDA(ctx, cudaMemcpy2DAsync(X, bstride * sizeof(double2), D + nn, mstride * sizeof(double2),
                                     bstride * sizeof(double2), (size_t)nw, cudaMemcpyDeviceToDevice, ctx->stream));
      if (!direct) {
        MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, nw), &work));
        MH_TRY(s_times(X, B));
        std::swap(B, X);
      }
    } else if (direct) {
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

int mh_fixpoint_points(mh_context* ctx, int64_t m, const double* x, double* out, int mem) {
  if (!ctx) return MH_ERR_ARG;
  if (m <= 0 || !x || !out) return fail(ctx, MH_ERR_ARG, "bad fixed-point arguments");
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  MH_TRY(set_device(ctx));
  double *in, *o;
  MH_TRY(ws_get_t(ctx, kSlotIn, (size_t)m, &in));
  MH_TRY(ws_get_t(ctx, kSlotX, (size_t)(4 * m), &o));
  MH_TRY(copy_in(ctx, in, x, sizeof(double) * m, mem));
  launch_fixpoint_points(ctx->stream, ctx->lc(), m, in, o);
  MH_TRY(check_launch(ctx, "fixed-point points"));
  MH_TRY(copy_out(ctx, out, o, sizeof(double) * 4 * m, mem));
  return sync(ctx, "fixed-point points");
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

}  // extern "C"
