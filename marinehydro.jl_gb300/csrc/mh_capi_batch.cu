// mh_capi_batch.cu -- the many-body batch of the C-ABI (mh_batch_hydrodynamic_coefficients):
// bodies placed on streams, the whole schedule captured into one CUDA graph and cached.
#include "mh_capi_internal.cuh"

namespace {

// ---------------------------------------------------------------------------
// Many-body batch: the bodies are grouped into size classes (orders within a factor of
// two); per class, on one of several streams, the bodies' assembly and right-hand sides,
// then one grouped factorization and solve of every matrix of the class (one launch per
// kernel and panel step for all of them), then the bodies' forces.  The whole schedule is
// captured into one CUDA graph, and the instantiated graph is cached for repeated calls
// with the same bodies and options.
// ---------------------------------------------------------------------------
struct BatchOpts {
  uint32_t gfs;
  int direct, precision, ir_sweeps;
  double rho, g;
  int64_t n_dofs, n_rad, n_inf, n_beta, nrhs;
  int64_t judge_samples;  // surrogate batches: pairs the exact term checks per matrix (0: none)
  uint64_t judge_seed;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Lay out (or size, when base == nullptr) the device buffers of one body.  The matrices D,
// their FP32 copies, the solutions and pivots live in the grouped arrays of the cache.
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
  b.B = (double2*)take(nw * nx * 16);
  b.B0 = mixed ? (double2*)take(nw * nx * 16) : nullptr;
  b.R = mixed ? (double2*)take(nw * nx * 16) : nullptr;
  b.work = (double2*)take(zgemm_work_elems(b.n, o.nrhs, b.nw) * 16);
  b.norms = (double*)take((2 * (size_t)o.nrhs * nw + nw) * 8);
  if (o.precision != MH_PREC_FP64) b.ozflag = (int*)take(64);  // the tensor-core products' timeout flag
  if (o.gfs & MH_GF_SURROGATE) {  // every self pair plus room for pairs outside the training box
    b.fb_cap = b.n * (b.nw + 64) + 4096;
    b.fb_list = (int4*)take((size_t)b.fb_cap * sizeof(int4));
    b.fb_state = (unsigned long long*)take(4 * sizeof(unsigned long long));
    if (o.judge_samples > 0) b.judge = (double*)take(2 * nw * sizeof(double));
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
  b.hnorms = (double*)take((2 * (size_t)o.nrhs * nw + nw) * 8);
  b.hparams = (double*)take(b.nparams * 8);
  b.hdofs = (double*)take((size_t)o.n_dofs * (size_t)b.n * 3 * 8);
  if ((o.gfs & MH_GF_SURROGATE) && o.judge_samples > 0) b.hjudge = (double*)take(2 * nw * sizeof(double));
  return off;
}

// The grouped arrays (device, then pinned): sizes and, with a base, the pointers.
size_t layout_grouped(BatchCache& c, const BatchOpts& o, char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += align256(std::max<size_t>(bytes, 8));
    return p;
  };
  size_t dn = 0, xn = 0;
  for (auto& b : c.bodies) {
    dn += (size_t)(b.nw * b.n * b.n);
    xn += (size_t)(b.nw * b.n * o.nrhs);
  }
  const size_t M = (size_t)c.M;
  c.D_all = (double2*)take(dn * 16);
  c.X_all = (double2*)take(xn * 16);
  if (o.precision == MH_PREC_MIXED) {
    c.LU32_all = (float2*)take(dn * 8);
    c.X32_all = (float2*)take(xn * 8);
    c.anorm_all = (double*)take(M * 8);
  }
  c.ipiv_all = (int32_t*)take(M * (size_t)c.n_max * 4);
  c.info_all = (int32_t*)take(M * 4);
  c.orders = (int64_t*)take(M * 8);
  c.offsets = (int64_t*)take(M * 8);
  c.xoffsets = (int64_t*)take(M * 8);
  for (auto& k : c.classes) {
    if (o.precision == MH_PREC_FP64_TC) k.oz = take(ozaki_workspace_bytes(k.n_max, k.count));
    else if (o.precision == MH_PREC_MIXED) k.oz = take(bx3_workspace_bytes(k.n_max, k.count));
    k.ozflag = (int*)take(64);
  }
  return off;
}

size_t pinned_grouped(BatchCache& c, const BatchOpts& o, char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += align256(std::max<size_t>(bytes, 8));
    return p;
  };
  c.hinfo_all = (int32_t*)take((size_t)c.M * 4);
  if (o.precision == MH_PREC_MIXED) c.hanorm_all = (double*)take((size_t)c.M * 8);
  return off;
}

// `count` matrices from global index m0 of class k in the grouped layout: orders, offsets and
// solution offsets from the global arrays, pivots at the class's stride (its largest order).
BatchDesc grouped_desc(const BatchCache& c, const BatchCache::SizeClass& k, int64_t m0, int64_t count) {
  BatchDesc d{k.n_max, count, 0};
  d.orders = c.orders + m0;
  d.offsets = c.offsets + m0;
  d.xoffsets = c.xoffsets + m0;
  return d;
}
int32_t* grouped_ipiv(const BatchCache& c, const BatchCache::SizeClass& k, int64_t m0) {
  return c.ipiv_all + k.m_start * c.n_max + (m0 - k.m_start) * k.n_max;
}

// The body's work before the factorization, enqueued on `st` with no host synchronisation:
// static and wave assembly (and the surrogate judge), boundary conditions, the right-hand
// sides of the factored system.
void enqueue_front(mh_context* ctx, LaunchCounter lc, cudaStream_t st, BodyPlan& b, const BatchOpts& o) {
  const int64_t n = b.n, nw = b.nw, nn = n * n, bstride = n * o.nrhs;
  const double* om_d = b.params;
  const double* ks_d = b.params + nw;
  const double* beta_d = b.params + 2 * nw;
  const int32_t* rad_d = (const int32_t*)(b.params + 2 * nw + o.n_beta);
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
  if (b.judge) {
    // the exact term judges every surrogate matrix on sampled pairs; the host re-runs the
    // frequency-solves whose estimate exceeds the tolerance after the graph
    cudaMemsetAsync(b.judge, 0, sizeof(double) * 2 * nw, st);
    launch_surrogate_judge(st, lc, p, st_kinds ? b.SR : nullptr, st_kinds ? b.DR : nullptr, (int)nw, ks_d, b.S, b.D,
                           nn, o.judge_samples, o.judge_seed, b.w_off, st_kinds ? 0 : 1, b.judge);
    cudaMemcpyAsync(b.hjudge, b.judge, sizeof(double) * 2 * nw, cudaMemcpyDeviceToHost, st);
  }
  EpilogueGeom eg{n, b.m->n_hull, b.m->C, b.m->N, b.m->A, b.dofs};
  launch_build_rhs(st, lc, eg, (int)nw, om_d, o.g, (int)o.n_rad, rad_d, (int)o.n_beta, beta_d, b.B, bstride);
  BatchDesc d{n, nw, nn};
  if (b.ozflag) cudaMemsetAsync(b.ozflag, 0, sizeof(int), st);
  // direct: X = S B (on the tensor cores, FP64-accurate, outside the plain FP64 path);
  // indirect: X = B
  if (o.direct) {
    if (o.precision == MH_PREC_FP64) zgemm_nn_batched(st, lc, d, b.S, b.B, o.nrhs, bstride, b.X, b.work);
    else zgemm_nn_tc_batched(st, lc, d, b.S, b.B, o.nrhs, bstride, b.X, b.work, b.ozflag);
  } else {
    cudaMemcpyAsync(b.X, b.B, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st);
  }
  if (o.precision == MH_PREC_MIXED)
    cudaMemcpyAsync(b.B0, b.X, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st);
}

// Every matrix of size class k factored and solved together: one launch per kernel and
// panel step for the class (matrices already factored leave at once), on `st`.
void enqueue_grouped(mh_context* ctx, LaunchCounter lc, cudaStream_t st, BatchCache& c, BatchCache::SizeClass& k,
                     const BatchOpts& o) {
  const BatchDesc g = grouped_desc(c, k, k.m_start, k.count);
  int32_t* ipiv = grouped_ipiv(c, k, k.m_start);
  int32_t* info = c.info_all + k.m_start;
  cudaMemsetAsync(k.ozflag, 0, sizeof(int), st);
  if (o.precision == MH_PREC_FP64 || o.precision == MH_PREC_FP64_TC) {
    lu_factor_batched<double>(st, lc, g, c.D_all, ipiv, info, k.oz, k.oz ? k.ozflag : nullptr);
    lu_solve_batched<double>(st, lc, g, c.D_all, ipiv, c.X_all, o.nrhs, 0, false);
  } else {
    // the class's solutions are contiguous: elementwise passes cover them in one launch
    const int64_t x0 = c.h_xoffsets[(size_t)k.m_start];
    const BodyPlan& last = c.bodies[(size_t)k.bodies.back()];
    const int64_t xn = c.h_xoffsets[(size_t)(last.m0 + last.nw - 1)] + last.n * o.nrhs - x0;
    convert_with_norms(st, lc, g, c.D_all, c.LU32_all, 0, c.anorm_all + k.m_start);
    lu_factor_batched<float>(st, lc, g, c.LU32_all, ipiv, info, k.oz, k.ozflag);
    convert_z_to_c(st, lc, c.X_all + x0, c.X32_all + x0, xn);
    lu_solve_batched<float>(st, lc, g, c.LU32_all, ipiv, c.X32_all, o.nrhs, 0, false);
    widen_c_to_z(st, lc, c.X32_all + x0, c.X_all + x0, xn);
    for (int it = 0; it < o.ir_sweeps; ++it) {
      for (int64_t bi : k.bodies) {
        BodyPlan& b = c.bodies[(size_t)bi];
        BatchDesc d{b.n, b.nw, b.n * b.n};
        residual_tc_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, b.n * o.nrhs, b.R, b.work, b.ozflag);
        convert_z_to_c(st, lc, b.R, b.X32, b.n * o.nrhs * b.nw);
      }
      lu_solve_batched<float>(st, lc, g, c.LU32_all, ipiv, c.X32_all, o.nrhs, 0, false);
      ir_update(st, lc, xn, c.X_all + x0, c.X32_all + x0);
    }
    cudaMemcpyAsync(c.hanorm_all + k.m_start, c.anorm_all + k.m_start, sizeof(double) * k.count,
                    cudaMemcpyDeviceToHost, st);
  }
  cudaMemcpyAsync(c.hinfo_all + k.m_start, info, sizeof(int32_t) * k.count, cudaMemcpyDeviceToHost, st);
}

// The body's work after the solves: the refinement's residual (mixed), phi (indirect: S x),
// forces and the copies to the host.
void enqueue_back(mh_context* ctx, LaunchCounter lc, cudaStream_t st, BodyPlan& b, const BatchOpts& o) {
  const int64_t n = b.n, nw = b.nw, nn = n * n, bstride = n * o.nrhs;
  const double* om_d = b.params;
  const double* beta_d = b.params + 2 * nw;
  const int32_t* inf_d = (const int32_t*)(b.params + 2 * nw + o.n_beta) + o.n_rad;
  BatchDesc d{n, nw, nn};
  if (o.precision == MH_PREC_MIXED) {
    // the residual of the returned x, judged on the host after the graph
    const int64_t ncols = o.nrhs * nw;
    residual_tc_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, bstride, b.R, b.work, b.ozflag);
    inf_norms_batched(st, lc, n, ncols, b.R, b.norms);
    inf_norms_batched(st, lc, n, ncols, b.X, b.norms + ncols);
    cudaMemcpyAsync(b.hnorms, b.norms, sizeof(double) * 2 * ncols, cudaMemcpyDeviceToHost, st);
  }
  EpilogueGeom eg{n, b.m->n_hull, b.m->C, b.m->N, b.m->A, b.dofs};
  double2* phi = b.X;
  if (!o.direct) {
    if (o.precision == MH_PREC_FP64) zgemm_nn_batched(st, lc, d, b.S, b.X, o.nrhs, bstride, b.B, b.work);
    else zgemm_nn_tc_batched(st, lc, d, b.S, b.X, o.nrhs, bstride, b.B, b.work, b.ozflag);
    phi = b.B;
  }
  if (o.n_inf > 0)
    launch_forces(st, lc, eg, (int)nw, om_d, o.rho, o.g, (int)o.nrhs, phi, bstride, (int)o.n_inf, inf_d,
                  (int)o.n_beta, beta_d, b.F, b.FK);
  cudaMemcpyAsync(b.hF, b.F, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.nrhs,
                  cudaMemcpyDeviceToHost, st);
  if (o.n_beta > 0)
    cudaMemcpyAsync(b.hFK, b.FK, sizeof(double2) * nw * std::max<int64_t>(o.n_inf, 1) * o.n_beta,
                    cudaMemcpyDeviceToHost, st);
}

// Host-side completion of one body after the graph: singular check, refinement
// convergence (extra sweeps or the FP64 fallback on the context stream).
int finish_body(mh_context* ctx, BatchCache& c, BodyPlan& b, const BatchOpts& o) {
  for (int64_t w = 0; w < b.nw; ++w)
    if (b.hinfo[w] != 0)
      return fail(ctx, MH_ERR_SINGULAR, "body with %lld panels, frequency %lld: zero pivot in column %d",
                  (long long)b.n, (long long)w, b.hinfo[w]);
  if (b.ozflag) {
    int flag = 0;
    MH_CUDA(ctx, cudaMemcpy(&flag, b.ozflag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of a batch product gave up");
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
    for (int64_t col = 0; col < ncols; ++col) {
      const double anrm = c.hanorm_all[b.m0 + col / o.nrhs];
      if (!(b.hnorms[col] <= cte * anrm * b.hnorms[ncols + col])) return false;
    }
    return true;
  };
  if (converged()) return MH_OK;
  cudaStream_t st = ctx->stream;
  const LaunchCounter lc = ctx->lc();
  BatchDesc d{n, nw, nn};
  const BatchCache::SizeClass& cls = c.classes[(size_t)b.cls];
  const BatchDesc gb = grouped_desc(c, cls, b.m0, nw);  // this body's matrices in the grouped layout
  int32_t* ipiv_b = grouped_ipiv(c, cls, b.m0);
  bool ok = false;
  for (int it = 0; it < 30 && !ok; ++it) {
    convert_z_to_c(st, lc, b.R, b.X32, bstride * nw);
    lu_solve_batched<float>(st, lc, gb, c.LU32_all, ipiv_b, c.X32_all, o.nrhs, 0, false);
    ir_update(st, lc, bstride * nw, b.X, b.X32);
    residual_batched(st, lc, d, b.D, b.X, b.B0, o.nrhs, bstride, b.R, b.work, false);
    inf_norms_batched(st, lc, n, ncols, b.R, b.norms);
    inf_norms_batched(st, lc, n, ncols, b.X, b.norms + ncols);
    MH_CUDA(ctx, cudaMemcpyAsync(b.hnorms, b.norms, sizeof(double) * 2 * ncols, cudaMemcpyDeviceToHost, st));
    MH_TRY(sync(ctx, "batch refinement"));
    ok = converged();
  }
  if (!ok) {
    // FP64 factors of this body's matrices (a uniform batch of its own, pivots at stride n
    // inside its slice of the grouped pivot array)
    MH_CUDA(ctx, cudaMemcpyAsync(b.X, b.B0, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st));
    lu_factor_batched<double>(st, lc, d, b.D, ipiv_b, b.info);
    lu_solve_batched<double>(st, lc, d, b.D, ipiv_b, b.X, o.nrhs, bstride, false);
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

extern "C" {

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
  const bool judging = (gfs & MH_GF_SURROGATE) && ctx->judge_samples > 0;
  BatchOpts o{gfs, direct ? 1 : 0, precision, 2, rho, g, n_dofs, n_rad, n_inf, n_beta, n_rad + n_beta,
              judging ? ctx->judge_samples : 0, judging ? ctx->judge_seed : 0};

  // cache key: everything the captured graph bakes in
  // with profiling on, the schedule runs uncaptured on one stream so that every launch is
  // timed by its own events (kernel shares of the batch); the graph is not built
  const bool profiling = profiler_on(ctx->prof);
  std::vector<double> key = {(double)n_bodies, (double)gfs, (double)o.direct, (double)precision, (double)S, rho, g,
                             (double)n_dofs, (double)n_rad, (double)n_inf, (double)n_beta, ctx->quad_rtol,
                             ctx->quad_atol, profiling ? 1.0 : 0.0, (double)o.judge_samples,
                             (double)(o.judge_seed >> 32), (double)(o.judge_seed & 0xFFFFFFFFULL)};
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
    // size classes: bodies by decreasing order, a new class whenever the order falls below
    // half the class's largest; matrices numbered class by class, body by body
    std::vector<int64_t> order(n_bodies);
    for (int64_t b = 0; b < n_bodies; ++b) order[b] = b;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t c) {
      return bc->bodies[a].n != bc->bodies[c].n ? bc->bodies[a].n > bc->bodies[c].n : a < c;
    });
    int64_t m = 0;
    for (int64_t b : order) {
      BodyPlan& p = bc->bodies[b];
      if (bc->classes.empty() || 2 * p.n < bc->classes.back().n_max) {
        BatchCache::SizeClass k;
        k.m_start = m;
        k.n_max = p.n;
        bc->classes.push_back(k);
      }
      BatchCache::SizeClass& k = bc->classes.back();
      k.bodies.push_back(b);
      k.count += p.nw;
      p.cls = (int)bc->classes.size() - 1;
      p.m0 = m;
      m += p.nw;
    }
    bc->M = m;
    bc->n_max = bc->classes.front().n_max;
    // classes onto streams, the costliest first onto the least-loaded stream
    {
      std::vector<double> load(S, 0.0);
      std::vector<double> cost(bc->classes.size(), 0.0);
      for (auto& p : bc->bodies) cost[(size_t)p.cls] += p.cost;
      std::vector<size_t> co(bc->classes.size());
      for (size_t q = 0; q < co.size(); ++q) co[q] = q;
      std::sort(co.begin(), co.end(), [&](size_t a, size_t c) { return cost[a] > cost[c]; });
      for (size_t q : co) {
        int best = 0;
        for (int t = 1; t < S; ++t) if (load[t] < load[best]) best = t;
        bc->classes[q].stream = best;
        load[best] += cost[q];
      }
      for (auto& p : bc->bodies) p.stream = bc->classes[(size_t)p.cls].stream;
    }
    bc->h_orders.resize((size_t)bc->M);
    bc->h_offsets.resize((size_t)bc->M);
    bc->h_xoffsets.resize((size_t)bc->M);
    {
      int64_t doffs = 0, xoffs = 0;
      for (auto& k : bc->classes)
        for (int64_t b : k.bodies) {
          BodyPlan& p = bc->bodies[b];
          for (int64_t w = 0; w < p.nw; ++w) {
            bc->h_orders[(size_t)(p.m0 + w)] = p.n;
            bc->h_offsets[(size_t)(p.m0 + w)] = doffs;
            bc->h_xoffsets[(size_t)(p.m0 + w)] = xoffs;
            doffs += p.n * p.n;
            xoffs += p.n * o.nrhs;
          }
        }
    }
    size_t dev_bytes = 0, host_bytes = 0;
    std::vector<size_t> doff(n_bodies), hoff(n_bodies);
    for (int64_t b = 0; b < n_bodies; ++b) {
      doff[b] = dev_bytes;
      dev_bytes += layout_body(bc->bodies[b], o, nullptr);
      hoff[b] = host_bytes;
      host_bytes += pinned_body(bc->bodies[b], o, nullptr);
    }
    const size_t gdev = dev_bytes;
    dev_bytes += layout_grouped(*bc, o, nullptr);
    const size_t ghost = host_bytes;
    host_bytes += pinned_grouped(*bc, o, nullptr);
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
    layout_grouped(*bc, o, (char*)bc->arena + gdev);
    pinned_grouped(*bc, o, bc->pinned + ghost);
    for (auto& p : bc->bodies) {
      const BatchCache::SizeClass& k = bc->classes[(size_t)p.cls];
      p.D = bc->D_all + bc->h_offsets[(size_t)p.m0];
      p.X = bc->X_all + bc->h_xoffsets[(size_t)p.m0];
      if (bc->LU32_all) {
        p.LU32 = bc->LU32_all + bc->h_offsets[(size_t)p.m0];
        p.X32 = bc->X32_all + bc->h_xoffsets[(size_t)p.m0];
      }
      p.ipiv = grouped_ipiv(*bc, k, p.m0);
      p.info = bc->info_all + p.m0;
      p.hinfo = bc->hinfo_all + p.m0;
    }
    MH_CUDA(ctx, cudaMemcpy(bc->orders, bc->h_orders.data(), sizeof(int64_t) * bc->M, cudaMemcpyHostToDevice));
    MH_CUDA(ctx, cudaMemcpy(bc->offsets, bc->h_offsets.data(), sizeof(int64_t) * bc->M, cudaMemcpyHostToDevice));
    MH_CUDA(ctx, cudaMemcpy(bc->xoffsets, bc->h_xoffsets.data(), sizeof(int64_t) * bc->M, cudaMemcpyHostToDevice));
    while ((int)ctx->side.size() < S - 1) {
      cudaStream_t st;
      MH_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      ctx->side.push_back(st);
    }
    bc->order = order;
    if (profiling) {
      ctx->batch = bc;
    } else {
      // capture the schedule: per size class on its stream, the bodies' assembly, the class's
      // grouped factorization and solves, the bodies' forces
      cudaStream_t s0 = ctx->stream;
      std::vector<cudaEvent_t> ev(S);
      for (auto& e : ev) MH_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      LaunchCounter cap{&bc->graph_kernels, nullptr, &ctx->tiles};
      MH_CUDA(ctx, cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
      cudaEventRecord(ev[0], s0);
      for (int q = 1; q < S; ++q) cudaStreamWaitEvent(ctx->side[q - 1], ev[0], 0);
      for (auto& k : bc->classes) {
        cudaStream_t st = k.stream == 0 ? s0 : ctx->side[k.stream - 1];
        for (int64_t b : k.bodies) enqueue_front(ctx, cap, st, bc->bodies[b], o);
        enqueue_grouped(ctx, cap, st, *bc, k, o);
        for (int64_t b : k.bodies) enqueue_back(ctx, cap, st, bc->bodies[b], o);
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
    for (auto& k : bc->classes) {
      for (int64_t b : k.bodies) enqueue_front(ctx, ctx->lc(), ctx->stream, bc->bodies[b], o);
      enqueue_grouped(ctx, ctx->lc(), ctx->stream, *bc, k, o);
      for (int64_t b : k.bodies) enqueue_back(ctx, ctx->lc(), ctx->stream, bc->bodies[b], o);
    }
  }
  MH_TRY(sync(ctx, "batch graph"));
  for (auto& k : bc->classes) {
    int flag = 0;
    MH_CUDA(ctx, cudaMemcpy(&flag, k.ozflag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(ctx, MH_ERR_TIMEOUT, "a tensor-core completion wait of the LU update gave up");
  }
  for (auto& p : bc->bodies) MH_TRY(finish_body(ctx, *bc, p, o));
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
  if (judging) {
    // per frequency-solve estimate; the ones above the tolerance go through the exact term
    ctx->judge_err.assign((size_t)total_w, 0.0);
    ctx->judge_rerun.assign((size_t)total_w, 0);
    const uint32_t exact_gfs = (gfs & ~MH_GF_SURROGATE) | MH_GF_EXACT_DELHOMMEAU;
    for (int64_t b = 0; b < n_bodies; ++b) {
      BodyPlan& p = bc->bodies[b];
      std::vector<double> redo;
      std::vector<int64_t> redo_w;
      for (int64_t w = 0; w < p.nw; ++w) {
        const double e2 = p.hjudge[2 * w], t2 = p.hjudge[2 * w + 1];
        const double err = t2 > 0 ? std::sqrt(e2 / t2) : 0.0;
        ctx->judge_err[(size_t)(p.w_off + w)] = err;
        if (!(err <= ctx->judge_tol)) {
          ctx->judge_rerun[(size_t)(p.w_off + w)] = 1;
          redo.push_back(omegas[p.w_off + w]);
          redo_w.push_back(w);
        }
      }
      if (redo.empty()) continue;
      const double* dofs_h = nullptr;
      if (n_dofs > 0) {
        if (mem == MH_MEM_DEVICE)
          MH_CUDA(ctx, cudaMemcpy(p.hdofs, dofs[b], sizeof(double) * n_dofs * p.n * 3, cudaMemcpyDeviceToHost));
        dofs_h = mem == MH_MEM_DEVICE ? p.hdofs : dofs[b];
      }
      const int64_t nr = (int64_t)redo.size();
      std::vector<double> rA((size_t)(n_inf * n_rad * nr)), rB(rA.size());
      std::vector<double2> rd((size_t)(n_inf * nr * n_beta)), rk(rd.size()), re(rd.size());
      // the exact re-run has no surrogate, so it leaves the judge's record of this call alone
      MH_TRY(mh_hydrodynamic_coefficients(ctx, p.m, nr, redo.data(), rho, g, exact_gfs, direct, n_dofs, dofs_h,
                                          n_rad, rad_idx, n_inf, inf_idx, n_beta, betas, precision,
                                          n_rad ? (double*)rA.data() : nullptr, n_rad ? (double*)rB.data() : nullptr,
                                          n_beta ? (double*)rd.data() : nullptr, n_beta ? (double*)rk.data() : nullptr,
                                          n_beta ? (double*)re.data() : nullptr, MH_MEM_HOST));
      for (int64_t q = 0; q < nr; ++q) {
        const int64_t w = redo_w[(size_t)q];
        for (int64_t i = 0; i < n_inf; ++i) {
          for (int64_t r = 0; r < n_rad; ++r) {
            const size_t dst = (size_t)(n_inf * n_rad * p.w_off) + (size_t)(i + n_inf * (r + n_rad * w));
            const size_t src = (size_t)(i + n_inf * (r + n_rad * q));
            hA[dst] = rA[src];
            hB[dst] = rB[src];
          }
          for (int64_t bb = 0; bb < n_beta; ++bb) {
            const size_t dst = (size_t)(n_inf * n_beta * p.w_off) + (size_t)(i + n_inf * (w + p.nw * bb));
            const size_t src = (size_t)(i + n_inf * (q + nr * bb));
            hd[dst] = rd[src];
            hk[dst] = rk[src];
            he[dst] = re[src];
          }
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

int mh_surrogate_set_judge(mh_context* ctx, int64_t n_samples, uint64_t seed, double tolerance) {
  if (!ctx) return MH_ERR_ARG;
  if (n_samples < 0 || n_samples > (int64_t)1 << 24) return fail(ctx, MH_ERR_ARG, "n_samples must be in [0, 2^24]");
  if (!(tolerance >= 0)) return fail(ctx, MH_ERR_ARG, "the tolerance must be >= 0");
  ctx->judge_samples = n_samples;
  ctx->judge_seed = seed;
  ctx->judge_tol = tolerance;
  return MH_OK;
}

int mh_surrogate_judge_read(mh_context* ctx, int64_t count, double* estimates, int32_t* rerun) {
  if (!ctx) return MH_ERR_ARG;
  if (count != (int64_t)ctx->judge_err.size())
    return fail(ctx, MH_ERR_ARG, "the last judged call had %lld frequency-solves, not %lld",
                (long long)ctx->judge_err.size(), (long long)count);
  if (estimates) std::memcpy(estimates, ctx->judge_err.data(), sizeof(double) * ctx->judge_err.size());
  if (rerun) std::memcpy(rerun, ctx->judge_rerun.data(), sizeof(int32_t) * ctx->judge_rerun.size());
  return MH_OK;
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
