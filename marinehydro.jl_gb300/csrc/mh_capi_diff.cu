// mh_capi_diff.cu -- derivatives through the C-ABI: the frequency derivative of the sweep
// (forward mode) and the hand-written adjoint (mh_hydro_gradient, mh_hydro_vjp).
#include "mh_capi_internal.cuh"

namespace {

// Reverse-mode product of the zero-speed radiation sweep: J = sum over omega, influenced q
// and radiating r of abar[q, r, w] A[q, r, w] + bbar[q, r, w] B[q, r, w] (host cotangents,
// n_inf x n_rad x n_omega, column-major) and its gradient with respect to every panel's
// centre, normal, area, Birk corners and the dof fields.  The gradient of the dof fields
// stays on the device (n_dofs x n x 3, *gd_out, workspace memory).
// Direct: phi = D^-1 S b, lam = D^-T w.  Indirect: sigma = K^-1 b, phi = S sigma,
// lam = K^-T S^T w, and the boundary conditions pair with lam instead of S^T lam.
int hydro_vjp_core(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                   uint32_t gfs, int direct, int64_t n_dofs, const double* dofs, int64_t n_rad, const int32_t* rad_idx,
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
  const uint32_t allowed = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE | MH_GF_WU |
                           MH_GF_EXACT_DELHOMMEAU;
  if (gfs == 0 || (gfs & ~allowed) || ((gfs & MH_GF_WU) && (gfs & MH_GF_EXACT_DELHOMMEAU)))
    return fail(ctx, MH_ERR_UNSUPPORTED,
                "the adjoint covers the Birk Rankine family with GFWu or ExactGuevelDelhommeau (got 0x%x)", gfs);
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
  size_t per_w = nn * sizeof(double2) * 2 + (size_t)n * ncol * sizeof(double2) * 7;
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
  double2* Y = nullptr;  // indirect: phi = S sigma (X holds sigma)
  if (!direct) MH_TRY(ws_get_t(ctx, kSlotY, (size_t)(bstride * chunk), &Y));
  const bool exact = (gfs & MH_GF_EXACT_DELHOMMEAU) != 0;
  double2* gvals = nullptr;  // exact term: G, dG/dr of every unordered pair at one wavenumber
  if (exact) MH_TRY(ws_get_t(ctx, kSlotEgd, (size_t)(2 * egd_packed_pairs(n)), &gvals));
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
  AssemblyParams pst = make_params(ctx, m, stk, direct, 1, nullptr);
  if (stk) {
    launch_assemble_static(st, lc, pst, SR, DR);
    MH_TRY(check_launch(ctx, "static assembly"));
  }
  AssemblyParams p = make_params(ctx, m, gfs, direct, 1, nullptr);
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
    // phi = D^-1 S b (direct) or phi = S K^-1 b (indirect), the forces, and the force weights
    // conj(w) (into lam, for the A^H solves)
    double2* Phi = direct ? X : Y;
    auto forces_and_weights = [&]() {
      if (!direct) zgemm_nn_batched(st, lc, d, S, X, ncol, bstride, Y, work);  // phi = S sigma
      launch_forces(st, lc, eg, (int)nw, om_d + w0, rho, g, (int)ncol, Phi, bstride, (int)ni, inf_d, (int)nb, beta_d,
                    F + w0 * ni * ncol, FK + w0 * ni * nb1);
      for (int64_t w = 0; w < nw; ++w)
        launch_force_weights(st, lc, n, m->N, m->A, dofs_d, inf_d, (int)ni, (int)ncol, cw + (w0 + w) * ni * ncol,
                             omegas[w0 + w], rho, lam + w * bstride);
      // indirect: the adjoint solve's right-hand side is conj(S^T w) = S^H conj(w), into t
      if (!direct) zgemm_adj_batched(st, lc, d, S, lam, ncol, bstride, t, work);
    };
    double2* adj = direct ? lam : t;  // the right-hand sides of the A^H solve
    bool done = false;
    if (precision == MH_PREC_MIXED) {
      // FP32 factors, both solves refined to FP64 backward error; any column that does not
      // converge sends the whole chunk to the FP64 factorization below (D is left intact)
      float2* LU32;
      double* anrm;
      MH_TRY(factor_mixed(ctx, d, D, &LU32, &anrm));
      if (direct) zgemm_nn_batched(st, lc, d, S, B, ncol, bstride, X, work);
      else MH_CUDA(ctx, cudaMemcpyAsync(X, B, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st));
      bool ok_fwd = false, ok_adj = false;
      MH_TRY(refine_mixed(ctx, d, D, LU32, anrm, X, ncol, bstride, false, &ok_fwd, nullptr));
      if (ok_fwd) {
        forces_and_weights();
        MH_TRY(refine_mixed(ctx, d, D, LU32, anrm, adj, ncol, bstride, true, &ok_adj, nullptr));
      }
      done = ok_fwd && ok_adj;
    }
    if (!done) {
      if (direct) zgemm_nn_batched(st, lc, d, S, B, ncol, bstride, X, work);
      else MH_CUDA(ctx, cudaMemcpyAsync(X, B, sizeof(double2) * bstride * nw, cudaMemcpyDeviceToDevice, st));
      lu_factor_batched<double>(st, lc, d, D, ipiv, info, oz_ws, oz_flag);
      lu_solve_batched<double>(st, lc, d, D, ipiv, X, ncol, bstride, false);    // phi (direct) / sigma
      forces_and_weights();
      lu_solve_batched<double>(st, lc, d, D, ipiv, adj, ncol, bstride, true);   // conj(lam)
    }
    MH_TRY(check_launch(ctx, "gradient solves"));
    MH_TRY(check_pivots(ctx, d, w0));
    if (direct) {
      zgemm_adj_batched(st, lc, d, S, lam, ncol, bstride, t, work);  // S^H conj(lam)
      launch_conj(st, lc, nw * bstride, t);                          // t = S^T lam
      launch_conj(st, lc, nw * bstride, lam);                        // lam = D^-T w
    } else {
      launch_conj(st, lc, nw * bstride, t);                          // t = lam = K^-T S^T w
      launch_conj(st, lc, nw * bstride, lam);                        // lam buffer = w
    }
    for (int64_t w = 0; w < nw; ++w) {
      const double om = omegas[w0 + w], k = om * om / g;
      if (exact) launch_egd_pair_values(st, lc, p, k, gvals);
      // wave-term gradient and the frequency-summed Rankine weights, the cotangent factors
      // already in the vectors; the wave kernel takes up to four columns at a time
      for (int64_t c0 = 0; c0 < ncol; c0 += 4) {
        const int64_t off = w * bstride + c0 * n;
        const int nh = (int)std::min<int64_t>(4, ncol - c0);
        if (direct)
          launch_wave_adjoint(st, lc, p, k, lam + off, B + off, lam + off, X + off, nh, make_double2(1.0, 0.0), gvals,
                              gc, gn, ga, RS, RD);
        else
          launch_wave_adjoint(st, lc, p, k, lam + off, X + off, t + off, X + off, nh, make_double2(1.0, 0.0), gvals,
                              gc, gn, ga, RS, RD);
      }
      launch_rhs_adjoint(st, lc, n, m->N, m->A, m->C, dofs_d, rad_d, (int)nr, inf_d, (int)ni, (int)nb, beta_d, om,
                         rho, g, cw + (w0 + w) * ni * ncol, Phi + w * bstride, t + w * bstride, gc, gn, ga, gd);
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
  if ((gfs & MH_GF_SURROGATE) || ((gfs & MH_GF_WU) && (gfs & MH_GF_EXACT_DELHOMMEAU)))
    return fail(ctx, MH_ERR_UNSUPPORTED,
                "the frequency derivative covers the Rankine kinds with GFWu or ExactGuevelDelhommeau (got 0x%x)", gfs);
  MH_TRY(check_gfs(ctx, gfs));
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
  const bool exact = (gfs & MH_GF_EXACT_DELHOMMEAU) != 0;
  double2* gvals = nullptr;  // exact term: G, dG/dr of every unordered pair at one wavenumber
  if (exact) MH_TRY(ws_get_t(ctx, kSlotEgd, (size_t)(2 * egd_packed_pairs(n)), &gvals));
  auto times = [&](const double2* A, const double2* in, double2* out) {
    zgemm_nn_batched(s0, lc, d, A, in, nrhs, bstride, out, work);
  };
  for (int64_t w = 0; w < n_omega; ++w) {
    const double om = omegas[w];
    launch_assemble_wave(s0, lc, p, SR, DR, 1, ks_all + w, S, D, (int64_t)nn, st ? 0 : 1);
    if (exact) {
      const double kw = om * om / g;
      launch_egd_pair_values(s0, lc, p, kw, gvals);
      launch_egd_dk(s0, lc, p, kw, gvals, dS, dD);
    } else if (gfs & MH_GF_WU) {
      launch_wave_dk(s0, lc, p, ks_all + w, dS, dD);
    } else {
      MH_CUDA(ctx, cudaMemsetAsync(dS, 0, sizeof(double2) * nn, s0));
      MH_CUDA(ctx, cudaMemsetAsync(dD, 0, sizeof(double2) * nn, s0));
    }
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

int mh_hydro_gradient(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                      uint32_t gfs, int direct, int64_t n_dofs, const double* dofs, int64_t n_obj, const int32_t* obj_idx,
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
  MH_TRY(hydro_vjp_core(ctx, m, n_omega, omegas, rho, g, gfs, direct, n_dofs, dofs, n_obj, obj_idx, n_obj, obj_idx,
                        bar.data(), bar.data(), 0, nullptr, nullptr, precision, J, grad_centers, grad_normals,
                        grad_areas, grad_vertices, &gd, mem));
  for (int64_t h = 0; h < n_obj; ++h)
    MH_TRY(copy_out(ctx, grad_dofs ? grad_dofs + 3 * m->n * h : nullptr, gd + (size_t)obj_idx[h] * m->n * 3,
                    sizeof(double) * 3 * m->n, mem));
  return sync(ctx, "gradient");
}

int mh_hydro_vjp(mh_context* ctx, mh_mesh* m, int64_t n_omega, const double* omegas, double rho, double g,
                 uint32_t gfs, int direct, int64_t n_dofs, const double* dofs, int64_t n_rad, const int32_t* rad_idx,
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
  MH_TRY(hydro_vjp_core(ctx, m, n_omega, omegas, rho, g, gfs, direct, n_dofs, dofs, n_rad, rad_idx, n_inf, inf_idx,
                        ab.data(), bb.data(), n_beta, hb.data(), fb.data(), precision, J, grad_centers, grad_normals,
                        grad_areas, grad_vertices, &gd, mem));
  MH_TRY(copy_out(ctx, grad_dofs, gd, sizeof(double) * 3 * m->n * n_dofs, mem));
  return sync(ctx, "vector-Jacobian product");
}

int mh_solve_pullback(mh_context* ctx, int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc,
                      int direct, const double* phi_bar, const double* sources_bar, int precision, double* phi,
                      double* sources, double* D_bar, double* S_bar, double* bc_bar, int mem) {
  NvtxRange nvtx_range("mh_solve_pullback");
  if (!ctx) return MH_ERR_ARG;
  if (n <= 0 || nrhs <= 0) return fail(ctx, MH_ERR_ARG, "bad sizes n=%lld nrhs=%lld", (long long)n, (long long)nrhs);
  if (!D || !S || !bc || !phi_bar || !phi) return fail(ctx, MH_ERR_ARG, "D, S, bc, phi_bar and phi must not be NULL");
  if (!direct && !sources) return fail(ctx, MH_ERR_ARG, "the indirect method needs a `sources` buffer");
  if (direct && sources_bar) return fail(ctx, MH_ERR_ARG, "the direct method has no sources to take a cotangent of");
  if (precision != MH_PREC_FP64 && precision != MH_PREC_MIXED && precision != MH_PREC_FP64_TC)
    return fail(ctx, MH_ERR_ARG, "bad precision %d", precision);
  if (mem != MH_MEM_HOST && mem != MH_MEM_DEVICE) return fail(ctx, MH_ERR_ARG, "bad memory kind %d", mem);
  if (n > kMaxOrder) return fail(ctx, MH_ERR_UNSUPPORTED, "order %lld exceeds the supported %lld", (long long)n, (long long)kMaxOrder);
  MH_TRY(set_device(ctx));
  const size_t nn = (size_t)n * (size_t)n, nx = (size_t)n * (size_t)nrhs;
  cudaStream_t st = ctx->stream;
  const LaunchCounter lc = ctx->lc();
  double2 *Ad, *Sd, *Bd, *Pb, *X, *T, *Y, *work;
  MH_TRY(ws_get_t(ctx, kSlotA64, nn, &Ad));
  MH_TRY(ws_get_t(ctx, kSlotS, nn, &Sd));
  MH_TRY(ws_get_t(ctx, kSlotIn, nx, &Bd));
  MH_TRY(ws_get_t(ctx, kSlotLam, nx, &Pb));
  MH_TRY(ws_get_t(ctx, kSlotT, nx, &T));
  MH_TRY(ws_get_t(ctx, kSlotY, nx, &Y));
  MH_TRY(copy_in(ctx, Ad, D, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Sd, S, nn * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Bd, bc, nx * sizeof(double2), mem));
  MH_TRY(copy_in(ctx, Pb, phi_bar, nx * sizeof(double2), mem));
  const BatchDesc d{n, 1, (int64_t)nn};
  // the adjoint solve A^H x = rhs with the factors of the forward solve (FP64 modes), or a
  // fresh mixed-precision solve of the caller's matrix
  auto adjoint_solve = [&](double2* rhs) -> int {
    if (precision == MH_PREC_MIXED) {
      MH_TRY(copy_in(ctx, Ad, D, nn * sizeof(double2), mem));
      return solve_core(ctx, d, Ad, rhs, nrhs, (int64_t)nx, precision, true);
    }
    int32_t* ipiv;
    MH_TRY(ws_get_t(ctx, kSlotIpiv, (size_t)n, &ipiv));
    lu_solve_batched<double>(st, lc, d, Ad, ipiv, rhs, nrhs, (int64_t)nx, true);
    return check_launch(ctx, "adjoint solve");
  };
  MH_TRY(ws_get_t(ctx, kSlotX, nx, &X));
  if (direct) {
    // phi = D^-1 (S bc);  lam = D^-H phi_bar;  D_bar = -lam phi^H, S_bar = lam bc^H, bc_bar = S^H lam
    MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
    zgemm_nn_batched(st, lc, d, Sd, Bd, nrhs, (int64_t)nx, X, work);
    MH_TRY(check_launch(ctx, "S*bc"));
    MH_TRY(solve_core(ctx, d, Ad, X, nrhs, (int64_t)nx, precision, false));
    MH_CUDA(ctx, cudaMemcpyAsync(T, Pb, nx * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MH_TRY(adjoint_solve(T));
    MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
    zgemm_adj_batched(st, lc, d, Sd, T, nrhs, (int64_t)nx, Y, work);  // bc_bar
    launch_outer_adj(st, lc, n, (int)nrhs, T, Bd, 1.0, Sd);            // S_bar (S no longer needed)
    launch_outer_adj(st, lc, n, (int)nrhs, T, X, -1.0, Ad);            // D_bar
    MH_TRY(check_launch(ctx, "pullback"));
    MH_TRY(copy_out(ctx, phi, X, nx * sizeof(double2), mem));
  } else {
    // sigma = K^-1 bc, phi = S sigma;  lam = K^-H (S^H phi_bar + sources_bar);
    // S_bar = phi_bar sigma^H, K_bar = -lam sigma^H, bc_bar = lam
    MH_CUDA(ctx, cudaMemcpyAsync(X, Bd, nx * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MH_TRY(solve_core(ctx, d, Ad, X, nrhs, (int64_t)nx, precision, false));
    MH_TRY(ws_get_t(ctx, kSlotWork, zgemm_work_elems(n, nrhs, 1), &work));
    zgemm_nn_batched(st, lc, d, Sd, X, nrhs, (int64_t)nx, Y, work);    // phi
    zgemm_adj_batched(st, lc, d, Sd, Pb, nrhs, (int64_t)nx, T, work);  // S^H phi_bar
    if (sources_bar) {
      double2* sb;
      MH_TRY(ws_get_t(ctx, kSlotR, nx, &sb));
      MH_TRY(copy_in(ctx, sb, sources_bar, nx * sizeof(double2), mem));
      launch_zaxpy(st, lc, (int64_t)nx, 1.0, sb, T);
    }
    MH_TRY(check_launch(ctx, "S products"));
    MH_TRY(adjoint_solve(T));                                          // lam
    launch_outer_adj(st, lc, n, (int)nrhs, Pb, X, 1.0, Sd);            // S_bar
    launch_outer_adj(st, lc, n, (int)nrhs, T, X, -1.0, Ad);            // K_bar
    MH_TRY(check_launch(ctx, "pullback"));
    MH_TRY(copy_out(ctx, phi, Y, nx * sizeof(double2), mem));
    MH_TRY(copy_out(ctx, sources, X, nx * sizeof(double2), mem));
  }
  if (D_bar) MH_TRY(copy_out(ctx, D_bar, Ad, nn * sizeof(double2), mem));
  if (S_bar) MH_TRY(copy_out(ctx, S_bar, Sd, nn * sizeof(double2), mem));
  if (bc_bar) MH_TRY(copy_out(ctx, bc_bar, direct ? Y : T, nx * sizeof(double2), mem));
  return sync(ctx, "solve pullback");
}

}  // extern "C"
