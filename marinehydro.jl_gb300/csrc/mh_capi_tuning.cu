// mh_capi_tuning.cu -- the batched LU's launch-shape table and its autotuner (mh_tile_table_*, mh_autotune).
#include "mh_capi_internal.cuh"

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
  // candidates: the cluster bound of the panel and, for the BF16x3 update, the column tiles
  // per CTA; the first candidate is the default shape
  std::vector<TileChoice> cands;
  const int caps[3] = {8, 4, 2};
  const int groups[4] = {4, 1, 2, 8};  // BF16x3 column tiles per CTA, the default first
  for (int cap : caps) {
    if (precision != MH_PREC_MIXED) {  // FP64 and FP64-TC: the panel's cluster bound only
      TileChoice c;
      c.cluster_f64 = cap;
      cands.push_back(c);
      continue;
    }
    for (int gi = 0; gi < 4; ++gi) {
      TileChoice c;
      c.bx_group = groups[gi];
      c.cluster_f32 = cap;
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

}  // extern "C"
