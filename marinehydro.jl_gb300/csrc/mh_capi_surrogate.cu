// mh_capi_surrogate.cu -- the learned wave-term surrogate through the C-ABI: parameters, point
// evaluation, the loss/gradient check and on-device training.
#include "mh_capi_internal.cuh"

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

extern "C" {

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
