// mh_surrogate.cu -- training and point evaluation of the learned Delhommeau
// wave-term surrogate (the network and its target are described in mh_mlp.cuh).
// No counterpart in the reference.
//
// Training data: samples (r, z) with log10(r) stratified over [-3, 3] (log-uniform r in
// [1e-3, 1e3]) and z uniform in [-50, 0], drawn from a counter-based generator (SplitMix64, Steele, Lea & Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014) so that sample q of
// a seed is the same on every device and launch shape.  Targets come from the exact
// kernel (egd_adaptive, the device restatement of exact_Guevel_Delhommeau.jl:15-46)
// and the Wu fits (wu_wave_term_and_derivs).
//
// Training step (batch B, one thread per sample):
//   mlp_fwd_bwd_kernel: forward with the BF16-rounded parameters (and BF16 activations into
//     the 64 x 64 layers, as the tensor-core assembly computes them), mean-squared
//     error, and back-propagation of the per-sample deltas (stored feature-major);
//   mlp_wgrad_kernel:   weight gradients dW = sum_b delta_b a_b^T per layer (chunks
//     of 256 samples staged in shared memory, atomically summed);
//   mlp_adam_kernel:    Adam on the FP32 master parameters, then BF16 rounding of
//     the copy the forward pass uses (quantisation-aware training).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mh_greens.cuh"
#include "mh_internal.cuh"
#include "mh_mlp.cuh"
#include "mh_wu_f32.cuh"

namespace mh {

namespace {

constexpr int kTrainThreads = 128;
constexpr int kGradChunk = 256;
constexpr int kActRows = 2 + 6 * kMlpH + kMlpOut;  // XB, H1..H3, D1..D3, G4 rows of B floats

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// sample q of M for `seed`: log10(r) stratified (one jittered point per 1/M of
// [-3, 3], so neighbouring threads get similar r and similar quadrature work),
// z uniform in [-50, 0]
__device__ __forceinline__ void sample_point(uint64_t seed, uint64_t q, uint64_t M, double& r, double& z) {
  const uint64_t h1 = splitmix64(seed ^ splitmix64(q));
  const uint64_t h2 = splitmix64(h1);
  r = exp10(-3.0 + 6.0 * (((double)q + u01(h1)) / (double)M));
  z = -50.0 * u01(h2);
}

constexpr int kSampleWarps = 4;

// one warp per sample (the exact kernel's warp-cooperative quadrature); lane 0 writes
__global__ void __launch_bounds__(32 * kSampleWarps) surrogate_samples_kernel(uint64_t seed, int64_t M,
                                                                               int64_t offset, int64_t count,
                                                                               double rtol, double atol,
                                                                               float2* __restrict__ X,
                                                                               float* __restrict__ Y8,
                                                                               double* __restrict__ R2) {
  __shared__ double sw[kSampleWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5;
  const int64_t t = blockIdx.x * (int64_t)kSampleWarps + warp;
  if (t >= count) return;  // warp-uniform
  const int64_t q = offset + t;
  double r, z;
  sample_point(seed, (uint64_t)q, (uint64_t)M, r, z);
  double2 G, Gr;
  egd_warp(r, z, rtol, atol, sw[warp], G, Gr);
  if ((threadIdx.x & 31) != 0) return;
  double2 GF, Gh, Gv;
  wu_wave_term_and_derivs(r, z, GF, Gh, Gv);
  const double d = sqrt(r * r + z * z);
  const double s = (1.0 + d) * (1.0 + d);
  const double sr = s * (1.0 + r) / r;
  const double2 Gz = make_double2(G.x + 2.0 / d, G.y);
  float u, v;
  mlp_inputs(r, z, u, v);
  X[q] = make_float2(u, v);
  float* y = Y8 + 8 * q;
  y[0] = (float)(s * (G.x - GF.x));
  y[1] = (float)(s * (G.y - GF.y));
  y[2] = (float)(sr * (Gr.x - Gh.x));
  y[3] = (float)(sr * (Gr.y - Gh.y));
  y[4] = (float)(s * (Gz.x - Gv.x));
  y[5] = (float)(s * (Gz.y - Gv.y));
  y[6] = 0.0f;
  y[7] = 0.0f;
  if (R2) {  // (r, z) in FP64 for the validation statistics
    R2[2 * q] = r;
    R2[2 * q + 1] = z;
  }
}

__device__ __forceinline__ void load_params(float4* dst, const float* __restrict__ src) {
  const float4* s4 = reinterpret_cast<const float4*>(src);
  for (int q = threadIdx.x; q < kMlpParamsPadded / 4; q += blockDim.x) dst[q] = s4[q];
}

// Hidden vectors live in shared memory, one column per thread ([feature][thread], so the
// per-thread accesses are bank-conflict free and the weights are warp-wide broadcasts).
__global__ void __launch_bounds__(kTrainThreads) mlp_fwd_bwd_kernel(const float* __restrict__ qparams,
                                                                     const float2* __restrict__ X,
                                                                     const float* __restrict__ Y8, int64_t M,
                                                                     int64_t base, int64_t prime, int B,
                                                                     float* __restrict__ acts,
                                                                     double* __restrict__ loss) {
  extern __shared__ float4 smp4[];
  __shared__ float red[kTrainThreads / 32];
  load_params(smp4, qparams);
  float* P = reinterpret_cast<float*>(smp4);
  float* ha = P + kMlpParamsPadded;
  float* hb = ha + kMlpH * kTrainThreads;
  const int t = threadIdx.x;
  const int b = blockIdx.x * blockDim.x + t;
  const bool active = b < B;
  const int64_t Bl = B;
  float* XB = acts;
  float* H1 = XB + 2 * Bl;
  float* H2 = H1 + kMlpH * Bl;
  float* H3 = H2 + kMlpH * Bl;
  float* D1 = H3 + kMlpH * Bl;
  float* D2 = D1 + kMlpH * Bl;
  float* D3 = D2 + kMlpH * Bl;
  float* G4 = D3 + kMlpH * Bl;
  float2 x = make_float2(0.0f, 0.0f);
  float y[kMlpOut] = {0, 0, 0, 0, 0, 0};
  if (active) {
    const int64_t idx = (int64_t)((((uint64_t)(base + b) % (uint64_t)M) * (uint64_t)prime) % (uint64_t)M);
    x = X[idx];
    for (int q = 0; q < kMlpOut; ++q) y[q] = Y8[8 * idx + q];
    XB[b] = x.x;
    XB[Bl + b] = x.y;
  }
  __syncthreads();
  // forward: ha = h1, hb = h2, ha = h3
  for (int j = 0; j < kMlpH; ++j) {
    const float v = bf16r(tanh_fast(fmaf(P[kMlpW1 + 2 * j], x.x, fmaf(P[kMlpW1 + 2 * j + 1], x.y, P[kMlpB1 + j]))));
    ha[j * kTrainThreads + t] = v;
    if (active) H1[j * Bl + b] = v;
  }
  for (int j = 0; j < kMlpH; ++j) {
    float acc = P[kMlpB2 + j];
#pragma unroll 16
    for (int i = 0; i < kMlpH; ++i) acc = fmaf(P[kMlpW2 + j * kMlpH + i], ha[i * kTrainThreads + t], acc);
    const float v = bf16r(tanh_fast(acc));
    hb[j * kTrainThreads + t] = v;
    if (active) H2[j * Bl + b] = v;
  }
  for (int j = 0; j < kMlpH; ++j) {
    float acc = P[kMlpB3 + j];
#pragma unroll 16
    for (int i = 0; i < kMlpH; ++i) acc = fmaf(P[kMlpW3 + j * kMlpH + i], hb[i * kTrainThreads + t], acc);
    const float v = tanh_fast(acc);
    ha[j * kTrainThreads + t] = v;  // h3
    if (active) H3[j * Bl + b] = v;
  }
  float g[kMlpOut];
  float err2 = 0.0f;
  const float gs = 2.0f / (float)(B * kMlpOut);
#pragma unroll
  for (int q = 0; q < kMlpOut; ++q) {
    float acc = P[kMlpB4 + q];
#pragma unroll 16
    for (int i = 0; i < kMlpH; ++i) acc = fmaf(P[kMlpW4 + q * kMlpH + i], ha[i * kTrainThreads + t], acc);
    const float e = active ? acc - y[q] : 0.0f;
    err2 = fmaf(e, e, err2);
    g[q] = gs * e;
    if (active) G4[q * Bl + b] = g[q];
  }
  // delta3 = W4^T g * (1 - h3^2) -> hb
  for (int i = 0; i < kMlpH; ++i) {
    float acc = 0.0f;
#pragma unroll
    for (int q = 0; q < kMlpOut; ++q) acc = fmaf(P[kMlpW4 + q * kMlpH + i], g[q], acc);
    const float h3 = ha[i * kTrainThreads + t];
    const float dv = acc * (1.0f - h3 * h3);
    hb[i * kTrainThreads + t] = dv;
    if (active) D3[i * Bl + b] = dv;
  }
  // delta2 = W3^T delta3 * (1 - h2^2) -> ha (h2 re-read from global: written by this thread)
  for (int i = 0; i < kMlpH; ++i) {
    float acc = 0.0f;
#pragma unroll 16
    for (int j = 0; j < kMlpH; ++j) acc = fmaf(P[kMlpW3 + j * kMlpH + i], hb[j * kTrainThreads + t], acc);
    const float h2 = active ? H2[i * Bl + b] : 0.0f;
    const float dv = acc * (1.0f - h2 * h2);
    ha[i * kTrainThreads + t] = dv;
    if (active) D2[i * Bl + b] = dv;
  }
  // delta1 = W2^T delta2 * (1 - h1^2)
  for (int i = 0; i < kMlpH; ++i) {
    float acc = 0.0f;
#pragma unroll 16
    for (int j = 0; j < kMlpH; ++j) acc = fmaf(P[kMlpW2 + j * kMlpH + i], ha[j * kTrainThreads + t], acc);
    if (active) {
      const float h1 = H1[i * Bl + b];
      D1[i * Bl + b] = acc * (1.0f - h1 * h1);
    }
  }
  // sum of squared errors over the CTA -> loss (mean over B * 6 outputs, accumulated)
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) err2 += __shfl_down_sync(0xffffffffu, err2, off);
  if ((t & 31) == 0) red[t >> 5] = err2;
  __syncthreads();
  if (t == 0) {
    float tot = 0.0f;
    for (int w = 0; w < kTrainThreads / 32; ++w) tot += red[w];
    atomicAdd(loss, (double)tot / (double)(B * kMlpOut));
  }
}

// dW[j][i] += sum_b D[j][b] A[i][b]; db[j] += sum_b D[j][b] over one chunk of samples;
// blockIdx.y = layer (0: W1 from the inputs, 1: W2, 2: W3, 3: W4 from the output deltas)
__global__ void __launch_bounds__(kGradChunk) mlp_wgrad_kernel(const float* __restrict__ acts, int B,
                                                                float* __restrict__ grad) {
  extern __shared__ float wsm[];
  const int layer = blockIdx.y;
  const int64_t Bl = B;
  const float* XB = acts;
  const float* H1 = XB + 2 * Bl;
  const float* H2 = H1 + kMlpH * Bl;
  const float* H3 = H2 + kMlpH * Bl;
  const float* D1 = H3 + kMlpH * Bl;
  const float* D2 = D1 + kMlpH * Bl;
  const float* D3 = D2 + kMlpH * Bl;
  const float* G4 = D3 + kMlpH * Bl;
  const float* Dl = layer == 0 ? D1 : layer == 1 ? D2 : layer == 2 ? D3 : G4;
  const float* Al = layer == 0 ? XB : layer == 1 ? H1 : layer == 2 ? H2 : H3;
  const int nout = layer == 3 ? kMlpOut : kMlpH;
  const int nin = layer == 0 ? kMlpIn : kMlpH;
  const int offW = layer == 0 ? kMlpW1 : layer == 1 ? kMlpW2 : layer == 2 ? kMlpW3 : kMlpW4;
  const int offB = layer == 0 ? kMlpB1 : layer == 1 ? kMlpB2 : layer == 2 ? kMlpB3 : kMlpB4;
  constexpr int kLd = kMlpH + 1;
  float* Ds = wsm;                       // [chunk][kLd]
  float* As = wsm + kGradChunk * kLd;    // [chunk][kLd]
  const int b0 = blockIdx.x * kGradChunk;
  const int nb = min(kGradChunk, B - b0);
  for (int q = threadIdx.x; q < kGradChunk * nout; q += blockDim.x) {
    const int f = q / kGradChunk, t = q % kGradChunk;
    Ds[t * kLd + f] = t < nb ? Dl[f * Bl + b0 + t] : 0.0f;
  }
  for (int q = threadIdx.x; q < kGradChunk * nin; q += blockDim.x) {
    const int f = q / kGradChunk, t = q % kGradChunk;
    As[t * kLd + f] = t < nb ? Al[f * Bl + b0 + t] : 0.0f;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nout * nin; q += blockDim.x) {
    const int j = q / nin, i = q % nin;
    float acc = 0.0f;
    for (int t = 0; t < nb; ++t) acc = fmaf(Ds[t * kLd + j], As[t * kLd + i], acc);
    atomicAdd(grad + offW + q, acc);
  }
  for (int j = threadIdx.x; j < nout; j += blockDim.x) {
    float acc = 0.0f;
    for (int t = 0; t < nb; ++t) acc += Ds[t * kLd + j];
    atomicAdd(grad + offB + j, acc);
  }
}

__global__ void mlp_adam_kernel(float* __restrict__ theta, float* __restrict__ qparams, float* __restrict__ grad,
                                float* __restrict__ m1, float* __restrict__ m2, float lr, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParamsPadded) return;
  if (p >= kMlpParams) {
    qparams[p] = 0.0f;
    return;
  }
  const float g = grad[p];
  const float a = 0.9f * m1[p] + 0.1f * g;
  const float v = 0.999f * m2[p] + 0.001f * g * g;
  m1[p] = a;
  m2[p] = v;
  const float th = theta[p] - lr * (a * c1) / (sqrtf(v * c2) + 1e-8f);
  theta[p] = th;
  qparams[p] = __bfloat162float(__float2bfloat16_rn(th));
  grad[p] = 0.0f;
}

__global__ void round_bf16_kernel(const float* __restrict__ in, float* __restrict__ out, int count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParamsPadded) return;
  out[p] = p < count ? __bfloat162float(__float2bfloat16_rn(in[p])) : 0.0f;
}

// surrogate GF, Gh, Gv at points (r, z) (the layout of the Wu point evaluator), one warp per
// point; points outside the training box take the exact kernel (warp-cooperative, as in
// assembly), inside it lane 0 evaluates the Wu terms and the network
__global__ void __launch_bounds__(32 * kSampleWarps) surrogate_points_kernel(const float* __restrict__ mlp, int64_t m,
                                                                              const double* __restrict__ r,
                                                                              const double* __restrict__ z,
                                                                              double rtol, double atol,
                                                                              double2* __restrict__ out) {
  extern __shared__ float4 spp4[];
  __shared__ double sw[kSampleWarps][8 * kGKWarpStack];
  load_params(spp4, mlp);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = blockIdx.x * (int64_t)kSampleWarps + warp;
  if (q >= m) return;  // warp-uniform
  const double rq = r[q], zq = z[q];
  double2 GF, Gh, Gv;
  if (surrogate_in_box((float)rq, (float)zq)) {
    // FP32 throughout, as the tensor-core assembly (wave_kernel_tc)
    if (lane != 0) return;
    const float rf = (float)rq, zf = (float)zq;
    float2 g, gh, gv, dG, dGr, dGz;
    wu_wave_term_and_derivs_f32(rf, zf, g, gh, gv);
    surrogate_correction(reinterpret_cast<const float*>(spp4), rf, zf, dG, dGr, dGz);
    GF = make_double2(g.x + dG.x, g.y + dG.y);
    Gh = make_double2(gh.x + dGr.x, gh.y + dGr.y);
    Gv = make_double2(gv.x + dGz.x, gv.y + dGz.y);
  } else {
    egd_warp(rq, zq, rtol, atol, sw[warp], GF, Gh);
    if (lane != 0) return;
    Gv = make_double2(GF.x + 2.0 / hypot(rq, zq), GF.y);
  }
  out[3 * q] = GF;
  out[3 * q + 1] = Gh;
  out[3 * q + 2] = Gv;
}

}  // namespace

int64_t mlp_act_floats(int B) { return (int64_t)kActRows * B; }

void launch_surrogate_samples(cudaStream_t st, LaunchCounter lc, uint64_t seed, int64_t M, int64_t offset,
                              int64_t count, double rtol, double atol, float2* X, float* Y8, double* R2) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "surrogate_samples",
            surrogate_samples_kernel<<<(unsigned)((count + kSampleWarps - 1) / kSampleWarps), 32 * kSampleWarps, 0,
                                       st>>>(seed, M, offset, count, rtol, atol, X, Y8, R2));
}

void launch_mlp_loss_grad(cudaStream_t st, LaunchCounter lc, const float* qparams, const float2* X, const float* Y8,
                          int64_t M, int64_t base, int64_t prime, int B, float* acts, double* loss, float* grad) {
  const size_t psmem = sizeof(float) * (kMlpParamsPadded + 2 * kMlpH * kTrainThreads);
  cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem);
  MH_LAUNCH(lc, st, "mlp_fwd_bwd",
            mlp_fwd_bwd_kernel<<<(unsigned)((B + kTrainThreads - 1) / kTrainThreads), kTrainThreads, psmem, st>>>(
                qparams, X, Y8, M, base, prime, B, acts, loss));
  const size_t gsmem = sizeof(float) * 2 * kGradChunk * (kMlpH + 1);
  cudaFuncSetAttribute(mlp_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsmem);
  dim3 g2((unsigned)((B + kGradChunk - 1) / kGradChunk), 4);
  MH_LAUNCH(lc, st, "mlp_wgrad", mlp_wgrad_kernel<<<g2, kGradChunk, gsmem, st>>>(acts, B, grad));
}

void launch_mlp_train_step(cudaStream_t st, LaunchCounter lc, float* theta, float* qparams, float* grad, float* m1,
                           float* m2, const float2* X, const float* Y8, int64_t M, int64_t base, int64_t prime, int B,
                           float* acts, double* loss, float lr, int t) {
  launch_mlp_loss_grad(st, lc, qparams, X, Y8, M, base, prime, B, acts, loss, grad);
  const float c1 = 1.0f / (1.0f - powf(0.9f, (float)t)), c2 = 1.0f / (1.0f - powf(0.999f, (float)t));
  MH_LAUNCH(lc, st, "mlp_adam",
            mlp_adam_kernel<<<(kMlpParamsPadded + 255) / 256, 256, 0, st>>>(theta, qparams, grad, m1, m2, lr, c1,
                                                                              c2));
}

void launch_round_bf16(cudaStream_t st, LaunchCounter lc, const float* in, float* out) {
  MH_LAUNCH(lc, st, "round_bf16",
            round_bf16_kernel<<<(kMlpParamsPadded + 255) / 256, 256, 0, st>>>(in, out, kMlpParams));
}

void launch_surrogate_points(cudaStream_t st, LaunchCounter lc, const float* mlp, int64_t m, const double* r,
                             const double* z, double rtol, double atol, double2* out) {
  if (m <= 0) return;
  const size_t psmem = sizeof(float) * kMlpParamsPadded;
  MH_LAUNCH(lc, st, "surrogate_points",
            surrogate_points_kernel<<<(unsigned)((m + kSampleWarps - 1) / kSampleWarps), 32 * kSampleWarps, psmem,
                                      st>>>(mlp, m, r, z, rtol, atol, out));
}

}  // namespace mh
