// mh_profile.cu -- launch accounting, per-kernel-group CUDA-event timing and FMA peak probes.
//
// When profiling is enabled on a context, every kernel launch is bracketed by two
// CUDA events recorded on the launching stream; mh_profile_read() resolves them
// into total device time and launch count per kernel group.  The probes measure
// the FP64 and FP32 fused-multiply-add throughput of the device (the roofline
// denominators of the FP64-bound assembly / LU kernels).
#include <cuda_runtime.h>

#include <algorithm>

#include <cstring>
#include <string>
#include <vector>

#include "mh_internal.cuh"
#include "mh_tc.cuh"

namespace mh {

struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaEvent_t pending = nullptr;
  struct Rec { int group; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<int64_t> count;

  cudaEvent_t take() {
    if (used == pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      pool.push_back(e);
    }
    return pool[used++];
  }
  int group_index(const char* g) {
    for (size_t i = 0; i < names.size(); ++i)
      if (names[i] == g) return (int)i;
    names.emplace_back(g);
    ms.push_back(0.0);
    count.push_back(0);
    return (int)names.size() - 1;
  }
  // requires the stream(s) to be synchronized
  void resolve() {
    for (const Rec& r : recs) {
      float t = 0.f;
      if (r.a && r.b && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) ms[r.group] += t;
      count[r.group] += 1;
    }
    recs.clear();
    used = 0;
  }
  void reset() {
    recs.clear();
    used = 0;
    names.clear();
    ms.clear();
    count.clear();
  }
  ~Profiler() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

void LaunchCounter::pre(cudaStream_t st) const {
  if (prof && prof->on) {
    prof->pending = prof->take();
    if (prof->pending) cudaEventRecord(prof->pending, st);
  }
}

void LaunchCounter::post(cudaStream_t st, const char* group) const {
  if (count) *count += 1;
  if (prof && prof->on) {
    cudaEvent_t e = prof->take();
    if (e) cudaEventRecord(e, st);
    prof->recs.push_back(Profiler::Rec{prof->group_index(group), prof->pending, e});
    prof->pending = nullptr;
  }
}

Profiler* profiler_create() { return new Profiler(); }
void profiler_destroy(Profiler* p) { delete p; }
void profiler_enable(Profiler* p, bool on) { p->on = on; }
bool profiler_on(const Profiler* p) { return p && p->on; }
void profiler_reset(Profiler* p) { p->reset(); }
int profiler_read(Profiler* p, int64_t capacity, char* names, double* total_ms, int64_t* launches, int64_t* n) {
  p->resolve();
  *n = (int64_t)p->names.size();
  for (int64_t i = 0; i < *n && i < capacity; ++i) {
    if (names) {
      std::memset(names + 32 * i, 0, 32);
      std::strncpy(names + 32 * i, p->names[i].c_str(), 31);
    }
    if (total_ms) total_ms[i] = p->ms[i];
    if (launches) launches[i] = p->count[i];
  }
  return 0;
}

namespace {

// 16 independent FMA chains per thread, the loop body unrolled 4 times so that loop
// control is ~1 instruction in 64; the peak is the best over three launch shapes
template <typename T>
__global__ void fma_probe_kernel(int iters, T a, T b, T* out) {
  T x[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) x[c] = (T)threadIdx.x * (T)1e-3 + (T)c;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 16; ++c) x[c] = fma(x[c], a, b);
  }
  T s = (T)0;
#pragma unroll
  for (int c = 0; c < 16; ++c) s += x[c];
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains live
}

template <typename T>
double run_probe(cudaStream_t st, int iters, T* scratch) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0.0;
  const int shapes[3][2] = {{8, 256}, {4, 512}, {16, 128}};  // blocks per SM, threads per block
  for (const auto& sh : shapes) {
    const int blocks = sms * sh[0], threads = sh[1];
    // warm-up long enough for the clocks to ramp, then the best of three timed runs
    for (int w = 0; w < 4; ++w) fma_probe_kernel<T><<<blocks, threads, 0, st>>>(iters, (T)0.999999, (T)1e-7, scratch);
    float ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(a, st);
      fma_probe_kernel<T><<<blocks, threads, 0, st>>>(iters, (T)0.999999, (T)1e-7, scratch);
      cudaEventRecord(b, st);
      cudaEventSynchronize(b);
      float t = 0.f;
      cudaEventElapsedTime(&t, a, b);
      if (t > 0.f && t < ms) ms = t;
    }
    const double flops = 2.0 * 16.0 * (double)iters * (double)blocks * (double)threads;
    if (ms > 0 && ms < 1e29f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

// The recovery path of every bounded completion wait in the tensor-core kernels, run
// on purpose: the CTA (one warp) holds tensor memory, waits on an mbarrier that nothing
// arrives at for `polls` polls, records the timeout, frees the tensor memory and returns.
__global__ void __launch_bounds__(32) wait_timeout_probe_kernel(uint32_t polls, int* __restrict__ flag) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  tc::tmem_alloc(&tmem_base, 32);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const bool ok = tc::mbar_wait(&bar, 0, polls);
  if (!ok && threadIdx.x == 0) atomicExch(flag, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::tmem_dealloc(tmem_base, 32);
}

}  // namespace

int probe_wait_timeout(cudaStream_t st, uint32_t polls, int* timed_out) {
  int* flag = nullptr;
  if (cudaMallocAsync((void**)&flag, sizeof(int), st) != cudaSuccess) return MH_ERR_NOMEM;
  cudaMemsetAsync(flag, 0, sizeof(int), st);
  wait_timeout_probe_kernel<<<1, 32, 0, st>>>(polls, flag);
  cudaError_t e = cudaGetLastError();
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(flag, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  *timed_out = h;
  return e == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int probe_fma_peaks(cudaStream_t st, double* fp64_tflops, double* fp32_tflops) {
  double* scratch = nullptr;
  if (cudaMallocAsync((void**)&scratch, 64, st) != cudaSuccess) return MH_ERR_NOMEM;
  double p64 = run_probe<double>(st, 1 << 14, scratch);
  double p32 = run_probe<float>(st, 1 << 15, (float*)scratch);
  cudaFreeAsync(scratch, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (fp64_tflops) *fp64_tflops = p64;
  if (fp32_tflops) *fp32_tflops = p32;
  return e == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

}  // namespace mh
