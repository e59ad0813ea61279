// mh_noalloc.cu -- influence-matrix assembly that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs under a device-memory pool
// which already owns the GPU's memory (a Julia CUDA.jl session, a framework with
// its own caching allocator), or code that must not allocate once it has been
// initialised (fixed-footprint services, real-time loops).  For them this file
// provides mh_assemble_matrices_noalloc: the caller passes device buffers for the
// mesh and for S and D, and the only scratch the assembly needs -- one 256-byte
// panel record per panel (the Birk local frame, area centroid and local corners)
// -- lives in a fixed file-scope device array, so no call allocates.
//
// The array holds at most kNoAllocMaxPanels records (2 MiB); every GPU that
// loads this library keeps it until the process exits.  All calls share it and
// it keeps the previous call's contents: each call rewrites the records of its
// own panels before reading them, so nothing needs clearing, but two calls whose
// work overlaps on the GPU (different streams, or different host threads) race
// on it.
//
// Set-up: the first call in a CUDA context (per device, and again after the
// context is replaced, e.g. by cudaDeviceReset) looks up the array's device
// address with cudaGetSymbolAddress and loads the module of every kernel the
// entry point launches.  Loading a module can allocate (the 2 MiB array comes
// into being then), so that first call belongs before any stream capture and may
// fail with MH_ERR_CUDA when the pool leaves no room for the module.
#include <cuda_runtime.h>

#include <mutex>

#include "mh_greens.cuh"
#include "mh_internal.cuh"

namespace mh {

namespace {

constexpr int64_t kNoAllocMaxPanels = 8192;
constexpr int kRows = 128;
constexpr int kCols = 8;
constexpr uint32_t kNoAllocKinds = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE |
                                   MH_GF_WU;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) PanelRec g_noalloc_panels[kNoAllocMaxPanels];

template <bool DIRECT>
__global__ void __launch_bounds__(128) noalloc_assembly_kernel(int64_t n, const PanelRec* __restrict__ P,
                                                               uint32_t gfs, int include_identity, int has_fixed,
                                                               double fx, double fy, double fz, double k,
                                                               double2* __restrict__ S, double2* __restrict__ D);

// Host-side: the device address of g_noalloc_panels per device, valid for the CUDA
// context it was looked up in.  (In host code the symbol name is only a host-side
// stand-in for the array, not a device address.)  The context is identified by the
// driver's context id, reached through the runtime's driver entry-point query so the
// library needs no link against libcuda; without it the address is looked up on
// every call.
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

struct NoAllocSetup {
  unsigned long long ctx_id = 0;  // 0: not set up
  PanelRec* panels = nullptr;
};

std::mutex g_setup_mutex;
NoAllocSetup g_setup[kMaxDevices];
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_ctx_fns_resolved = false;

unsigned long long current_context_id() {
  if (!g_ctx_fns_resolved) {
    g_ctx_fns_resolved = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != 0 || !ctx || g_ctx_get_id(ctx, &id) != 0) return 0;
  return id;
}

// Once per device and context, with that device current: the array's address, and every
// kernel of the entry point loaded now rather than lazily at a later (possibly captured)
// launch.
int panels_address(int device, PanelRec** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  NoAllocSetup& su = g_setup[device];
  const unsigned long long id = current_context_id();
  if (id == 0 || su.ctx_id != id) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_panels) != cudaSuccess) return MH_ERR_CUDA;
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, noalloc_assembly_kernel<true>) != cudaSuccess ||
        cudaFuncGetAttributes(&attr, noalloc_assembly_kernel<false>) != cudaSuccess ||
        load_panel_geometry_kernel() != cudaSuccess)
      return MH_ERR_CUDA;
    su.panels = static_cast<PanelRec*>(p);
    su.ctx_id = id;
  }
  *out = su.panels;
  return MH_OK;
}

// Static (Birk Rankine + image) and Wu parts of one pair, summed in the same
// order as the cached-static path: S = scale*s_static + scale*s_wave.
template <bool DIRECT>
__global__ void __launch_bounds__(128) noalloc_assembly_kernel(int64_t n, const PanelRec* __restrict__ P,
                                                               uint32_t gfs, int include_identity, int has_fixed,
                                                               double fx, double fy, double fz, double k,
                                                               double2* __restrict__ S, double2* __restrict__ D) {
  __shared__ PanelRec sp[kCols];
  const int64_t i = blockIdx.x * (int64_t)kRows + threadIdx.x;
  const int64_t j0 = blockIdx.y * (int64_t)kCols;
  const int64_t avail = n - j0;
  const int ncol = (int)(avail < kCols ? avail : kCols);
  {
    const double2* src = reinterpret_cast<const double2*>(P + j0);
    double2* dst = reinterpret_cast<double2*>(sp);
    for (int q = threadIdx.x; q < ncol * 16; q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  if (i >= n) return;
  double ci[3], ni[3];
  for (int c = 0; c < 3; ++c) { ci[c] = P[i].c[c]; ni[c] = P[i].n[c]; }
  const bool need_R = (gfs & MH_GF_RANKINE) != 0;
  const bool need_I = (gfs & MH_GF_RANKINE_REFLECTED) != 0;
  const bool need_N = (gfs & MH_GF_RANKINE_REFLECTED_NEGATIVE) != 0;
  const bool has_static = need_R || need_I || need_N;
  const bool has_wave = (gfs & MH_GF_WU) != 0;
  const double image_sign = (need_I ? 1.0 : 0.0) + (need_N ? -1.0 : 0.0);
  const double jump = has_fixed ? 0.5 * (fx * ni[0] + fy * ni[1] + fz * ni[2]) : 0.5;
  for (int jj = 0; jj < ncol; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    double nv[3];
    if (has_fixed) { nv[0] = fx; nv[1] = fy; nv[2] = fz; }
    else if (DIRECT) { nv[0] = Pj.n[0]; nv[1] = Pj.n[1]; nv[2] = Pj.n[2]; }
    else { nv[0] = ni[0]; nv[1] = ni[1]; nv[2] = ni[2]; }
    double sr = 0.0, dr = 0.0;
    if (has_static) {
      double s = 0.0, d = 0.0, phi, g[3];
      if (need_R) {
        vrankine_from_geom(ci, Pj, phi, g);
        if (!DIRECT) { g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
        s += phi;
        d += nv[0] * g[0] + nv[1] * g[1] + nv[2] * g[2];
      }
      if (need_I || need_N) {
        double cr[3] = {ci[0], ci[1], -ci[2]};
        vrankine_from_geom(cr, Pj, phi, g);
        if (!DIRECT) { g[0] = -g[0]; g[1] = -g[1]; }
        s += image_sign * phi;
        d += image_sign * (nv[0] * g[0] + nv[1] * g[1] + nv[2] * g[2]);
      }
      sr = kMinusInv4Pi * s;
      dr = kMinusInv4Pi * d;
      if (include_identity && i == j) dr += jump;
    }
    double2 sv = make_double2(sr, 0.0), dv = make_double2(dr, 0.0);
    if (has_wave) {
      double2 s, d;
      const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
      const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
      wu_sd(ci, Pj.c, nv, Pj.area, k, dx1, dx2, s, d);
      sv = make_double2(kMinusInv4Pi * s.x, kMinusInv4Pi * s.y);
      dv = make_double2(kMinusInv4Pi * d.x, kMinusInv4Pi * d.y);
      if (!has_static && include_identity && i == j) dv.x += jump;
      if (has_static) {
        sv.x = sr + sv.x;
        dv.x = dr + dv.x;
      }
    }
    S[i + j * n] = sv;
    D[i + j * n] = dv;
  }
}

}  // namespace

}  // namespace mh

extern "C" int mh_assemble_matrices_noalloc(void* stream, int64_t n_panels, const double* vertices,
                                            const double* centers, const double* normals, const double* areas,
                                            const double* radii, double wavenumber, uint32_t gfs, int direct,
                                            int include_identity, const double* fixed_normal, double* S, double* D) {
  using namespace mh;
  if (n_panels <= 0 || n_panels > kNoAllocMaxPanels) return MH_ERR_ARG;
  if (!vertices || !centers || !normals || !areas || !radii || !S || !D) return MH_ERR_ARG;
  if (gfs == 0 || (gfs & ~kNoAllocKinds)) return MH_ERR_UNSUPPORTED;
  if ((gfs & MH_GF_WU) && !(wavenumber > 0)) return MH_ERR_ARG;
  // an error that earlier work left pending on this thread is reported, and left pending,
  // before anything is launched, so that it is not taken for this call's own failure
  if (cudaPeekAtLastError() != cudaSuccess) return MH_ERR_CUDA;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return MH_ERR_CUDA;
  PanelRec* panels = nullptr;
  int rc = panels_address(device, &panels);
  if (rc != MH_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const LaunchCounter none{nullptr, nullptr};
  launch_panel_geometry(st, none, n_panels, vertices, centers, normals, areas, radii, panels);
  dim3 grid((unsigned)((n_panels + kRows - 1) / kRows), (unsigned)((n_panels + kCols - 1) / kCols));
  const int has_fixed = fixed_normal ? 1 : 0;
  const double fx = has_fixed ? fixed_normal[0] : 0.0, fy = has_fixed ? fixed_normal[1] : 0.0,
               fz = has_fixed ? fixed_normal[2] : 0.0;
  if (direct)
    noalloc_assembly_kernel<true><<<grid, kRows, 0, st>>>(n_panels, panels, gfs, include_identity ? 1 : 0,
                                                          has_fixed, fx, fy, fz, wavenumber, (double2*)S,
                                                          (double2*)D);
  else
    noalloc_assembly_kernel<false><<<grid, kRows, 0, st>>>(n_panels, panels, gfs, include_identity ? 1 : 0,
                                                           has_fixed, fx, fy, fz, wavenumber, (double2*)S,
                                                           (double2*)D);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
