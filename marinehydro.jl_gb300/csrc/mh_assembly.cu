// mh_assembly.cu -- influence-matrix assembly kernels (sm_103a, FP64).
//
// Replaces the reference's StaticArraysMesh assembly (matrix_assembly.jl:167-369)
// and its GPU broadcast / KernelAbstractions kernels (matrix_assembly.jl:56-128).
//
// Layout: S and D are n x n column-major.  A CTA owns 128 consecutive rows i
// (one thread per row, so the complex stores of a column are coalesced) and
// kColsPerCta consecutive columns j; the source-panel records of its columns are
// staged in shared memory and read as warp-wide broadcasts, the field-panel data
// of its row stays in registers.
//
// The wavenumber-independent part (Rankine + image, and the identity jump) is a
// separate kernel writing real n x n arrays, so a frequency sweep computes it
// once per mesh (the reference re-assembles it for every problem; the sum
// S = S_static + S_wave is the reference's own split, matrix_assembly.jl:183-208).
#include <cuda_runtime.h>

#include <algorithm>

#include "mh_greens.cuh"
#include "mh_internal.cuh"
#include "mh_mlp.cuh"
#include "mh_tc.cuh"
#include "mh_wu_f32.cuh"

namespace mh {

namespace {

constexpr int kRowsPerCta = 128;
constexpr int kColsPerCta = 8;

constexpr uint32_t kBirkKinds = MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_RANKINE_REFLECTED_NEGATIVE;
constexpr uint32_t kDelhKinds = MH_GF_DELHOMMEAU_RANKINE | MH_GF_DELHOMMEAU_RANKINE_REFLECTED;

// birk_panel_geometry (rankine_vectorized.jl:79-137) for every panel, plus the
// mesh's own center / normal / area / radius.
__global__ void panel_geometry_kernel(int64_t n, const double* __restrict__ V, const double* __restrict__ C,
                                      const double* __restrict__ N, const double* __restrict__ A,
                                      const double* __restrict__ R, PanelRec* __restrict__ out) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double* v = V + 12 * j;
  double mid[4][3], mgc[3], s[3], tt[3], nn[3], t[3];
  for (int i = 0; i < 4; ++i) {
    int ip = (i + 1) & 3;
    for (int c = 0; c < 3; ++c) mid[i][c] = (v[3 * i + c] + v[3 * ip + c]) / 2;
  }
  for (int c = 0; c < 3; ++c) {
    mgc[c] = (mid[1][c] + mid[3][c]) / 2;
    s[c] = mid[1][c] - mid[3][c];
    tt[c] = mid[2][c] - mid[0][c];
  }
  double ns = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  for (int c = 0; c < 3; ++c) s[c] /= ns;
  nn[0] = s[1] * tt[2] - s[2] * tt[1];
  nn[1] = s[2] * tt[0] - s[0] * tt[2];
  nn[2] = s[0] * tt[1] - s[1] * tt[0];
  double nl = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
  for (int c = 0; c < 3; ++c) nn[c] /= nl;
  t[0] = nn[1] * s[2] - nn[2] * s[1];
  t[1] = nn[2] * s[0] - nn[0] * s[2];
  t[2] = nn[0] * s[1] - nn[1] * s[0];
  double tl = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  for (int c = 0; c < 3; ++c) t[c] /= tl;
  double tc[4][2];
  for (int k = 0; k < 4; ++k) {
    double d0 = v[3 * k] - mgc[0], d1 = v[3 * k + 1] - mgc[1], d2 = v[3 * k + 2] - mgc[2];
    tc[k][0] = d0 * s[0] + d1 * s[1] + d2 * s[2];
    tc[k][1] = d0 * t[0] + d1 * t[1] + d2 * t[2];
  }
  double Ar = 0.0, Mx = 0.0, My = 0.0;
  for (int k = 0; k < 4; ++k) {
    int kn = (k + 1) & 3;
    double xk = tc[k][0], yk = tc[k][1], xk1 = tc[kn][0], yk1 = tc[kn][1];
    Ar += (yk1 - yk) * (xk + xk1) / 2;
    Mx += (xk1 - xk) * (yk * yk + yk * yk1 + yk1 * yk1) / 6;
    My += (yk1 - yk) * (xk * xk + xk * xk1 + xk1 * xk1) / 6;
  }
  double clx = My / Ar, cly = -Mx / Ar;
  PanelRec P;
  for (int c = 0; c < 3; ++c) {
    P.T[c] = s[c];
    P.T[3 + c] = t[c];
    P.T[6 + c] = nn[c];
    P.qgc[c] = mgc[c] + clx * s[c] + cly * t[c];
    P.c[c] = C[3 * j + c];
    P.n[c] = N[3 * j + c];
  }
  for (int k = 0; k < 4; ++k) {
    P.lc[2 * k] = tc[k][0] - clx;
    P.lc[2 * k + 1] = tc[k][1] - cly;
  }
  P.area = A[j];
  P.radius = R[j];
  for (int k = 0; k < 4; ++k) {  // the same expression the Birk integral evaluated per pair
    const int kn = (k + 1) & 3;
    P.edge[k] = hypot(P.lc[2 * kn] - P.lc[2 * k], P.lc[2 * kn + 1] - P.lc[2 * k + 1]);
  }
  out[j] = P;
}

__device__ __forceinline__ void stage_panels(PanelRec* sp, const PanelRec* __restrict__ P, int64_t j0, int64_t n) {
  // kColsPerCta records of 16 double2 each
  const double2* src = reinterpret_cast<const double2*>(P + j0);
  double2* dst = reinterpret_cast<double2*>(sp);
  int64_t avail = n - j0;
  int cnt = (int)(avail < kColsPerCta ? avail : kColsPerCta) * 16;
  for (int q = threadIdx.x; q < cnt; q += blockDim.x) dst[q] = __ldg(src + q);
}

template <bool DIRECT>
__device__ __forceinline__ void pick_normal(const AssemblyParams& p, const PanelRec& Pj, const double ni[3],
                                            double nv[3]) {
  // _panel_or_fixed (matrix_assembly.jl:228-230)
  if (p.has_fixed) { nv[0] = p.fixed[0]; nv[1] = p.fixed[1]; nv[2] = p.fixed[2]; }
  else if (DIRECT) { nv[0] = Pj.n[0]; nv[1] = Pj.n[1]; nv[2] = Pj.n[2]; }
  else { nv[0] = ni[0]; nv[1] = ni[1]; nv[2] = ni[2]; }
}

__device__ __forceinline__ double identity_jump(const AssemblyParams& p, const double ni[3]) {
  // _add_identity! (matrix_assembly.jl:234-245)
  if (p.has_fixed) return 0.5 * (p.fixed[0] * ni[0] + p.fixed[1] * ni[1] + p.fixed[2] * ni[2]);
  return 0.5;
}

// Static (Rankine-family) part.  BIRK: assemble_birk_rankine (matrix_assembly.jl:274-331);
// otherwise the broadcasting sum over the static tuple (matrix_assembly.jl:70-88).
template <bool DIRECT, bool BIRK>
__global__ void __launch_bounds__(kRowsPerCta) static_kernel(AssemblyParams p, double* __restrict__ SR,
                                                             double* __restrict__ DR) {
  __shared__ PanelRec sp[kColsPerCta];
  const int64_t n = p.n;
  const int64_t i = blockIdx.x * (int64_t)kRowsPerCta + threadIdx.x;
  const int64_t j0 = blockIdx.y * (int64_t)kColsPerCta;
  stage_panels(sp, p.P, j0, n);
  __syncthreads();
  if (i >= n) return;
  double ci[3], ni[3];
  for (int c = 0; c < 3; ++c) { ci[c] = __ldg(&p.P[i].c[c]); ni[c] = __ldg(&p.P[i].n[c]); }
  const bool need_R = (p.gfs & MH_GF_RANKINE) != 0;
  const bool need_I = (p.gfs & MH_GF_RANKINE_REFLECTED) != 0;
  const bool need_N = (p.gfs & MH_GF_RANKINE_REFLECTED_NEGATIVE) != 0;
  const double image_sign = (need_I ? 1.0 : 0.0) + (need_N ? -1.0 : 0.0);
  const int jmax = (int)((n - j0) < kColsPerCta ? (n - j0) : kColsPerCta);
  for (int jj = 0; jj < jmax; ++jj) {
    const int64_t j = j0 + jj;
    const PanelRec& Pj = sp[jj];
    double nv[3];
    pick_normal<DIRECT>(p, Pj, ni, nv);
    double s = 0.0, d = 0.0;
    if (BIRK) {
      double phi, g[3];
      if (need_R) {
        vrankine_from_geom(ci, Pj, phi, g);
        if (!DIRECT) { g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
        s += phi;
        d += nv[0] * g[0] + nv[1] * g[1] + nv[2] * g[2];
      }
      if (need_I || need_N) {
        double cr[3] = {ci[0], ci[1], -ci[2]};
        vrankine_from_geom(cr, Pj, phi, g);
        if (!DIRECT) { g[0] = -g[0]; g[1] = -g[1]; }  // vertical_reflection(-g)
        s += image_sign * phi;
        d += image_sign * (nv[0] * g[0] + nv[1] * g[1] + nv[2] * g[2]);
      }
    } else {
      // canonical tuple order: Rankine, RankineReflected, RankineReflectedNegative,
      // DelhommeauRankine, DelhommeauRankineReflected
      const double* vj = p.V + 12 * j;
      double v12[12];
      for (int q = 0; q < 12; ++q) v12[q] = __ldg(vj + q);
      double gs[3] = {0.0, 0.0, 0.0};
      const uint32_t kinds[5] = {MH_GF_RANKINE, MH_GF_RANKINE_REFLECTED, MH_GF_RANKINE_REFLECTED_NEGATIVE,
                                 MH_GF_DELHOMMEAU_RANKINE, MH_GF_DELHOMMEAU_RANKINE_REFLECTED};
      for (int q = 0; q < 5; ++q) {
        const uint32_t kd = kinds[q];
        if (!(p.gfs & kd)) continue;
        const bool refl = kd == MH_GF_RANKINE_REFLECTED || kd == MH_GF_RANKINE_REFLECTED_NEGATIVE ||
                          kd == MH_GF_DELHOMMEAU_RANKINE_REFLECTED;
        double pt[3] = {ci[0], ci[1], refl ? -ci[2] : ci[2]};
        double I, g[3];
        if (kd & kBirkKinds) {
          vrankine_from_geom(pt, Pj, I, g);
          if (!DIRECT) { g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
        } else {
          delhommeau_rankine(pt, Pj, v12, !DIRECT, I, g);
        }
        if (refl && !DIRECT) g[2] = -g[2];
        if (kd == MH_GF_RANKINE_REFLECTED_NEGATIVE) { I = -I; g[0] = -g[0]; g[1] = -g[1]; g[2] = -g[2]; }
        s += I;
        gs[0] += g[0]; gs[1] += g[1]; gs[2] += g[2];
      }
      d = nv[0] * gs[0] + nv[1] * gs[1] + nv[2] * gs[2];
    }
    double sv = kMinusInv4Pi * s, dv = kMinusInv4Pi * d;
    if (p.include_identity && i == j) dv += identity_jump(p, ni);
    SR[i + j * n] = sv;
    DR[i + j * n] = dv;
  }
}

// Wave part for a batch of wavenumbers (blockIdx.z), added to the cached static
// part.  WU: the fused centres loop (matrix_assembly.jl:343-369, wu.jl:104-127);
// EGD (or Wu + EGD): broadcasting sum over the wave tuple (matrix_assembly.jl:70-88).
//
// The wave term depends on the pair only through hh = k |x_h - xi_h| and
// vv = k (z + zeta), both symmetric in (i, j) in IEEE arithmetic, so each
// unordered pair {i, j} evaluates the special functions once and writes both
// S/D entries: for (j, i) the horizontal gradient factors are the exact negations
// of those of (i, j) and the area / normal are swapped.  The result is the same
// as evaluating every ordered pair.  CTAs whose tile lies strictly below the
// diagonal exit at once; within a tile, a thread handles the pairs with i <= j.
struct WaveTerms {
  double2 I;    // -1/4pi times the integral, without the source area
  double2 Gh;   // -1/4pi times the horizontal gradient factor: the gradient component c of the
                // (i, j) orientation is Gh dx_c
  double2 Gz;   // -1/4pi times the vertical gradient component
};

// the wave terms of one exact Delhommeau pair from its integrals G and dG/dr at (r, z)
__device__ __forceinline__ WaveTerms egd_wave_terms(double r, double z, double k, double2 GF, double2 dGdr) {
  const double kc1 = kMinusInv4Pi * k, kc2 = kc1 * k, kc3 = kc2 * k;
  const double2 dGdz = make_double2(GF.x + 2 / hypot(r, z), GF.y);
  const double a = fabs(r) > 1e-6 ? kc3 / r : 0.0;
  WaveTerms w;
  w.I = make_double2(kc1 * GF.x, kc1 * GF.y);
  w.Gh = make_double2(a * dGdr.x, a * dGdr.y);
  w.Gz = make_double2(kc2 * dGdz.x, kc2 * dGdz.y);
  return w;
}

// WMODE bits: 1 = Wu, 2 = exact Delhommeau (the learned surrogate has its own kernel,
// wave_kernel_tc).  kc[m] = -k^m / 4pi (m = 1, 2, 3), the pair-independent factors of the
// terms: I = kc1 G, Gh dx_c = kc3 (1/hh) dx_c dG/dh, Gz = kc2 dG/dz (wu.jl:118-126).
template <bool DIRECT, int WMODE>
__device__ __forceinline__ void wave_terms(const AssemblyParams& p, const double ci[3], const double cj[3], double k,
                                           const double kc[4], WaveTerms& w) {
  w.I = make_double2(0.0, 0.0);
  w.Gh = w.Gz = w.I;
  if (WMODE & 1) {  // _wu_sd (wu.jl:112-127)
    double hh, vv;
    reduced_coords(ci, cj, k, hh, vv);
    double2 GF, Gh, Gv;
    double inv_hh;  // 1/hh, or 0 where the horizontal gradient is zeroed (hh <= 1e-6)
    wu_wave_term_and_derivs(hh, vv, GF, Gh, Gv, &inv_hh);
    const double a = kc[3] * inv_hh;
    w.I = make_double2(kc[1] * GF.x, kc[1] * GF.y);
    w.Gh = make_double2(a * Gh.x, a * Gh.y);
    w.Gz = make_double2(kc[2] * Gv.x, kc[2] * Gv.y);
  }
  if (WMODE & 2) {  // both_greens_and_gradient_greens(::ExactGuevelDelhommeau)
    double r, z;
    reduced_coords(ci, cj, k, r, z);
    const WaveTerms e = egd_wave_terms(r, z, k, egd_adaptive<false>(r, z, p.quad_rtol, p.quad_atol),
                                       egd_adaptive<true>(r, z, p.quad_rtol, p.quad_atol));
    w.I = zadd(w.I, e.I);
    w.Gh = zadd(w.Gh, e.Gh);
    w.Gz = zadd(w.Gz, e.Gz);
  }
}

// S and D entries (before adding the static part) from the wave terms: `sgn` = -1 gives the
// mirrored (j, i) orientation, `area` is the entry's source area and `an` its normal times
// that area.
__device__ __forceinline__ void wave_entry(const WaveTerms& w, double dx1, double dx2, double sgn, double area,
                                           const double an[3], double2& sv, double2& dv) {
  const double proj = sgn * (an[0] * dx1 + an[1] * dx2);
  sv = make_double2(w.I.x * area, w.I.y * area);
  dv = make_double2(fma(proj, w.Gh.x, an[2] * w.Gz.x), fma(proj, w.Gh.y, an[2] * w.Gz.y));
}

// writes the (i, j) entry and, for i != j, the mirrored (j, i) entry of one unordered pair;
// ani, anj: area-weighted normals of panels i and j (used as the entries' normals in the
// direct formulation with panel normals)
template <bool DIRECT>
__device__ __forceinline__ void store_pair(const AssemblyParams& p, const WaveTerms& w, int64_t i, int64_t j,
                                           const double ni[3], double ai, const double ani[3], const PanelRec& Pj,
                                           const double anj[3], double dx1, double dx2,
                                           const double* __restrict__ SR, const double* __restrict__ DR,
                                           double2* __restrict__ Sb, double2* __restrict__ Db, int wave_identity) {
  const int64_t n = p.n;
  const bool own = DIRECT && !p.has_fixed;  // entry normals are the source panels' own
  // (i, j): source j
  double an[3];
  if (own) {
    an[0] = anj[0]; an[1] = anj[1]; an[2] = anj[2];
  } else {
    double nv[3];
    pick_normal<DIRECT>(p, Pj, ni, nv);
    for (int c = 0; c < 3; ++c) an[c] = Pj.area * nv[c];
  }
  double2 sv, dv;
  wave_entry(w, dx1, dx2, 1.0, Pj.area, an, sv, dv);
  if (wave_identity && i == j) dv.x += identity_jump(p, ni);
  const int64_t idx = i + j * n;
  if (SR) {
    sv.x = SR[idx] + sv.x;
    dv.x = DR[idx] + dv.x;
  }
  Sb[idx] = sv;
  Db[idx] = dv;
  if (i == j) return;
  // (j, i): source i, field j -- normal of the source (direct) / field (indirect) swaps
  if (own) {
    an[0] = ani[0]; an[1] = ani[1]; an[2] = ani[2];
  } else {
    double nm[3];
    if (p.has_fixed) { nm[0] = p.fixed[0]; nm[1] = p.fixed[1]; nm[2] = p.fixed[2]; }
    else if (DIRECT) { nm[0] = ni[0]; nm[1] = ni[1]; nm[2] = ni[2]; }
    else { nm[0] = Pj.n[0]; nm[1] = Pj.n[1]; nm[2] = Pj.n[2]; }
    for (int c = 0; c < 3; ++c) an[c] = ai * nm[c];
  }
  double2 sm, dm;
  wave_entry(w, dx1, dx2, -1.0, ai, an, sm, dm);
  const int64_t mdx = j + i * n;
  if (SR) {
    sm.x = SR[mdx] + sm.x;
    dm.x = DR[mdx] + dm.x;
  }
  Sb[mdx] = sm;
  Db[mdx] = dm;
}

template <bool DIRECT, int WMODE>  // WMODE 1 = Wu only, 2 = exact Delhommeau, 3 = both
__global__ void __launch_bounds__(kRowsPerCta) wave_kernel(AssemblyParams p, const double* __restrict__ SR,
                                                           const double* __restrict__ DR,
                                                           const double* __restrict__ ks, double2* __restrict__ S,
                                                           double2* __restrict__ D, int64_t sstride,
                                                           int wave_identity) {
  __shared__ PanelRec sp[kColsPerCta];
  __shared__ double san[kColsPerCta][3];  // area-weighted normals of the staged panels
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kRowsPerCta;
  const int64_t j0 = blockIdx.y * (int64_t)kColsPerCta;
  if (i0 > j0 + kColsPerCta - 1) return;  // tile strictly below the diagonal
  const int64_t i = i0 + threadIdx.x;
  const double k = ks[blockIdx.z];
  const double kc[4] = {0.0, kMinusInv4Pi * k, kMinusInv4Pi * k * k, kMinusInv4Pi * k * k * k};
  double2* Sb = S + blockIdx.z * sstride;
  double2* Db = D + blockIdx.z * sstride;
  stage_panels(sp, p.P, j0, n);
  __syncthreads();
  const int jmax = (int)((n - j0) < kColsPerCta ? (n - j0) : kColsPerCta);
  for (int q = threadIdx.x; q < 3 * jmax; q += blockDim.x) san[q / 3][q % 3] = sp[q / 3].area * sp[q / 3].n[q % 3];
  __syncthreads();
  if (i >= n) return;
  double ci[3], ni[3], ani[3];
  for (int c = 0; c < 3; ++c) { ci[c] = __ldg(&p.P[i].c[c]); ni[c] = __ldg(&p.P[i].n[c]); }
  const double ai = __ldg(&p.P[i].area);
  for (int c = 0; c < 3; ++c) ani[c] = ai * ni[c];
  for (int jj = 0; jj < jmax; ++jj) {
    const int64_t j = j0 + jj;
    if (i > j) continue;
    const PanelRec& Pj = sp[jj];
    WaveTerms w;
    wave_terms<DIRECT, WMODE>(p, ci, Pj.c, k, kc, w);
    // (i, j) orientation: gradient w.r.t. the source (direct) or the field point (indirect)
    const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
    const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
    store_pair<DIRECT>(p, w, i, j, ni, ai, ani, Pj, san[jj], dx1, dx2, SR, DR, Sb, Db, wave_identity);
  }
}

// ---------------------------------------------------------------------------------------
// Surrogate wave assembly with the network's two 64 x 64 layers on the tensor cores.
//
// The CTA's 128 threads own 128 rows i; for each of its kColsPerCta columns j the 128 pairs
// (i, j) form one M = 128 batch: every thread evaluates its pair's Wu terms (FP32,
// mh_wu_f32.cuh: the network's own error is ~1e-3, so the base it corrects needs no FP64)
// and the first layer (2 -> 64, CUDA cores) into row i of a BF16 activation tile in shared memory,
// thread 0 issues tcgen05.mma (M = 128, N = 64, K = 64 in four K = 16 steps) against the
// BF16 weight tile, the FP32 result lands in tensor memory, and each thread reads its row
// back (tcgen05.ld), applies bias and tanh, and writes the next layer's activations; the
// last layer (64 -> 6, of which outputs 0 and 2 are used) runs on the CUDA cores.
// Shared memory: W2, W3 (64 x 64 BF16, 8 KB each), the activation tile (128 x 64 BF16,
// 16 KB), and the FP32 first/last-layer parameters.  Tensor memory: 64 columns.
constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 64;                  // TMEM columns (FP32 accumulator, N = 64)
constexpr uint32_t kTcWaitPolls = 1u << 24;       // bounded mbarrier wait
constexpr int kTcSmemW2 = 0, kTcSmemW3 = 8192, kTcSmemA = 16384, kTcSmemF = 32768;
constexpr int kTcSmemFloats = 128 + 64 + 64 + 64 + 128 + 2;  // W1, b1, b2, b3, W4 rows 0 and 2, b4[0], b4[2]
constexpr int kTcSmemBytes = kTcSmemF + 4 * kTcSmemFloats;

// FP32 wave terms of the surrogate path (as WaveTerms) and their S/D entries; the static
// Rankine part they are added to stays FP64
struct WaveTermsF {
  float2 I, gh[2], gz;
};

__device__ __forceinline__ void wu_to_wave_terms_f(float hh, float k, float dx1, float dx2, float2 GF, float2 Gh,
                                                   float2 Gv, WaveTermsF& w) {
  float dr1 = 0.0f, dr2 = 0.0f;
  if (fabsf(hh) > 1e-6f) {
    const float kk_hh = k * k / hh;
    dr1 = kk_hh * dx1;
    dr2 = kk_hh * dx2;
  }
  w.I = make_float2(k * GF.x, k * GF.y);
  w.gh[0] = make_float2(k * (dr1 * Gh.x), k * (dr1 * Gh.y));
  w.gh[1] = make_float2(k * (dr2 * Gh.x), k * (dr2 * Gh.y));
  w.gz = make_float2(k * (k * Gv.x), k * (k * Gv.y));
}

__device__ __forceinline__ void wave_entry_f(const WaveTermsF& w, float sgn, float area, const double nd[3],
                                             double2& sv, double2& dv) {
  const float nv[3] = {(float)nd[0], (float)nd[1], (float)nd[2]};
  const float c = (float)kMinusInv4Pi * area;
  const float g0x = sgn * w.gh[0].x, g0y = sgn * w.gh[0].y, g1x = sgn * w.gh[1].x, g1y = sgn * w.gh[1].y;
  sv = make_double2(c * w.I.x, c * w.I.y);
  dv = make_double2(c * fmaf(nv[0], g0x, fmaf(nv[1], g1x, nv[2] * w.gz.x)),
                    c * fmaf(nv[0], g0y, fmaf(nv[1], g1y, nv[2] * w.gz.y)));
}

// store_pair for FP32 wave terms
template <bool DIRECT>
__device__ __forceinline__ void store_pair_f(const AssemblyParams& p, const WaveTermsF& w, int64_t i, int64_t j,
                                             const double ni[3], double ai, const PanelRec& Pj,
                                             const double* __restrict__ SR, const double* __restrict__ DR,
                                             double2* __restrict__ Sb, double2* __restrict__ Db, int wave_identity) {
  const int64_t n = p.n;
  double nv[3];
  pick_normal<DIRECT>(p, Pj, ni, nv);
  double2 sv, dv;
  wave_entry_f(w, 1.0f, (float)Pj.area, nv, sv, dv);
  if (wave_identity && i == j) dv.x += identity_jump(p, ni);
  const int64_t idx = i + j * n;
  if (SR) {
    sv.x = SR[idx] + sv.x;
    dv.x = DR[idx] + dv.x;
  }
  Sb[idx] = sv;
  Db[idx] = dv;
  if (i == j) return;
  double nm[3];
  if (p.has_fixed) { nm[0] = p.fixed[0]; nm[1] = p.fixed[1]; nm[2] = p.fixed[2]; }
  else if (DIRECT) { nm[0] = ni[0]; nm[1] = ni[1]; nm[2] = ni[2]; }
  else { nm[0] = Pj.n[0]; nm[1] = Pj.n[1]; nm[2] = Pj.n[2]; }
  double2 sm, dm;
  wave_entry_f(w, -1.0f, (float)ai, nm, sm, dm);
  const int64_t mdx = j + i * n;
  if (SR) {
    sm.x = SR[mdx] + sm.x;
    dm.x = DR[mdx] + dm.x;
  }
  Sb[mdx] = sm;
  Db[mdx] = dm;
}

template <bool DIRECT>
__global__ void __launch_bounds__(kTcRows) wave_kernel_tc(AssemblyParams p, const double* __restrict__ SR,
                                                          const double* __restrict__ DR,
                                                          const double* __restrict__ ks, double2* __restrict__ S,
                                                          double2* __restrict__ D, int64_t sstride,
                                                          int wave_identity) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ PanelRec sp[kColsPerCta];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int64_t n = p.n;
  const int64_t i0 = blockIdx.x * (int64_t)kTcRows;
  const int64_t j0 = blockIdx.y * (int64_t)kColsPerCta;
  if (i0 > j0 + kColsPerCta - 1) return;  // tile strictly below the diagonal (whole CTA)
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t i = i0 + tid;
  const double k = ks[blockIdx.z];
  double2* Sb = S + blockIdx.z * sstride;
  double2* Db = D + blockIdx.z * sstride;
  unsigned char* W2s = tsm + kTcSmemW2;
  unsigned char* W3s = tsm + kTcSmemW3;
  unsigned char* As = tsm + kTcSmemA;
  float* F = reinterpret_cast<float*>(tsm + kTcSmemF);
  float* W1f = F;            // 64 x 2
  float* b1f = F + 128;
  float* b2f = F + 192;
  float* b3f = F + 256;
  float* W4f = F + 320;      // rows 0 and 2 of W4, 2 x 64
  float* b4f = F + 448;      // b4[0], b4[2]
  stage_panels(sp, p.P, j0, n);
  // weights: W2, W3 as BF16 in the canonical K-major layout (row = output, K = input)
  for (int q = tid; q < kMlpH * kMlpH; q += kTcRows) {
    const int r = q / kMlpH, c = q % kMlpH;
    *reinterpret_cast<__nv_bfloat16*>(W2s + tc::kmajor_offset(r, c, kMlpH)) = __float2bfloat16_rn(p.mlp[kMlpW2 + q]);
    *reinterpret_cast<__nv_bfloat16*>(W3s + tc::kmajor_offset(r, c, kMlpH)) = __float2bfloat16_rn(p.mlp[kMlpW3 + q]);
  }
  for (int q = tid; q < 128; q += kTcRows) W1f[q] = p.mlp[kMlpW1 + q];
  for (int q = tid; q < 64; q += kTcRows) {
    b1f[q] = p.mlp[kMlpB1 + q];
    b2f[q] = p.mlp[kMlpB2 + q];
    b3f[q] = p.mlp[kMlpB3 + q];
    W4f[q] = p.mlp[kMlpW4 + 0 * kMlpH + q];
    W4f[64 + q] = p.mlp[kMlpW4 + 2 * kMlpH + q];
  }
  if (tid == 0) {
    b4f[0] = p.mlp[kMlpB4 + 0];
    b4f[1] = p.mlp[kMlpB4 + 2];
    tc::mbar_init(&mbar, 1);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kTcCols);
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 TMEM lanes
  const uint32_t idesc = tc::idesc_bf16_f32(kTcRows, kMlpH);
  const uint32_t a_base = tc::smem_u32(As), w2_base = tc::smem_u32(W2s), w3_base = tc::smem_u32(W3s);
  const bool row_ok = i < n;
  double ci[3] = {0, 0, 0}, ni[3] = {0, 0, 1};
  double ai = 0.0;
  if (row_ok) {
    for (int c = 0; c < 3; ++c) { ci[c] = p.P[i].c[c]; ni[c] = p.P[i].n[c]; }
    ai = p.P[i].area;
  }
  uint32_t phase = 0;
  bool timed_out = false;
  const int jmax = (int)((n - j0) < kColsPerCta ? (n - j0) : kColsPerCta);
  const float kf = (float)k;
  for (int jj = 0; jj < jmax && !timed_out; ++jj) {
    const int64_t j = j0 + jj;
    const bool active = row_ok && i <= j;
    const PanelRec& Pj = sp[jj];
    float hh = 1.0f, vv = -1.0f;
    float2 GF = make_float2(0.0f, 0.0f), Gh = GF, Gv = GF;
    if (active) {
      // reduced coordinates (wu.jl:7-18): the differences of the FP64 centres, then FP32
      const float ex = (float)(ci[0] - Pj.c[0]), ey = (float)(ci[1] - Pj.c[1]);
      hh = kf * sqrtf(fmaf(ex, ex, ey * ey));
      vv = kf * (float)(ci[2] + Pj.c[2]);
      wu_wave_term_and_derivs_f32(hh, vv, GF, Gh, Gv);
    }
    // first layer (CUDA cores) -> BF16 activation row `tid`
    float u, v;
    mlp_inputs_f(fmaxf(hh, (float)kSurrRMin), fmaxf(vv, (float)kSurrZMin), u, v);
#pragma unroll 8
    for (int q = 0; q < kMlpH; ++q) {
      const float h = tanh_fast(fmaf(W1f[2 * q], u, fmaf(W1f[2 * q + 1], v, b1f[q])));
      *reinterpret_cast<__nv_bfloat16*>(As + tc::kmajor_offset(tid, q, kMlpH)) = __float2bfloat16_rn(h);
    }
    float y0 = b4f[0], y2 = b4f[1];
    for (int layer = 0; layer < 2 && !timed_out; ++layer) {
      // make the activation tile visible to the tensor cores, then one thread issues
      tc::fence_proxy_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t w_base = layer == 0 ? w2_base : w3_base;
#pragma unroll
        for (int kk = 0; kk < kMlpH / 16; ++kk) {
          const uint64_t ad = tc::smem_desc(a_base + kk * 256, 128, (kMlpH / 8) * 128);
          const uint64_t bd = tc::smem_desc(w_base + kk * 256, 128, (kMlpH / 8) * 128);
          tc::mma_bf16(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(&mbar);
      }
      const bool ok = tc::mbar_wait(&mbar, phase, kTcWaitPolls);
      phase ^= 1u;
      if (__syncthreads_or(!ok)) {
        timed_out = true;
        break;
      }
      tc::fence_after_sync();
      const float* bl = layer == 0 ? b2f : b3f;
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        float acc[32];
        tc::tmem_ld32(trow + half * 32, acc);
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int c = half * 32 + q;
          const float h = tanh_fast(acc[q] + bl[c]);
          if (layer == 0) {
            *reinterpret_cast<__nv_bfloat16*>(As + tc::kmajor_offset(tid, c, kMlpH)) = __float2bfloat16_rn(h);
          } else {
            y0 = fmaf(W4f[c], h, y0);
            y2 = fmaf(W4f[64 + c], h, y2);
          }
        }
      }
    }
    if (timed_out) break;
    // all TMEM reads of this batch are done before the next batch's MMA overwrites it
    tc::fence_before_sync();
    __syncthreads();
    if (!active) continue;
    const bool in_box = surrogate_in_box(hh, vv) && i != j;
    if (in_box) {
      float2 dG, dGr, dGz;
      surrogate_apply(y0, y2, hh, vv, dG, dGr, dGz);
      GF = make_float2(GF.x + dG.x, GF.y + dG.y);
      Gh = make_float2(Gh.x + dGr.x, Gh.y + dGr.y);
      Gv = make_float2(Gv.x + dGz.x, Gv.y + dGz.y);
    } else {
      // outside the training box, and the self pairs: queued for the exact kernel
      const unsigned long long slot = atomicAdd(p.fb_state, 1ull);
      if ((int64_t)slot < p.fb_cap) p.fb_list[slot] = make_int4((int)i, (int)j, (int)blockIdx.z, 0);
    }
    const float dx1 = (float)(DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0]);
    const float dx2 = (float)(DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1]);
    WaveTermsF w;
    wu_to_wave_terms_f(hh, kf, dx1, dx2, GF, Gh, Gv, w);
    store_pair_f<DIRECT>(p, w, i, j, ni, ai, Pj, SR, DR, Sb, Db, wave_identity);
  }
  if (timed_out) {
    // reported by the host as a timeout; let the MMAs in flight finish (bounded) before the
    // tensor memory is released
    if (tid == 0) atomicExch(p.fb_state + 2, 1ull);
    tc::mbar_wait(&mbar, phase ^ 1u, kTcWaitPolls);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTcCols);
}

// The exact Delhommeau terms of one unordered pair {i, j} at wavenumber k, computed by the
// whole warp (egd_warp); lane 0 writes both S/D entries.
template <bool DIRECT>
__device__ __forceinline__ void exact_pair_warp(const AssemblyParams& p, int64_t i, int64_t j, double k, double* sw,
                                                const double* __restrict__ SR, const double* __restrict__ DR,
                                                double2* __restrict__ Sb, double2* __restrict__ Db, int wave_identity) {
  const PanelRec& Pi = p.P[i];
  const PanelRec& Pj = p.P[j];
  const double ci[3] = {Pi.c[0], Pi.c[1], Pi.c[2]};
  double r, z;
  reduced_coords(ci, Pj.c, k, r, z);
  double2 GF, dGdr;
  if (r == 0.0) {
    // self pairs and vertically stacked centres: at r = 0 the integrand does not depend on
    // theta (zeta = z), so 4 times its integral over [0, pi/2] is 2 pi times its value; the
    // r-derivative is not needed (the horizontal gradient vanishes for r <= 1e-6)
    if ((threadIdx.x & 31) != 0) return;
    const double2 f = egd_integrand<false>(0.0, 0.0, z);
    GF = make_double2(2.0 * kPi * f.x, 2.0 * kPi * f.y);
    dGdr = make_double2(0.0, 0.0);
  } else {
    egd_warp(r, z, p.quad_rtol, p.quad_atol, sw, GF, dGdr);
    if ((threadIdx.x & 31) != 0) return;
  }
  // both_greens_and_gradient_greens + with_reduced_coordinates_derivative, as wave_terms<., 2>
  const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
  const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
  const WaveTerms w = egd_wave_terms(r, z, k, GF, dGdr);
  const double ni[3] = {Pi.n[0], Pi.n[1], Pi.n[2]};
  const double ani[3] = {Pi.area * ni[0], Pi.area * ni[1], Pi.area * ni[2]};
  const double anj[3] = {Pj.area * Pj.n[0], Pj.area * Pj.n[1], Pj.area * Pj.n[2]};
  store_pair<DIRECT>(p, w, i, j, ni, Pi.area, ani, Pj, anj, dx1, dx2, SR, DR, Sb, Db, wave_identity);
}

constexpr int kExactWarps = 4;  // warps per CTA of the warp-per-pair exact kernels

// Exact Delhommeau wave part: one warp per unordered pair {i <= j}, pairs in column-major
// upper-triangle order q = j (j + 1) / 2 + i, grid-strided; blockIdx.y = wavenumber.
template <bool DIRECT>
__global__ void __launch_bounds__(32 * kExactWarps) exact_wave_warp_kernel(AssemblyParams p,
                                                                            const double* __restrict__ SR,
                                                                            const double* __restrict__ DR,
                                                                            const double* __restrict__ ks,
                                                                            double2* __restrict__ S,
                                                                            double2* __restrict__ D, int64_t sstride,
                                                                            int wave_identity) {
  __shared__ double sw[kExactWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5;
  const int64_t npairs = p.n * (p.n + 1) / 2;
  const double k = ks[blockIdx.y];
  double2* Sb = S + blockIdx.y * sstride;
  double2* Db = D + blockIdx.y * sstride;
  for (int64_t q = blockIdx.x * (int64_t)kExactWarps + warp; q < npairs; q += (int64_t)gridDim.x * kExactWarps) {
    int64_t j = (int64_t)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > q) --j;
    while ((j + 1) * (j + 2) / 2 <= q) ++j;
    const int64_t i = q - j * (j + 1) / 2;
    exact_pair_warp<DIRECT>(p, i, j, k, sw[warp], SR, DR, Sb, Db, wave_identity);
  }
}

// Exact Delhommeau terms for the pairs the surrogate queued (one warp per pair).
template <bool DIRECT>
__global__ void __launch_bounds__(32 * kExactWarps) surrogate_fallback_kernel(AssemblyParams p,
                                                                               const double* __restrict__ SR,
                                                                               const double* __restrict__ DR,
                                                                               const double* __restrict__ ks,
                                                                               double2* __restrict__ S,
                                                                               double2* __restrict__ D,
                                                                               int64_t sstride, int wave_identity) {
  __shared__ double sw[kExactWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5;
  const unsigned long long queued = p.fb_state[0];
  if (blockIdx.x == 0 && threadIdx.x == 0 && (int64_t)queued > p.fb_cap) p.fb_state[1] = 1ull;  // sticky overflow
  const int64_t count = (int64_t)queued < p.fb_cap ? (int64_t)queued : p.fb_cap;
  for (int64_t q = blockIdx.x * (int64_t)kExactWarps + warp; q < count; q += (int64_t)gridDim.x * kExactWarps) {
    const int4 e = p.fb_list[q];
    exact_pair_warp<DIRECT>(p, e.x, e.y, ks[e.z], sw[warp], SR, DR, S + e.z * sstride, D + e.z * sstride,
                            wave_identity);
  }
}

__global__ void static_only_kernel(int64_t count, const double* __restrict__ SR, const double* __restrict__ DR,
                                   double2* __restrict__ S, double2* __restrict__ D) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= count) return;
  S[q] = make_double2(SR[q], 0.0);
  D[q] = make_double2(DR[q], 0.0);
}

__global__ void wu_points_kernel(int64_t m, const double* __restrict__ hh, const double* __restrict__ vv,
                                 double2* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  double2 a, b, c;
  wu_wave_term_and_derivs(hh[q], vv[q], a, b, c);
  out[3 * q] = a;
  out[3 * q + 1] = b;
  out[3 * q + 2] = c;
}

__global__ void fixpoint_points_kernel(int64_t m, const double* __restrict__ x, double* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  const double a = fabs(x[q]);
  out[4 * q] = fx::exp_nonpos(-a);
  out[4 * q + 1] = fx::log_pos(a);
  out[4 * q + 2] = fx::recip(a);
  out[4 * q + 3] = fx::sqrt_pos(a);
}

__global__ void bessel01_points_kernel(int64_t m, const double* __restrict__ x, double* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  double J0, J1, Y0, Y1;
  bessel01(x[q], J0, J1, Y0, Y1);
  const bool y_defined = x[q] >= 3.0;
  out[4 * q] = J0;
  out[4 * q + 1] = J1;
  out[4 * q + 2] = y_defined ? Y0 : __longlong_as_double(0x7FF8000000000000LL);
  out[4 * q + 3] = y_defined ? Y1 : __longlong_as_double(0x7FF8000000000000LL);
}

// one warp per point
__global__ void __launch_bounds__(32 * kExactWarps) exact_points_kernel(int64_t m, const double* __restrict__ r,
                                                                         const double* __restrict__ z, double rtol,
                                                                         double atol, double2* __restrict__ out) {
  __shared__ double sw[kExactWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5;
  const int64_t q = blockIdx.x * (int64_t)kExactWarps + warp;
  if (q >= m) return;  // warp-uniform
  double2 G, Gr;
  egd_warp(r[q], z[q], rtol, atol, sw[warp], G, Gr);
  if ((threadIdx.x & 31) == 0) {
    out[2 * q] = G;
    out[2 * q + 1] = Gr;
  }
}

// The exact path's check of a surrogate-assembled matrix (the learned term approximates
// exact_Guevel_Delhommeau.jl:15-46): one warp per sampled ordered pair (i, j), drawn from a
// counter-based SplitMix64 stream of (seed, matrix, sample), recomputes the pair's S and D
// entries with the exact term (the adaptive quadrature at the assembly's tolerance; the
// closed form at r = 0), adds the static part as the assembly does, and accumulates the
// squared differences to the assembled entries and the squared assembled entries per matrix:
// acc[2 b] += |dS|^2 + |dD|^2, acc[2 b + 1] += |S|^2 + |D|^2.
__device__ __forceinline__ uint64_t judge_mix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

template <bool DIRECT>
__global__ void __launch_bounds__(32 * kExactWarps) surrogate_judge_kernel(
    AssemblyParams p, const double* __restrict__ SR, const double* __restrict__ DR, const double* __restrict__ ks,
    const double2* __restrict__ S, const double2* __restrict__ D, int64_t sstride, int64_t n_samples, uint64_t seed,
    int64_t first_matrix, int wave_identity, double* __restrict__ acc) {
  __shared__ double sw[kExactWarps][8 * kGKWarpStack];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = blockIdx.x * (int64_t)kExactWarps + warp;
  const int b = blockIdx.y;
  if (q >= n_samples) return;  // warp-uniform
  const int64_t n = p.n;
  const uint64_t h = judge_mix(seed ^ judge_mix(((uint64_t)(first_matrix + b) << 32) ^ (uint64_t)q));
  const int64_t i = (int64_t)((h & 0xFFFFFFFFULL) % (uint64_t)n);
  const int64_t j = (int64_t)((h >> 32) % (uint64_t)n);
  const double k = ks[b];
  const PanelRec& Pi = p.P[i];
  const PanelRec& Pj = p.P[j];
  const double ci[3] = {Pi.c[0], Pi.c[1], Pi.c[2]};
  double r, z;
  reduced_coords(ci, Pj.c, k, r, z);
  double2 GF, dGdr;
  if (r == 0.0) {
    if (lane != 0) return;
    const double2 f = egd_integrand<false>(0.0, 0.0, z);
    GF = make_double2(2.0 * kPi * f.x, 2.0 * kPi * f.y);
    dGdr = make_double2(0.0, 0.0);
  } else {
    egd_warp(r, z, p.quad_rtol, p.quad_atol, sw[warp], GF, dGdr);
    if (lane != 0) return;
  }
  // the (i, j) entries as exact_pair_warp and store_pair form them
  const double dx1 = DIRECT ? Pj.c[0] - ci[0] : ci[0] - Pj.c[0];
  const double dx2 = DIRECT ? Pj.c[1] - ci[1] : ci[1] - Pj.c[1];
  const WaveTerms w = egd_wave_terms(r, z, k, GF, dGdr);
  const double ni[3] = {Pi.n[0], Pi.n[1], Pi.n[2]};
  double nv[3];
  pick_normal<DIRECT>(p, Pj, ni, nv);
  const double an[3] = {Pj.area * nv[0], Pj.area * nv[1], Pj.area * nv[2]};
  double2 sv, dv;
  wave_entry(w, dx1, dx2, 1.0, Pj.area, an, sv, dv);
  if (wave_identity && i == j) dv.x += identity_jump(p, ni);
  const int64_t idx = i + j * n;
  if (SR) {
    sv.x = SR[idx] + sv.x;
    dv.x = DR[idx] + dv.x;
  }
  const double2 sa = S[b * sstride + idx], da = D[b * sstride + idx];
  const double e2 = (sa.x - sv.x) * (sa.x - sv.x) + (sa.y - sv.y) * (sa.y - sv.y) + (da.x - dv.x) * (da.x - dv.x) +
                    (da.y - dv.y) * (da.y - dv.y);
  const double t2 = sa.x * sa.x + sa.y * sa.y + da.x * da.x + da.y * da.y;
  atomicAdd(acc + 2 * b, e2);
  atomicAdd(acc + 2 * b + 1, t2);
}

}  // namespace

void launch_panel_geometry(cudaStream_t st, LaunchCounter lc, int64_t n, const double* V, const double* C,
                           const double* N, const double* A, const double* R, PanelRec* out) {
  if (n <= 0) return;
  MH_LAUNCH(lc, st, "panel_geometry",
            panel_geometry_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, V, C, N, A, R, out));
}

cudaError_t load_panel_geometry_kernel() {
  cudaFuncAttributes attr;
  return cudaFuncGetAttributes(&attr, panel_geometry_kernel);
}

void launch_assemble_static(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, double* SR, double* DR) {
  if (p.n <= 0) return;
  dim3 grid((unsigned)((p.n + kRowsPerCta - 1) / kRowsPerCta), (unsigned)((p.n + kColsPerCta - 1) / kColsPerCta));
  const bool birk = (p.gfs & kDelhKinds) == 0;
  lc.pre(st);
  if (p.direct) {
    if (birk) static_kernel<true, true><<<grid, kRowsPerCta, 0, st>>>(p, SR, DR);
    else static_kernel<true, false><<<grid, kRowsPerCta, 0, st>>>(p, SR, DR);
  } else {
    if (birk) static_kernel<false, true><<<grid, kRowsPerCta, 0, st>>>(p, SR, DR);
    else static_kernel<false, false><<<grid, kRowsPerCta, 0, st>>>(p, SR, DR);
  }
  lc.post(st, "assemble_static");
}

void launch_assemble_wave(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* SR,
                          const double* DR, int nk, const double* ks_dev, double2* S, double2* D, int64_t sstride,
                          int wave_identity) {
  if (p.n <= 0 || nk <= 0) return;
  const uint32_t wv = p.gfs & (MH_GF_WU | MH_GF_EXACT_DELHOMMEAU | MH_GF_SURROGATE);
  if (!wv) {
    // static only: widen to complex for every requested wavenumber
    int64_t count = p.n * p.n;
    for (int b = 0; b < nk; ++b) {
      MH_LAUNCH(lc, st, "assemble_static_widen",
                static_only_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, SR, DR, S + b * sstride,
                                                                                     D + b * sstride));
    }
    return;
  }
  dim3 grid((unsigned)((p.n + kRowsPerCta - 1) / kRowsPerCta), (unsigned)((p.n + kColsPerCta - 1) / kColsPerCta),
            (unsigned)nk);
  if (wv & MH_GF_SURROGATE) {
    // Wu + learned correction; pairs outside the training box are queued and then
    // recomputed by the exact kernel (the caller validates that no other wave kind is set)
    lc.pre(st);
    cudaMemsetAsync(p.fb_state, 0, sizeof(unsigned long long), st);
    static_assert(kTcRows == kRowsPerCta, "tensor-core tile rows");
    if (p.direct) wave_kernel_tc<true><<<grid, kTcRows, kTcSmemBytes, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    else wave_kernel_tc<false><<<grid, kTcRows, kTcSmemBytes, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    lc.post(st, "assemble_wave_surrogate");
    lc.pre(st);
    const int fbg = 8 * 152;
    if (p.direct) surrogate_fallback_kernel<true><<<fbg, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    else surrogate_fallback_kernel<false><<<fbg, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    lc.post(st, "assemble_wave_fallback");
    return;
  }
  if (wv == MH_GF_EXACT_DELHOMMEAU) {
    // one warp per unordered pair; enough CTAs for several resident per SM
    const int64_t npairs = p.n * (p.n + 1) / 2;
    const int64_t want = (npairs + kExactWarps - 1) / kExactWarps;
    dim3 g((unsigned)std::min<int64_t>(want, 152 * 16), (unsigned)nk);
    lc.pre(st);
    if (p.direct) exact_wave_warp_kernel<true><<<g, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    else exact_wave_warp_kernel<false><<<g, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity);
    lc.post(st, "assemble_wave_exact");
    return;
  }
  const int mode = (wv == MH_GF_WU) ? 1 : (wv == MH_GF_EXACT_DELHOMMEAU ? 2 : 3);
  lc.pre(st);
#define MH_WAVE(DIR, MODE) wave_kernel<DIR, MODE><<<grid, kRowsPerCta, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, wave_identity)
  if (p.direct) {
    if (mode == 1) MH_WAVE(true, 1); else if (mode == 2) MH_WAVE(true, 2); else MH_WAVE(true, 3);
  } else {
    if (mode == 1) MH_WAVE(false, 1); else if (mode == 2) MH_WAVE(false, 2); else MH_WAVE(false, 3);
  }
#undef MH_WAVE
  lc.post(st, mode == 1 ? "assemble_wave_wu" : "assemble_wave_exact");
}

void launch_surrogate_judge(cudaStream_t st, LaunchCounter lc, const AssemblyParams& p, const double* SR,
                            const double* DR, int nk, const double* ks_dev, const double2* S, const double2* D,
                            int64_t sstride, int64_t n_samples, uint64_t seed, int64_t first_matrix,
                            int wave_identity, double* acc) {
  if (p.n <= 0 || nk <= 0 || n_samples <= 0) return;
  dim3 g((unsigned)((n_samples + kExactWarps - 1) / kExactWarps), (unsigned)nk);
  if (p.direct)
    MH_LAUNCH(lc, st, "surrogate_judge",
              surrogate_judge_kernel<true><<<g, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, n_samples,
                                                                         seed, first_matrix, wave_identity, acc));
  else
    MH_LAUNCH(lc, st, "surrogate_judge",
              surrogate_judge_kernel<false><<<g, 32 * kExactWarps, 0, st>>>(p, SR, DR, ks_dev, S, D, sstride, n_samples,
                                                                          seed, first_matrix, wave_identity, acc));
}

void launch_fixpoint_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* x, double* out) {
  MH_LAUNCH(lc, st, "fixpoint_points", fixpoint_points_kernel<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(m, x, out));
}

void launch_bessel01_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* x, double* out) {
  MH_LAUNCH(lc, st, "bessel_points", bessel01_points_kernel<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(m, x, out));
}

void launch_wu_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* hh, const double* vv, double2* out) {
  if (m <= 0) return;
  MH_LAUNCH(lc, st, "wu_points", wu_points_kernel<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(m, hh, vv, out));
}

void launch_exact_points(cudaStream_t st, LaunchCounter lc, int64_t m, const double* r, const double* z, double rtol,
                         double atol, double2* out) {
  if (m <= 0) return;
  MH_LAUNCH(lc, st, "exact_points",
            exact_points_kernel<<<(unsigned)((m + kExactWarps - 1) / kExactWarps), 32 * kExactWarps, 0, st>>>(
                m, r, z, rtol, atol, out));
}

}  // namespace mh
