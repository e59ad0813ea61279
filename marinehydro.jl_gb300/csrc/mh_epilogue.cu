// mh_epilogue.cu -- boundary conditions and force integration (O(N) per RHS).
//
// Right-hand sides (one column per radiating dof, then one per heading):
//   radiation  bc_i = -i omega (n_i . dof_i)                 waves.jl:183-199, 203-211
//   diffraction bc_i = -(v_airy(c_i) . n_i)                   waves.jl:266-282
// Forces: F = sum_i p_i * -(dof_i . n_i) * a_i with p = i rho omega phi
//   (solve.jl:47-55, waves.jl:154-178); Froude-Krylov with the Airy pressure
//   (waves.jl:259-264, 294-303).
// Lid panels (index >= n_hull, irregular-frequency removal): the hull boundary
//   conditions are padded with zeros there and only hull pressures enter the
//   forces (solve.jl:2-10 _pad_hull_bc, :47-55 pressure[hull_mask]).
#include <cuda_runtime.h>

#include "mh_internal.cuh"

namespace mh {

namespace {

__global__ void build_rhs_kernel(EpilogueGeom g, const double* __restrict__ omegas, double gacc, int n_rad,
                                 const int32_t* __restrict__ rad_idx, int n_beta, const double* __restrict__ betas,
                                 double2* __restrict__ B, int64_t bstride) {
  const int64_t n = g.n;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int col = blockIdx.y;
  const int w = blockIdx.z;
  if (i >= n) return;
  if (i >= g.n_hull) {
    B[w * bstride + col * n + i] = make_double2(0.0, 0.0);
    return;
  }
  const double omega = omegas[w];
  const double nx = g.N[3 * i], ny = g.N[3 * i + 1], nz = g.N[3 * i + 2];
  double2 v;
  if (col < n_rad) {
    const double* dof = g.dofs + (int64_t)rad_idx[col] * n * 3 + 3 * i;
    double disp = nx * dof[0] + ny * dof[1] + nz * dof[2];
    v = make_double2(0.0 * disp, -omega * disp);
  } else {
    const double beta = betas[col - n_rad];
    const double k = omega * omega / gacc;
    const double cx = g.C[3 * i], cy = g.C[3 * i + 1], cz = g.C[3 * i + 2];
    double sb, cb;
    sincos(beta, &sb, &cb);
    const double wbar = cx * cb + cy * sb;
    const double cih = exp(k * cz);
    double sw, cw;
    sincos(k * wbar, &sw, &cw);
    const double s = gacc * k / omega;
    // amp = s e^{i k wbar}; v = (amp cos b cih, amp sin b cih, -i amp cih)
    const double ar = s * cw, ai = s * sw;
    const double v1r = ar * cb * cih, v1i = ai * cb * cih;
    const double v2r = ar * sb * cih, v2i = ai * sb * cih;
    const double v3r = ai * cih, v3i = -ar * cih;
    v = make_double2(-(v1r * nx + v2r * ny + v3r * nz), -(v1i * nx + v2i * ny + v3i * nz));
  }
  B[w * bstride + col * n + i] = v;
}

// d/d omega of build_rhs_kernel's columns, with k = omega^2 / g (compute_wavenumber):
//   radiation   d bc / d omega = -i (n . dof)
//   diffraction the Airy amplitude g k / omega = omega, so
//               d bc / d omega = bc (1 / omega + (z + i wbar) 2 omega / g)
__global__ void build_drhs_kernel(EpilogueGeom g, const double* __restrict__ omegas, double gacc, int n_rad,
                                  const int32_t* __restrict__ rad_idx, int n_beta, const double* __restrict__ betas,
                                  double2* __restrict__ dB, int64_t bstride) {
  const int64_t n = g.n;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int col = blockIdx.y;
  const int w = blockIdx.z;
  if (i >= n) return;
  if (i >= g.n_hull) {
    dB[w * bstride + col * n + i] = make_double2(0.0, 0.0);
    return;
  }
  const double omega = omegas[w];
  const double nx = g.N[3 * i], ny = g.N[3 * i + 1], nz = g.N[3 * i + 2];
  double2 v;
  if (col < n_rad) {
    const double* dof = g.dofs + (int64_t)rad_idx[col] * n * 3 + 3 * i;
    double disp = nx * dof[0] + ny * dof[1] + nz * dof[2];
    v = make_double2(0.0 * disp, -disp);
  } else {
    const double beta = betas[col - n_rad];
    const double k = omega * omega / gacc;
    const double cx = g.C[3 * i], cy = g.C[3 * i + 1], cz = g.C[3 * i + 2];
    double sb, cb;
    sincos(beta, &sb, &cb);
    const double wbar = cx * cb + cy * sb;
    const double cih = exp(k * cz);
    double sw, cw;
    sincos(k * wbar, &sw, &cw);
    const double s = gacc * k / omega;
    const double ar = s * cw, ai = s * sw;
    const double v1r = ar * cb * cih, v1i = ai * cb * cih;
    const double v2r = ar * sb * cih, v2i = ai * sb * cih;
    const double v3r = ai * cih, v3i = -ar * cih;
    const double br = -(v1r * nx + v2r * ny + v3r * nz), bi = -(v1i * nx + v2i * ny + v3i * nz);
    const double dk = 2.0 * omega / gacc;
    const double fr = 1.0 / omega + cz * dk, fi = wbar * dk;
    v = make_double2(br * fr - bi * fi, br * fi + bi * fr);
  }
  dB[w * bstride + col * n + i] = v;
}

__global__ void zaxpy_kernel(int64_t count, double alpha, const double2* __restrict__ x, double2* __restrict__ y) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) {
    const double2 a = x[q], b = y[q];
    y[q] = make_double2(fma(alpha, a.x, b.x), fma(alpha, a.y, b.y));
  }
}

// One CTA per (influenced dof, rhs column, omega): deterministic tree reduction.
__global__ void __launch_bounds__(256) force_kernel(EpilogueGeom g, const double* __restrict__ omegas, double rho,
                                                    double gacc, int nrhs, const double2* __restrict__ Phi,
                                                    int64_t pstride, int n_inf, const int32_t* __restrict__ inf_idx,
                                                    int n_beta, const double* __restrict__ betas,
                                                    double2* __restrict__ F, double2* __restrict__ FK) {
  const int64_t n = g.n;
  const int64_t nh = g.n_hull;
  const int d = blockIdx.x;
  const int col = blockIdx.y;  // 0..nrhs-1 pressure columns, then n_beta Froude-Krylov columns
  const int w = blockIdx.z;
  const double omega = omegas[w];
  const double k = omega * omega / gacc;
  const double* dof = g.dofs + (int64_t)inf_idx[d] * n * 3;
  double sr = 0.0, si = 0.0;
  if (col < nrhs) {
    const double2* phi = Phi + w * pstride + (int64_t)col * n;
    const double s = rho * omega;
    for (int64_t i = threadIdx.x; i < nh; i += blockDim.x) {
      double disp = g.N[3 * i] * dof[3 * i] + g.N[3 * i + 1] * dof[3 * i + 1] + g.N[3 * i + 2] * dof[3 * i + 2];
      double2 p = make_double2(-s * phi[i].y, s * phi[i].x);
      double f = -disp * g.A[i];
      sr += p.x * f;
      si += p.y * f;
    }
  } else {
    const double beta = betas[col - nrhs];
    double sb, cb;
    sincos(beta, &sb, &cb);
    for (int64_t i = threadIdx.x; i < nh; i += blockDim.x) {
      double disp = g.N[3 * i] * dof[3 * i] + g.N[3 * i + 1] * dof[3 * i + 1] + g.N[3 * i + 2] * dof[3 * i + 2];
      const double cx = g.C[3 * i], cy = g.C[3 * i + 1], cz = g.C[3 * i + 2];
      const double wbar = cx * cb + cy * sb;
      double sw, cw;
      sincos(k * wbar, &sw, &cw);
      // phi_airy = -i g/omega e^{kz} e^{i k wbar};  p = i omega rho phi_airy = rho g e^{kz} e^{i k wbar}
      const double a = rho * gacc * exp(k * cz);
      double f = -disp * g.A[i];
      sr += (a * cw) * f;
      si += (a * sw) * f;
    }
  }
  __shared__ double rr[8], ri[8];
  for (int off = 16; off > 0; off >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, off);
    si += __shfl_down_sync(0xffffffffu, si, off);
  }
  if ((threadIdx.x & 31) == 0) { rr[threadIdx.x >> 5] = sr; ri[threadIdx.x >> 5] = si; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int q = 0; q < 8; ++q) { tr += rr[q]; ti += ri[q]; }
    if (col < nrhs) F[((int64_t)w * n_inf + d) * nrhs + col] = make_double2(tr, ti);
    else FK[((int64_t)w * n_inf + d) * n_beta + (col - nrhs)] = make_double2(tr, ti);
  }
}

__global__ void combine_kernel(int64_t count, const double* __restrict__ re, double2* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < count) out[q] = make_double2(re[q], 0.0);
}

}  // namespace

void launch_build_rhs(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                      double gacc, int n_rad, const int32_t* rad_idx_dev, int n_beta, const double* betas_dev,
                      double2* Bmat, int64_t bstride) {
  const int ncol = n_rad + n_beta;
  if (g.n <= 0 || ncol <= 0 || nw <= 0) return;
  dim3 grid((unsigned)((g.n + 127) / 128), (unsigned)ncol, (unsigned)nw);
  MH_LAUNCH(lc, st, "build_rhs",
            build_rhs_kernel<<<grid, 128, 0, st>>>(g, omegas_dev, gacc, n_rad, rad_idx_dev, n_beta, betas_dev, Bmat,
                                                   bstride));
}

void launch_build_drhs(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                       double gacc, int n_rad, const int32_t* rad_idx_dev, int n_beta, const double* betas_dev,
                       double2* dB, int64_t bstride) {
  const int ncol = n_rad + n_beta;
  if (g.n <= 0 || ncol <= 0 || nw <= 0) return;
  dim3 grid((unsigned)((g.n + 127) / 128), (unsigned)ncol, (unsigned)nw);
  MH_LAUNCH(lc, st, "build_drhs",
            build_drhs_kernel<<<grid, 128, 0, st>>>(g, omegas_dev, gacc, n_rad, rad_idx_dev, n_beta, betas_dev, dB,
                                                    bstride));
}

void launch_zaxpy(cudaStream_t st, LaunchCounter lc, int64_t count, double alpha, const double2* x, double2* y) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "zaxpy", zaxpy_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, alpha, x, y));
}

void launch_forces(cudaStream_t st, LaunchCounter lc, const EpilogueGeom& g, int nw, const double* omegas_dev,
                   double rho, double gacc, int nrhs, const double2* Phi, int64_t pstride, int n_inf,
                   const int32_t* inf_idx_dev, int n_beta, const double* betas_dev, double2* F, double2* FK) {
  if (g.n <= 0 || n_inf <= 0 || nw <= 0 || (nrhs + n_beta) <= 0) return;
  dim3 grid((unsigned)n_inf, (unsigned)(nrhs + n_beta), (unsigned)nw);
  MH_LAUNCH(lc, st, "forces",
            force_kernel<<<grid, 256, 0, st>>>(g, omegas_dev, rho, gacc, nrhs, Phi, pstride, n_inf, inf_idx_dev,
                                               n_beta, betas_dev, F, FK));
}

void launch_combine_real_to_complex(cudaStream_t st, LaunchCounter lc, int64_t count, const double* re,
                                    double2* out) {
  if (count <= 0) return;
  MH_LAUNCH(lc, st, "combine", combine_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, re, out));
}

}  // namespace mh
