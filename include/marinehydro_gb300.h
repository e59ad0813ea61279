/*
 * marinehydro_gb300.h -- C-ABI of libmarinehydro_cuda.so, the GB300 (sm_103a)
 * implementation of MarineHydro.jl's dense boundary-element hot path:
 * influence-matrix assembly (Birk / Delhommeau Rankine panel integrals and their
 * free-surface image, the Wu and exact Guevel-Delhommeau infinite-depth wave
 * Green functions) and the complex linear solve that turns S and D into added
 * mass, radiation damping and excitation forces.
 *
 * Every entry point names the reference (MarineHydro.jl) interface it replaces,
 * as file:line in the MarineHydro.jl tree.
 *
 * Conventions
 *   - All arithmetic on the plain path is FP64.
 *   - Complex numbers are interleaved (re, im) doubles, i.e. the memory layout of
 *     Julia's ComplexF64, C99 double _Complex and cuDoubleComplex.
 *   - Matrices are column-major (Julia's layout): entry (i, j) at [i + j*n].
 *   - A mesh is passed per panel ("gathered" vertices), so no face-index base
 *     (Julia 1-based vs Capytaine 0-based) crosses the ABI:
 *       vertices n x 4 x 3 (panel, corner, xyz), centers n x 3, normals n x 3,
 *       areas n, radii n  (meshes.jl:42-51, 255-277).
 *   - Buffers are owned by the caller.  `mem` says where they live:
 *     MH_MEM_HOST (pageable or pinned host memory; the library copies) or
 *     MH_MEM_DEVICE (device pointers on the context's device).
 *   - Calls are synchronous: on return, outputs are complete in the caller's
 *     buffers.  A context is not thread-safe; use one context per host thread.
 *   - Every function returns an mh_status; mh_last_error() describes the last
 *     failure on a context.  No C++ exception crosses the ABI.
 */
#ifndef MARINEHYDRO_GB300_H
#define MARINEHYDRO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MH_ABI_VERSION 2

typedef enum {
    MH_OK = 0,
    MH_ERR_ARG = 1,           /* bad argument (maps to ArgumentError / DimensionMismatch) */
    MH_ERR_UNSUPPORTED = 2,   /* unsupported combination (ArgumentError) */
    MH_ERR_SINGULAR = 3,      /* exactly zero pivot (LinearAlgebra.SingularException) */
    MH_ERR_CUDA = 4,          /* CUDA runtime error */
    MH_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
    MH_ERR_NOT_CONVERGED = 6, /* mixed-precision refinement did not converge */
    MH_ERR_NOMEM = 7          /* device allocation failed */
} mh_status;

/* Green-function selection: a bit set mirroring the reference's GF tuples
   (formulations.jl:5-37; green_functions/*.jl).  The default formulation
   (Rankine(), RankineReflected(), GFWu()) is MH_GF_DEFAULT_WU. */
#define MH_GF_RANKINE                        1u  /* Birk vectorized Rankine (rankine_vectorized.jl) */
#define MH_GF_RANKINE_REFLECTED              2u  /* its free-surface image (rankine_reflected.jl) */
#define MH_GF_RANKINE_REFLECTED_NEGATIVE     4u  /* minus the image (rankine_reflected_negative.jl) */
#define MH_GF_DELHOMMEAU_RANKINE             8u  /* Capytaine-style Rankine (rankine.jl) */
#define MH_GF_DELHOMMEAU_RANKINE_REFLECTED  16u  /* its image */
#define MH_GF_WU                            32u  /* GFWu (wu.jl) */
#define MH_GF_EXACT_DELHOMMEAU              64u  /* ExactGuevelDelhommeau (exact_Guevel_Delhommeau.jl) */
#define MH_GF_SURROGATE                    128u  /* learned approximation of ExactGuevelDelhommeau
                                                    (mh_surrogate_train / mh_surrogate_set); no
                                                    counterpart in the reference */
#define MH_GF_DEFAULT_WU  (MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_WU)
#define MH_GF_DEFAULT_EGD (MH_GF_RANKINE | MH_GF_RANKINE_REFLECTED | MH_GF_EXACT_DELHOMMEAU)

#define MH_MEM_HOST 0
#define MH_MEM_DEVICE 1

/* Linear-solve precision.  MH_PREC_FP64: LU, pivoting and substitution in FP64
   (the reference's arithmetic).  MH_PREC_MIXED: LU factors in FP32 with FP64
   partial pivoting decisions on FP32 data, then FP64 iterative refinement of
   every right-hand side to a backward error below 1e-14 (falls back to FP64 LU
   when refinement stalls).  MH_PREC_FP64_TC: the FP64 LU with its trailing
   update on the BF16 tensor cores by Ozaki splitting (each row / column scaled
   by a power of two, cut into eight 7-bit digits, digit products summed exactly
   in FP32 and recombined in 64-bit integers): FP64 results to within the
   rounding of the row and column scales; panel, pivoting and substitution as
   MH_PREC_FP64.  Accepted by every entry point that takes a precision. */
#define MH_PREC_FP64 0
#define MH_PREC_MIXED 1
#define MH_PREC_FP64_TC 2

typedef struct mh_context mh_context;
typedef struct mh_mesh mh_mesh;

/* ---- context ---------------------------------------------------------- */
int mh_abi_version(void);
/* Creates a context on CUDA device `device` with its own stream. */
int mh_create(int device, mh_context** out);
int mh_destroy(mh_context* ctx);
/* Text of the last error on this context ("" if none).  Never NULL. */
const char* mh_last_error(const mh_context* ctx);
/* The cudaStream_t the context launches on (as void*).  mh_set_stream(ctx, NULL)
   restores the context's own stream. */
int mh_get_stream(mh_context* ctx, void** stream);
int mh_set_stream(mh_context* ctx, void* stream);
int mh_synchronize(mh_context* ctx);
/* Number of kernels this context has launched since creation. */
int64_t mh_launch_count(const mh_context* ctx);
/* Device bytes currently held by the context's workspaces. */
int64_t mh_workspace_bytes(const mh_context* ctx);

/* ---- mesh --------------------------------------------------------------- */
/* Replaces StaticArraysMesh(...) + element(mesh, j) (meshes.jl:42-51, 255-277):
   uploads one body's panels and precomputes the per-panel Birk frame
   (birk_panel_geometry, rankine_vectorized.jl:129-137).  Host arrays holding a NaN or
   an infinity are rejected with MH_ERR_ARG. */
int mh_mesh_create(mh_context* ctx, int64_t n_panels, const double* vertices, const double* centers,
                   const double* normals, const double* areas, const double* radii, int mem, mh_mesh** out);
int mh_mesh_destroy(mh_mesh* mesh);
int64_t mh_mesh_panels(const mh_mesh* mesh);
/* Replaces the hull + lid mesh of irregular-frequency removal (solve.jl:20-28,
   `_mesh_including_lid`; bodies.jl:9-23 `lid_mesh`): the mesh holds the hull's
   n_hull panels first and the lid's panels after them (`fb.mesh + fb.lid_mesh`).
   Assembly covers all panels; in mh_hydrodynamic_coefficients and the batch the
   boundary conditions are zero on the lid (`_pad_hull_bc`, solve.jl:2-10) and
   only hull pressures enter the forces (`pressure[hull_mask]`, solve.jl:47-55).
   Every lid panel centre must lie below z = -1e-8 (at the free surface the wave
   terms are singular at the self pairs); n_hull = n_panels removes the lid.
   mh_hydro_gradient and mh_hydro_vjp reject meshes with a lid (MH_ERR_UNSUPPORTED). */
int mh_mesh_set_lid(mh_mesh* mesh, int64_t n_hull);

/* ---- assembly ----------------------------------------------------------- */
/* Replaces assemble_matrices(green_functions, mesh::StaticArraysMesh, k;
   direct, include_identity, all_normals) -> (S, D)   (matrix_assembly.jl:167-222,
   274-369, 70-88).  S, D: n x n complex, column-major.  fixed_normal: NULL or
   3 doubles (the reference's `all_normals`, e.g. [1,0,0] for forward speed).
   The wavenumber-independent Rankine part is cached on the mesh per
   (gfs, direct, include_identity, fixed_normal) and reused across wavenumbers. */
int mh_assemble_matrices(mh_context* ctx, mh_mesh* mesh, double wavenumber, uint32_t gfs, int direct,
                         int include_identity, const double* fixed_normal, double* S, double* D, int mem);

/* ---- dense complex solves ------------------------------------------------ */
/* Replaces linsolve(A, b) / _linearsolve / gpu_linsolve (matrix_assembly.jl:396-434):
   X = A \ B, A n x n, B and X n x nrhs complex.  X may alias B. */
int mh_linsolve(mh_context* ctx, int64_t n, int64_t nrhs, const double* A, const double* B, double* X,
                int precision, int mem);
/* Replaces solve(D, S, bc; direct) -> (phi, sources) (matrix_assembly.jl:436-449).
   direct: phi = D \ (S bc), `sources` untouched (may be NULL).
   indirect: sources = D \ bc (D is K), phi = S sources. */
int mh_solve(mh_context* ctx, int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc,
             int direct, double* phi, double* sources, int precision, int mem);
/* The adjoint solve of the IFT rule for _linearsolve / gpu_linsolve
   (ad_rules.jl:360-414): lambda = A^H \ ybar. */
int mh_linsolve_adjoint(mh_context* ctx, int64_t n, int64_t nrhs, const double* A, const double* Ybar,
                        double* Lambda, int precision, int mem);

/* Influence-matrix assembly that allocates no device memory.  No counterpart in
   the reference.  For callers that cannot call cudaMalloc: code running under a
   device-memory pool that already owns the GPU's memory (a Julia CUDA.jl session,
   a framework with its own caching allocator) or code that must not allocate once
   initialised.  Same result as mh_assemble_matrices for gfs made of
   MH_GF_RANKINE, MH_GF_RANKINE_REFLECTED, MH_GF_RANKINE_REFLECTED_NEGATIVE and
   MH_GF_WU (other kinds: MH_ERR_UNSUPPORTED).
     - vertices, centers, normals, areas, radii, S, D: DEVICE pointers on the
       current device, laid out as for mh_mesh_create / mh_assemble_matrices;
       fixed_normal: NULL or 3 doubles in host memory.
     - The per-panel scratch is a fixed file-scope device array of 8192 panel
       records (2 MiB) that every GPU loading the library keeps until exit:
       n_panels > 8192 is rejected with MH_ERR_ARG.  Calls share the array and it
       keeps the last call's contents (each call rewrites its own panels first);
       calls whose work overlaps on the GPU (other streams or host threads) race.
     - The first call in a CUDA context (per device, and again once the context
       has been replaced, e.g. after cudaDeviceReset) is the set-up: it looks up
       the array's device address and loads the module of every kernel this entry
       point launches.  Loading a module can allocate, so make that first call
       before any stream capture; under a pool that leaves no device memory free
       it can fail with MH_ERR_CUDA.
     - A CUDA error that earlier work left pending on the calling thread is
       returned as MH_ERR_CUDA before anything is launched, and left pending.
     - Stream-ordered: kernels are queued on `stream` (a cudaStream_t, NULL = the
       default stream) and the call returns without synchronizing; S and D are
       complete when the stream reaches that point.  No cudaMalloc, cudaFree or
       allocating library routine is called. */
int mh_assemble_matrices_noalloc(void* stream, int64_t n_panels, const double* vertices, const double* centers,
                                 const double* normals, const double* areas, const double* radii, double wavenumber,
                                 uint32_t gfs, int direct, int include_identity, const double* fixed_normal,
                                 double* S, double* D);

/* ---- hydrodynamic coefficients over a frequency sweep ------------------- */
/* Replaces hydrodynamic_coefficients(body, params, formulation)
   (problems_and_results.jl:464-495) with _hydro_one_frequency (:472-478) for a
   zero-forward-speed body: for every omega, S and D are assembled once and all
   radiation and diffraction right-hand sides are solved together.
     dofs:      n_dofs x n x 3 dof fields (bodies.jl:74-118), [d][i][xyz]
     rad_idx:   n_rad indices into dofs (radiating_dofs)
     inf_idx:   n_inf indices into dofs (influenced_dofs)
     betas:     n_beta wave directions (wave_directions)
   Outputs (column-major, like the reference's arrays with n_U = 1):
     added_mass, radiation_damping: n_inf x n_rad x n_omega doubles
     diffraction_force, froude_krylov_force, excitation_force:
                                    n_inf x n_omega x n_beta complex
   Any output may be NULL when its group is empty. */
int mh_hydrodynamic_coefficients(mh_context* ctx, mh_mesh* mesh, int64_t n_omega, const double* omegas,
                                 double rho, double g, uint32_t gfs, int direct, int64_t n_dofs,
                                 const double* dofs, int64_t n_rad, const int32_t* rad_idx, int64_t n_inf,
                                 const int32_t* inf_idx, int64_t n_beta, const double* betas, int precision,
                                 double* added_mass, double* radiation_damping, double* diffraction_force,
                                 double* froude_krylov_force, double* excitation_force, int mem);

/* Replaces ForwardDiff.derivative(ω -> hydrodynamic_coefficients(body, (wave_frequencies = ω, …)), ω)
   (test/outputs_differentiation.jl:39-150, solve_problem_differentiation.jl:89-110,
   diffraction_differentiation.jl:63-78): the coefficients of mh_hydrodynamic_coefficients
   (same arguments and layouts, FP64) and their derivatives with respect to ω, k = ω²/g
   included.  Forward mode on the device: dS/dk, dD/dk of the Wu term from one dual
   direction through the same fits, the boundary conditions' ω-derivatives, and
   dφ = D⁻¹(dS b + S db − dD φ) (direct; indirect: dσ = D⁻¹(db − dD σ), dφ = dS σ + S dσ)
   with the LU factors of D reused.  Green functions: the Rankine kinds and MH_GF_WU
   (others: MH_ERR_UNSUPPORTED).  Derivative outputs may be NULL. */
int mh_hydro_frequency_derivative(mh_context* ctx, mh_mesh* mesh, int64_t n_omega, const double* omegas,
                                  double rho, double g, uint32_t gfs, int direct, int64_t n_dofs,
                                  const double* dofs, int64_t n_rad, const int32_t* rad_idx, int64_t n_inf,
                                  const int32_t* inf_idx, int64_t n_beta, const double* betas,
                                  double* added_mass, double* radiation_damping, double* diffraction_force,
                                  double* froude_krylov_force, double* excitation_force, double* d_added_mass,
                                  double* d_radiation_damping, double* d_diffraction_force,
                                  double* d_froude_krylov_force, double* d_excitation_force, int mem);

/* Replaces a loop of hydrodynamic_coefficients over many bodies
   (problems_and_results.jl:464-495): body b is meshes[b] with n_omega[b]
   frequencies (omegas holds them concatenated in body order); every body has the
   same dof names, dofs[b] is its n_dofs x n_b x 3 field block.  Outputs are the
   per-body arrays of mh_hydrodynamic_coefficients concatenated along the
   frequency axis in body order (body b's block starts at the sum of the earlier
   bodies' n_omega).  The whole schedule -- every body's static and wave assembly,
   factorization, refinement, solves and forces -- is captured into ONE CUDA graph
   over n_streams streams (0 = 4), bodies placed longest-first on the least-loaded
   stream; the instantiated graph and its buffers are cached on the context and
   reused while the bodies, frequency counts and options are unchanged (omegas,
   betas and dof values may change between calls).  Mixed precision runs two
   refinement sweeps inside the graph and finishes any right-hand side that has
   not met the backward-error test on the host afterwards.  With MH_GF_SURROGATE
   each body keeps its own queue of pairs for the exact kernel inside the graph
   (the surrogate parameters are read when the graph runs, so mh_surrogate_set
   between calls takes effect). */
int mh_batch_hydrodynamic_coefficients(mh_context* ctx, int64_t n_bodies, mh_mesh* const* meshes,
                                       const int64_t* n_omega, const double* omegas, double rho, double g,
                                       uint32_t gfs, int direct, int64_t n_dofs, const double* const* dofs,
                                       int64_t n_rad, const int32_t* rad_idx, int64_t n_inf, const int32_t* inf_idx,
                                       int64_t n_beta, const double* betas, int precision, int n_streams,
                                       double* added_mass, double* radiation_damping, double* diffraction_force,
                                       double* froude_krylov_force, double* excitation_force, int mem);
/* Frees the cached batch graph and its device buffers. */
int mh_batch_release(mh_context* ctx);

/* ---- launch-shape table and autotuner ------------------------------------ */
/* No counterpart in the reference (its LAPACK / cuSOLVER LU picks its own blocking):
   the launch shapes of the batched LU that depend on the matrix order n.  Entry q
   covers n <= n_max[q] (ascending; the last entry covers every larger n) with four
   choices, each 1..8:
     choices[4q+0]  reserved (the FP64 tensor-core update, MH_PREC_FP64_TC, is a persistent
                    kernel over equal slices of its tiles; the value is kept and ignored)
     choices[4q+1]  128-column tiles per CTA of the BF16x3 FP32 update (MH_PREC_MIXED)
     choices[4q+2]  largest thread-block cluster of the FP64 LU panel
     choices[4q+3]  largest thread-block cluster of the FP32 LU panel
   n_entries = 0 restores the defaults (8, 4, 8, 8).  The table applies to every later
   factorization of the context, including the captured batch graph (a changed table
   re-captures it).  The shapes change only the schedule: each output entry is computed
   by the same arithmetic. */
int mh_tile_table_set(mh_context* ctx, int64_t n_entries, const int64_t* n_max, const int32_t* choices);
/* Copies the context's table out (*n_entries = its length; n_max, choices need capacity). */
int mh_tile_table_get(mh_context* ctx, int64_t capacity, int64_t* n_max, int32_t* choices, int64_t* n_entries);
/* The project's autotuner: for each order sizes[q] (ascending, 32..12000) times the
   batched factorization of `batch` random complex matrices in `precision` with every
   candidate launch shape -- panel cluster bound 8, 4, 2 and, for the BF16x3 update,
   1, 2, 4 or 8 column tiles per CTA -- (smallest of `reps` timed runs after a warm-up,
   CUDA events on the context's stream) and installs the fastest per order bucket
   (bounds at the geometric means of neighbouring sizes).  A shape replaces the default
   only when it is more than 2 % faster.  Fields of the other precisions keep the
   values the previous table gave for each size.  ms_best / ms_default (NULL or n_sizes
   doubles) receive the chosen and the default shape's times.  Allocates workspace. */
int mh_autotune(mh_context* ctx, int precision, int64_t n_sizes, const int64_t* sizes, int64_t batch, int reps,
                double* ms_best, double* ms_default);

/* ---- reverse-mode gradient (hand-written adjoint) ------------------------ */
/* Replaces a reverse-mode gradient through assemble_matrices -> _mulvec ->
   _linearsolve -> force integration: the rules of ad_rules.jl:300-414
   (_mulvec: dS = ybar bc^H, dbc = S^H ybar; _linearsolve: lambda = A^-H ybar,
   dA = -lambda y^H) and the Birk kernel rules (ad_rules.jl:79-294), applied
   to the objective
       J = sum_omega sum_h ( A_hh(omega) + B_hh(omega) ),  h over obj_idx
   (added mass plus radiation damping of the objective dofs, zero forward
   speed).  Each frequency reuses its LU factors for one adjoint solve; no N^2
   cotangent is stored: the pair derivatives are recomputed tile by tile and
   contracted with rank-n_obj weights, the frequency-independent Rankine part
   once with frequency-summed weights.
     gfs:       Birk Rankine kinds (MH_GF_RANKINE*) with MH_GF_WU or
                MH_GF_EXACT_DELHOMMEAU (not both).  The exact term's second
                derivatives come from its value and r-derivative at each pair
                (dG/dz = G + 2/d, exact_Guevel_Delhommeau.jl:52-59, and Laplace's
                equation in (r, z)); its quadrature runs once per pair and frequency
                at the context's tolerance, as in the primal
     direct:    1 DirectBEM (phi = D^-1 S bc), 0 IndirectBEM (sigma = K^-1 bc,
                phi = S sigma): solve(D, S, bc; direct), matrix_assembly.jl:436-449
     dofs:      n_dofs x n x 3 dof fields, held fixed
     obj_idx:   1..4 indices into dofs
     precision: MH_PREC_FP64, or MH_PREC_MIXED: FP32 factors with both the forward and
                the adjoint solve refined to the FP64 backward-error test (a frequency
                chunk that does not converge is redone with FP64 factors)
   Outputs (any may be NULL):
     J                   the objective
     grad_centers[n][3], grad_normals[n][3], grad_areas[n]: dJ w.r.t. the
                         panel fields passed to mh_mesh_create
     grad_vertices[n][12]: dJ w.r.t. the 4 corners (Birk near-field terms)
     grad_dofs[n_obj][n][3]: dJ w.r.t. the objective dof fields
   The caller chains these through its mesh and dof construction. */
int mh_hydro_gradient(mh_context* ctx, mh_mesh* mesh, int64_t n_omega, const double* omegas, double rho, double g,
                      uint32_t gfs, int direct, int64_t n_dofs, const double* dofs, int64_t n_obj, const int32_t* obj_idx,
                      int precision, double* J, double* grad_centers, double* grad_normals, double* grad_areas,
                      double* grad_vertices, double* grad_dofs, int mem);
/* The general pullback of the same sweep, what Zygote / Enzyme reverse mode returns for
   arbitrary cotangents of hydrodynamic_coefficients' arrays:
       J = sum over omega, influenced q, radiating r of
             added_mass_bar[q, r, w] A[q, r, w] + radiation_damping_bar[q, r, w] B[q, r, w]
         + sum over omega, influenced q, heading b of
             Re(excitation_force_bar[q, w, b]) Re Fe[q, w, b] + Im(…) Im Fe[q, w, b]
   (A, B cotangents n_inf x n_rad x n_omega doubles; excitation cotangents n_inf x n_omega x
   n_beta complex; column-major, the output layouts of mh_hydrodynamic_coefficients;
   1..64 dofs and headings each, n_rad or n_beta may be 0).  Fe = diffraction +
   Froude-Krylov, both differentiated (the Airy condition and pressure depend on the panel
   centres).  Same method, Green functions and precisions as mh_hydro_gradient, which is
   this call with identity cotangents on the objective dofs; per frequency one adjoint
   solve per radiating dof and heading.  grad_dofs is n_dofs x n x 3 (every dof field,
   zero for dofs outside rad_idx / inf_idx). */
int mh_hydro_vjp(mh_context* ctx, mh_mesh* mesh, int64_t n_omega, const double* omegas, double rho, double g,
                 uint32_t gfs, int direct, int64_t n_dofs, const double* dofs, int64_t n_rad, const int32_t* rad_idx,
                 int64_t n_inf, const int32_t* inf_idx, int64_t n_beta, const double* betas,
                 const double* added_mass_bar, const double* radiation_damping_bar, const double* excitation_force_bar,
                 int precision, double* J, double* grad_centers, double* grad_normals, double* grad_areas,
                 double* grad_vertices, double* grad_dofs, int mem);

/* The pullback of solve(D, S, bc; direct) (matrix_assembly.jl:436-449) through the
   _mulvec and _linearsolve rules (ad_rules.jl:300-414): given the cotangent phi_bar of
   the potential (and, indirect, sources_bar of the sources, may be NULL), returns the
   primal outputs and the cotangents of D, S and bc (complex, Julia's conventions:
   dS = ybar bc^H, lambda = A^-H ybar, dA = -lambda y^H, dbc = lambda):
     direct:   phi = D^-1 (S bc); lambda = D^-H phi_bar;
               D_bar = -lambda phi^H, S_bar = lambda bc^H, bc_bar = S^H lambda
     indirect: sources = K^-1 bc, phi = S sources (K = D);
               lambda = K^-H (S^H phi_bar + sources_bar);
               S_bar = phi_bar sources^H, D_bar = -lambda sources^H, bc_bar = lambda
   D, S, D_bar, S_bar: n x n complex column-major; bc, phi_bar, sources_bar, phi,
   sources, bc_bar: n x nrhs complex.  D_bar, S_bar, bc_bar may be NULL; `sources` is
   required for the indirect method.  FP64 precisions factor once and reuse the factors
   for the adjoint solve; MH_PREC_MIXED refines both solves to FP64 backward error. */
int mh_solve_pullback(mh_context* ctx, int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc,
                      int direct, const double* phi_bar, const double* sources_bar, int precision, double* phi,
                      double* sources, double* D_bar, double* S_bar, double* bc_bar, int mem);

/* ---- learned wave-term surrogate (no counterpart in the reference) --------- */
/* A 2 -> 64 -> 64 -> 64 -> 6 tanh network with BF16 weights and FP32 arithmetic that
   corrects the Wu fits (wu.jl:28-37) toward the exact Guevel-Delhommeau wave term
   (exact_Guevel_Delhommeau.jl:15-46).  Inputs u = log10(r)/3, v = z/25 + 1 in the
   reduced coordinates (r, z) = (k |x_h - xi_h|, k (z + zeta)); outputs (1 + d)^2 times
   the real and imaginary parts of G_exact - G_Wu, its r-derivative and its
   z-derivative, d = sqrt(r^2 + z^2).  Used inside r in [1e-3, 1e3], z in [-50, 0];
   assembly with MH_GF_SURROGATE recomputes every pair outside that box with the
   exact kernel.  Parameters are packed as W1[64][2], b1, W2[64][64], b2, W3[64][64],
   b3, W4[6][64], b4 (mh_surrogate_param_count() floats). */
int mh_surrogate_param_count(void);
/* Trains on the device: n_samples points drawn with `seed` (r log-uniform, z uniform
   in the box), targets from the exact kernel at the context's quadrature
   tolerances; Adam with cosine-decayed learning rate from lr, `epochs` passes in
   batches of `batch`, BF16-rounded forward weights.  Installs the result on the
   context and writes it to params_out (may be NULL).  report (may be NULL), 10
   doubles: final mean squared error; RMS and max relative error of G over held-out
   points for the surrogate, then for the Wu fits; max relative error of dG/dr,
   surrogate then Wu; seconds of sample generation; seconds of training; number of
   held-out points. */
int mh_surrogate_train(mh_context* ctx, int64_t n_samples, uint64_t seed, int epochs, int batch, double lr,
                       float* params_out, double* report);
/* Installs parameters (rounded to BF16) on the context. */
int mh_surrogate_set(mh_context* ctx, const float* params);
/* Surrogate GF, dGF/dr, dGF/dz at m points (3 complex per point, the layout of
   mh_wu_wave_terms); points outside the training box take the exact kernel. */
int mh_surrogate_wave_terms(mh_context* ctx, int64_t m, const double* r, const double* z, double* out, int mem);
/* Mean squared error of the network (parameters rounded to BF16) on m samples
   (inputs m x 2 as (u, v), targets m x 6) and its gradient with respect to the
   parameters, computed by the training kernels.  Host buffers, m <= 2^20. */
int mh_surrogate_loss_grad(mh_context* ctx, const float* params, int64_t m, const float* inputs, const float* targets,
                           float* grad, double* loss);

/* The exact path's check of surrogate results (no counterpart in the reference; the
   surrogate approximates exact_Guevel_Delhommeau.jl:15-46).  With n_samples > 0, every
   sweep (mh_hydrodynamic_coefficients) and batch that assembles with MH_GF_SURROGATE has
   each frequency's S and D checked against the exact term on n_samples ordered panel
   pairs drawn from `seed` (the adaptive quadrature at the context's tolerance): the
   estimate is the relative error sqrt(sum |S - S_exact|^2 + |D - D_exact|^2) /
   sqrt(sum |S|^2 + |D|^2) over the sampled entries.  A frequency whose estimate exceeds
   `tolerance` is solved with the exact term instead (the sweep assembles that matrix
   again before its factorization; the batch re-runs those frequency-solves after its
   graph).  n_samples = 0 turns the check off (the default). */
int mh_surrogate_set_judge(mh_context* ctx, int64_t n_samples, uint64_t seed, double tolerance);
/* The estimates (count doubles) and re-run flags (count int32, 1 = solved with the exact
   term) of the last judged sweep or batch, one per frequency-solve in output order (a
   batch: bodies in input order); count must equal that call's number of frequency-solves.
   Either output may be NULL. */
int mh_surrogate_judge_read(mh_context* ctx, int64_t count, double* estimates, int32_t* rerun);

/* ---- wave-term evaluators (kernel-level parity entry points) ------------- */
/* _wu_wave_term_and_derivs(hh, vv) (wu.jl:28-37) for m points: out 3 complex
   per point (GF, dGF/dhh, dGF/dvv), i.e. 6 doubles. */
int mh_wu_wave_terms(mh_context* ctx, int64_t m, const double* hh, const double* vv, double* out, int mem);
/* _dimless_wave_term and _d_dimless_wave_term_dr (exact_Guevel_Delhommeau.jl:15-46)
   for m points: out 2 complex per point; rtol/atol: adaptive Gauss-Kronrod
   tolerances (the reference's Integrals.jl call uses its defaults). */
int mh_exact_wave_terms(mh_context* ctx, int64_t m, const double* r, const double* z, double rtol, double atol,
                        double* out, int mem);
/* J0, J1, Y0, Y1 at m points x >= 0, as the Wu kernels evaluate them: out 4 doubles
   per point (Y0, Y1 are NaN below x = 3, where the Wu term does not use them).  The
   reference calls SpecialFunctions.jl besselj0/besselj1/bessely0/bessely1 at the same
   argument (wu.jl:203, 335, 396, 431). */
int mh_bessel01_points(mh_context* ctx, int64_t m, const double* x, double* out, int mem);
/* Tolerances used by assembly with MH_GF_EXACT_DELHOMMEAU (default 1e-12, 1e-14). */
int mh_set_quadrature_tolerance(mh_context* ctx, double rtol, double atol);

/* ---- diagnostics (no counterpart in the reference) ---------------------- */
/* exp(-|x|), log|x|, 1/|x| and sqrt|x| for each x as the Wu kernels evaluate them in 64-bit
   fixed point on the integer pipe: m x 4 values, `out` row-major (4 per point). */
int mh_fixpoint_points(mh_context* ctx, int64_t m, const double* x, double* out, int mem);
/* Per-kernel-group device timing with CUDA events on the launching stream.
   mh_profile_read fills up to `capacity` groups: names (32 chars each, NUL
   padded), total milliseconds and launch counts; *n_groups = groups recorded. */
int mh_profile_enable(mh_context* ctx, int enable);
int mh_profile_reset(mh_context* ctx);
int mh_profile_read(mh_context* ctx, int64_t capacity, char* names, double* total_ms, int64_t* launches,
                    int64_t* n_groups);
/* Measured FP64 / FP32 fused-multiply-add throughput of the device (TFLOP/s),
   the denominators of the FP64-bound kernels' roofline. */
int mh_probe_fma_peaks(mh_context* ctx, double* fp64_tflops, double* fp32_tflops);
/* No counterpart in the reference: runs the recovery path of the bounded completion
   waits of the tensor-core kernels on purpose.  One warp holds tensor memory, waits on
   an mbarrier that nothing arrives at for `polls` (1..2^20) polls, frees the tensor
   memory and returns; the call reports MH_ERR_TIMEOUT and the context stays usable. */
int mh_probe_wait_timeout(mh_context* ctx, uint32_t polls);

#ifdef __cplusplus
}
#endif
#endif /* MARINEHYDRO_GB300_H */
