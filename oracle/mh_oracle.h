/*
 * mh_oracle.h -- CPU FP64 restatement of MarineHydro.jl's dense-BEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA library
 * (libmarinehydro_cuda.so).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  No product
 * code path calls it.
 *
 * Every function names the reference file:line it restates (paths are relative
 * to the MarineHydro.jl source tree).  Parity is pinned by the known-answer
 * values in the reference's own tests (Birk 2021 tables, Capytaine Delhommeau
 * point values, Wu vs Delhommeau, reflected Rankine closed forms, Hulme 1982);
 * see tests/golden/.
 *
 * Conventions (same as the C-ABI of the product library):
 *   - complex numbers are interleaved (re, im) doubles;
 *   - matrices are column-major, entry (i, j) at [i + j*n];
 *   - a mesh is given per panel: vertices n x 4 x 3 (panel-major, corner,
 *     coordinate), centers n x 3, normals n x 3, areas n, radii n.
 */
#ifndef MH_ORACLE_H
#define MH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Green-function bit flags: the same values as MH_GF_* in the product header. */
#define OR_GF_RANKINE                         1u
#define OR_GF_RANKINE_REFLECTED               2u
#define OR_GF_RANKINE_REFLECTED_NEGATIVE      4u
#define OR_GF_DELHOMMEAU_RANKINE              8u
#define OR_GF_DELHOMMEAU_RANKINE_REFLECTED   16u
#define OR_GF_WU                             32u
#define OR_GF_EXACT_DELHOMMEAU               64u

/* ---- Birk (2021) panel kernels: green_functions/rankine_vectorized.jl ---- */
/* out: T[9] column-major (s, t, n columns), qgc[3], lc[8] = 4 local corners (x,y), area */
void or_birk_panel_geometry(const double* v12, double* T, double* qgc, double* lc, double* area);
double or_birk_velocity_potential(double x, double y, double z, const double* lc);
void or_birk_velocity_derivatives(double x, double y, double z, const double* lc, double* v);
void or_birk_velocity_hessian(double x, double y, double z, const double* lc, double* H /*3x3 col-major*/);
void or_birk_phi_and_velocity(double x, double y, double z, const double* lc, double* phi, double* v);
/* _vrankine_from_geom: phi (= integral of 1/r) and gradient w.r.t. source */
void or_vrankine_from_geom(const double* point, const double* source_point, double source_radius,
                           double source_area, const double* T, const double* qgc, const double* lc,
                           double* phi, double* grad);

/* ---- Delhommeau Rankine: green_functions/rankine.jl ---- */
double or_delhommeau_rankine_integral(const double* point, const double* v12, const double* center,
                                      const double* normal, double area, double radius);
void or_delhommeau_rankine_both(const double* point, const double* v12, const double* center,
                                const double* normal, double area, double radius, int wrt_first,
                                double* integral, double* grad);

/* ---- Wu wave term: green_functions/wu.jl ---- */
void or_wu_wave_term_and_derivs(double hh, double vv, double* GF /*2*/, double* dGF_dhh /*2*/,
                                double* dGF_dvv /*2*/);
double or_struve_h0(double x);
double or_struve_h1(double x);
/* _wu_sd: s (2) and d (2) for one pair, before the -1/4pi scale */
void or_wu_sd(const double* x, const double* xi, const double* n, double area2, double k,
              double dx1, double dx2, double* s, double* d);

/* ---- exact Guevel-Delhommeau: green_functions/exact_Guevel_Delhommeau.jl ---- */
void or_exp_e1(double zr, double zi, double* gr, double* gi);   /* e^z E1(z) */
void or_e1(double zr, double zi, double* er, double* ei);       /* E1(z) */
void or_egd_dimless(double r, double z, double rtol, double atol, double* G /*2*/);
void or_egd_dimless_dr(double r, double z, double rtol, double atol, double* dG /*2*/);
void or_egd_set_tolerance(double rtol, double atol);

/* ---- point Green functions (greens / gradient_greens) for KAT tests ---- */
/* kind: one OR_GF_* flag; out g (2), grad (6 = 3 complex) */
void or_point_greens(unsigned kind, const double* c1, const double* c2, double k, int wrt_first,
                     double* g, double* grad);
/* panel integrals for one pair (element_1 = field center; element_2 = panel j) */
void or_pair_integrals(unsigned kind, const double* c1, const double* v12, const double* c2,
                       const double* n2, double a2, double r2, double k, int wrt_first,
                       double* integral /*2*/, double* grad /*6*/);

/* ---- assembly: matrix_assembly.jl:164-369 ---- */
/* S, D: n x n complex column-major (2*n*n doubles).  fixed_normal may be NULL.
   nthreads <= 0 uses all OpenMP threads (ignored in a build without OpenMP). */
int or_assemble(int64_t n, const double* vertices, const double* centers, const double* normals,
                const double* areas, const double* radii, double k, unsigned gfs, int direct,
                int include_identity, const double* fixed_normal, double* S, double* D, int nthreads);

/* ---- dense complex LU solve (LAPACK zgetrf/zgetrs semantics) ---- */
/* A n x n complex col-major (overwritten), B n x nrhs complex (overwritten by X). returns info */
int or_lu_solve(int64_t n, int64_t nrhs, double* A, double* B);
/* matrix_assembly.jl:436-449 solve(D, S, bc; direct) */
int or_solve(int64_t n, int64_t nrhs, const double* D, const double* S, const double* bc, int direct,
             double* phi, double* sources);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
