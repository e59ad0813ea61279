"""CPU FP64 oracle for the MarineHydro.jl dense-BEM hot path (TEST INFRASTRUCTURE).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` import it.  The product library (``libmarinehydro_cuda.so``)
neither links nor calls anything here.

It wraps ``mh_oracle.c`` (a C restatement of the reference's Green functions,
assembly and LU solve) through ctypes and adds the O(N) pre/post-processing of
the reference in numpy:

* boundary conditions: ``radiation_bc`` (waves.jl:183-199, 201-211) and the Airy
  diffraction condition ``_airy_bc`` (waves.jl:266-282);
* pressure and force integration: ``_integrate_dof_pressure`` (waves.jl:170-178),
  ``_airy_pressure`` (waves.jl:259-264, 301-303);
* coefficient packing of ``hydrodynamic_coefficients``
  (problems_and_results.jl:207-219, 291-380, 464-495).

Parity of this oracle with the reference is pinned by the known-answer values in
the reference's own tests, extracted into ``tests/golden/reference_kats.json``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmh_oracle.so")

GF_RANKINE = 1
GF_RANKINE_REFLECTED = 2
GF_RANKINE_REFLECTED_NEGATIVE = 4
GF_DELHOMMEAU_RANKINE = 8
GF_DELHOMMEAU_RANKINE_REFLECTED = 16
GF_WU = 32
GF_EXACT_DELHOMMEAU = 64
DEFAULT_WU = GF_RANKINE | GF_RANKINE_REFLECTED | GF_WU
DEFAULT_EGD = GF_RANKINE | GF_RANKINE_REFLECTED | GF_EXACT_DELHOMMEAU

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile mh_oracle.c into oracle/_build/libmh_oracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "mh_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mh_oracle.h"))
    ):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [
        "gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas",
        src, "-o", tmp, "-lm",
    ]
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            D = ctypes.c_double
            P = ctypes.POINTER(ctypes.c_double)
            i64 = ctypes.c_int64
            L.or_birk_panel_geometry.argtypes = [P, P, P, P, P]
            L.or_birk_velocity_potential.argtypes = [D, D, D, P]
            L.or_birk_velocity_potential.restype = D
            L.or_birk_velocity_derivatives.argtypes = [D, D, D, P, P]
            L.or_birk_velocity_hessian.argtypes = [D, D, D, P, P]
            L.or_birk_phi_and_velocity.argtypes = [D, D, D, P, P, P]
            L.or_vrankine_from_geom.argtypes = [P, P, D, D, P, P, P, P, P]
            L.or_wu_wave_term_and_derivs.argtypes = [D, D, P, P, P]
            L.or_struve_h0.argtypes = [D]
            L.or_struve_h0.restype = D
            L.or_struve_h1.argtypes = [D]
            L.or_struve_h1.restype = D
            L.or_exp_e1.argtypes = [D, D, P, P]
            L.or_e1.argtypes = [D, D, P, P]
            L.or_egd_dimless.argtypes = [D, D, D, D, P]
            L.or_egd_dimless_dr.argtypes = [D, D, D, D, P]
            L.or_egd_set_tolerance.argtypes = [D, D]
            L.or_point_greens.argtypes = [ctypes.c_uint, P, P, D, ctypes.c_int, P, P]
            L.or_pair_integrals.argtypes = [ctypes.c_uint, P, P, P, P, D, D, D, ctypes.c_int, P, P]
            L.or_assemble.argtypes = [i64, P, P, P, P, P, D, ctypes.c_uint, ctypes.c_int, ctypes.c_int, P, P, P,
                                      ctypes.c_int]
            L.or_assemble.restype = ctypes.c_int
            L.or_lu_solve.argtypes = [i64, i64, P, P]
            L.or_lu_solve.restype = ctypes.c_int
            L.or_solve.argtypes = [i64, i64, P, P, P, ctypes.c_int, P, P]
            L.or_solve.restype = ctypes.c_int
            L.or_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


# --------------------------------------------------------------------------
# kernel-level wrappers (known-answer tests)
# --------------------------------------------------------------------------
def birk_panel_geometry(corners):
    """birk_panel_geometry (rankine_vectorized.jl:129-137) -> T (3x3), qgc, local corners (4x2), area."""
    v = _f64(corners, (12,))
    T = np.zeros(9)
    q = np.zeros(3)
    lc = np.zeros(8)
    a = np.zeros(1)
    lib().or_birk_panel_geometry(_p(v), _p(T), _p(q), _p(lc), _p(a))
    return T.reshape(3, 3).T.copy(), q, lc.reshape(4, 2), float(a[0])


def birk_velocity_potential(x, y, z, lc):
    lc = _f64(lc, (8,))
    return lib().or_birk_velocity_potential(x, y, z, _p(lc))


def birk_velocity_derivatives(x, y, z, lc):
    lc = _f64(lc, (8,))
    v = np.zeros(3)
    lib().or_birk_velocity_derivatives(x, y, z, _p(lc), _p(v))
    return v


def birk_velocity_hessian(x, y, z, lc):
    lc = _f64(lc, (8,))
    H = np.zeros(9)
    lib().or_birk_velocity_hessian(x, y, z, _p(lc), _p(H))
    return H.reshape(3, 3).T.copy()


def birk_phi_and_velocity(x, y, z, lc):
    lc = _f64(lc, (8,))
    phi = np.zeros(1)
    v = np.zeros(3)
    lib().or_birk_phi_and_velocity(x, y, z, _p(lc), _p(phi), _p(v))
    return float(phi[0]), v


def wu_wave_term_and_derivs(hh, vv):
    g = np.zeros(2)
    gh = np.zeros(2)
    gv = np.zeros(2)
    lib().or_wu_wave_term_and_derivs(float(hh), float(vv), _p(g), _p(gh), _p(gv))
    return complex(*g), complex(*gh), complex(*gv)


def exp_e1(z):
    gr = np.zeros(1)
    gi = np.zeros(1)
    lib().or_exp_e1(z.real, z.imag, _p(gr), _p(gi))
    return complex(gr[0], gi[0])


def e1(z):
    er = np.zeros(1)
    ei = np.zeros(1)
    lib().or_e1(z.real, z.imag, _p(er), _p(ei))
    return complex(er[0], ei[0])


def egd_dimless(r, z, rtol=1e-13, atol=1e-15):
    g = np.zeros(2)
    lib().or_egd_dimless(float(r), float(z), rtol, atol, _p(g))
    return complex(*g)


def egd_dimless_dr(r, z, rtol=1e-13, atol=1e-15):
    g = np.zeros(2)
    lib().or_egd_dimless_dr(float(r), float(z), rtol, atol, _p(g))
    return complex(*g)


def set_egd_tolerance(rtol=1e-13, atol=1e-15):
    lib().or_egd_set_tolerance(rtol, atol)


def point_greens(kind, c1, c2, k=1.0, wrt_first=False):
    c1 = _f64(c1, (3,))
    c2 = _f64(c2, (3,))
    g = np.zeros(2)
    gr = np.zeros(6)
    lib().or_point_greens(kind, _p(c1), _p(c2), float(k), int(bool(wrt_first)), _p(g), _p(gr))
    return complex(*g), gr[0::2] + 1j * gr[1::2]


def pair_integrals(kind, c1, vertices2, c2, n2, a2, r2, k=1.0, wrt_first=False):
    c1 = _f64(c1, (3,))
    v = _f64(vertices2, (12,))
    c2 = _f64(c2, (3,))
    n2 = _f64(n2, (3,))
    i2 = np.zeros(2)
    g = np.zeros(6)
    lib().or_pair_integrals(kind, _p(c1), _p(v), _p(c2), _p(n2), float(a2), float(r2), float(k),
                            int(bool(wrt_first)), _p(i2), _p(g))
    return complex(*i2), g[0::2] + 1j * g[1::2]


# --------------------------------------------------------------------------
# assembly and dense solve
# --------------------------------------------------------------------------
def assemble_matrices(mesh, k, gfs=DEFAULT_WU, direct=True, include_identity=True, fixed_normal=None,
                      nthreads=0):
    """assemble_matrices(gfs, mesh::StaticArraysMesh, k; direct, include_identity, all_normals)."""
    n = int(mesh.nfaces)
    V = _f64(mesh.panel_vertices, (n, 4, 3))
    C = _f64(mesh.centers, (n, 3))
    N = _f64(mesh.normals, (n, 3))
    A = _f64(mesh.areas, (n,))
    R = _f64(mesh.radii, (n,))
    S = np.zeros((n, n), dtype=np.complex128, order="F")
    D = np.zeros((n, n), dtype=np.complex128, order="F")
    fx = None
    if fixed_normal is not None:
        fx = _f64(fixed_normal, (3,))
    rc = lib().or_assemble(n, _p(V), _p(C), _p(N), _p(A), _p(R), float(k), int(gfs), int(bool(direct)),
                           int(bool(include_identity)), _p(fx) if fx is not None else None,
                           S.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                           D.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(nthreads))
    assert rc == 0
    return S, D


def lu_solve(A, B):
    """LU with partial pivoting (LAPACK zgetrf/zgetrs semantics), the oracle's own C loop."""
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    B = np.array(B, dtype=np.complex128, copy=True)
    vec = B.ndim == 1
    B = np.asfortranarray(B.reshape(A.shape[0], -1))
    n, nrhs = B.shape
    info = lib().or_lu_solve(n, nrhs, A.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             B.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if info:
        raise np.linalg.LinAlgError(f"singular matrix: zero pivot at column {info}")
    return B[:, 0].copy() if vec else B


def linsolve(A, B, lapack=False):
    """linsolve(A, b) (matrix_assembly.jl:396-416): the C LU, or LAPACK zgesv via numpy."""
    if lapack:
        return np.linalg.solve(A, B)
    return lu_solve(A, B)


def solve(D, S, bc, direct=True, lapack=False):
    """solve(D, S, bc; direct) (matrix_assembly.jl:436-449) -> (phi, sources)."""
    b = np.asarray(bc, dtype=np.complex128)
    if direct:
        return linsolve(D, S @ b, lapack), None
    src = linsolve(D, b, lapack)
    return S @ src, src


def solve_pullback(D, S, bc, phi_bar, direct=True, sources_bar=None, lapack=False):
    """Reverse-mode pullback of solve(D, S, bc; direct) (matrix_assembly.jl:436-449) by the
    reference's rules: _mulvec y = S bc -> S_bar = ybar bc', bc_bar = S' ybar
    (ad_rules.jl:300-312) and _linearsolve y = A \\ b -> lambda = A' \\ ybar,
    A_bar = -lambda y', b_bar = lambda (ad_rules.jl:360-371); ' is the adjoint.
    Returns (phi, sources, D_bar, S_bar, bc_bar)."""
    D = np.asarray(D, dtype=np.complex128)
    S = np.asarray(S, dtype=np.complex128)
    b = np.asarray(bc, dtype=np.complex128)
    pb = np.asarray(phi_bar, dtype=np.complex128)
    outer = lambda u, v: (u.reshape(len(u), -1) @ v.reshape(len(v), -1).conj().T)
    if direct:
        y = S @ b
        phi = linsolve(D, y, lapack)
        lam = linsolve(D.conj().T, pb, lapack)    # _linearsolve pullback
        D_bar = -outer(lam, phi)
        S_bar = outer(lam, b)                      # _mulvec pullback with ybar = lam
        bc_bar = S.conj().T @ lam
        return phi, None, D_bar, S_bar, bc_bar
    src = linsolve(D, b, lapack)
    phi = S @ src
    S_bar = outer(pb, src)                         # _mulvec pullback
    src_bar = S.conj().T @ pb
    if sources_bar is not None:
        src_bar = src_bar + np.asarray(sources_bar, dtype=np.complex128)
    lam = linsolve(D.conj().T, src_bar, lapack)   # _linearsolve pullback
    D_bar = -outer(lam, src)
    return phi, src, D_bar, S_bar, lam


# --------------------------------------------------------------------------
# O(N) physics around the solve (numpy)
# --------------------------------------------------------------------------
def radiation_bc(normals, dof_field, omega):
    """radiation_bc(problem) (waves.jl:183-199): -i omega (n . dof) per panel."""
    disp = np.einsum("ij,ij->i", np.asarray(normals), np.asarray(dof_field))
    return (-1j * omega) * disp


def airy_bc(centers, normals, omega, k, beta, g):
    """_airy_bc (waves.jl:266-282): -(v_airy . n) with v from _airy_vel."""
    c = np.asarray(centers)
    wbar = c[:, 0] * np.cos(beta) + c[:, 1] * np.sin(beta)
    cih = np.exp(k * c[:, 2])
    amp = g * k / omega * np.exp(1j * k * wbar)
    v1 = amp * np.cos(beta) * cih
    v2 = amp * np.sin(beta) * cih
    v3 = -1j * amp * cih
    n = np.asarray(normals)
    return -(v1 * n[:, 0] + v2 * n[:, 1] + v3 * n[:, 2])


def airy_pressure(centers, omega, k, beta, rho, g):
    """_airy_pressure (waves.jl:301-303) with _airy_phi (waves.jl:259-264)."""
    c = np.asarray(centers)
    wbar = c[:, 0] * np.cos(beta) + c[:, 1] * np.sin(beta)
    phi = -1j * g / omega * np.exp(k * c[:, 2]) * np.exp(1j * k * wbar)
    return 1j * omega * rho * phi


def integrate_dof_pressure(normals, areas, dof_field, pressure):
    """_integrate_dof_pressure (waves.jl:170-178): sum p_i * -(dof_i . n_i) * a_i."""
    disp = np.einsum("ij,ij->i", np.asarray(normals), np.asarray(dof_field))
    return np.sum(np.asarray(pressure) * -disp * np.asarray(areas))


def pad_hull_bc(bc_on_hull, n_total):
    """_pad_hull_bc (solve.jl:2-10): hull values first, zeros on the lid panels after them."""
    v = np.asarray(bc_on_hull, dtype=np.complex128)
    out = np.zeros((n_total,) + v.shape[1:], dtype=np.complex128)
    out[:v.shape[0]] = v
    return out


def hydro_one_frequency(mesh, dofs, omega, rho=1000.0, g=9.81, gfs=DEFAULT_WU, direct=True,
                        radiating=None, influenced=None, betas=(), lapack=False, nthreads=0, lid_mesh=None):
    """_hydro_one_frequency (problems_and_results.jl:472-478) for one omega.

    ``dofs`` maps dof name -> (n, 3) field on the hull.  Returns (A [n_inf, n_rad], B,
    Fd [n_inf, n_beta], Fk, Fe) with the reference's per-problem arithmetic; S and D are
    assembled once (the reference re-assembles them for each problem: identical matrices).
    With ``lid_mesh`` the matrices cover hull + lid (``_mesh_including_lid``, solve.jl:22-28),
    the boundary conditions are padded with zeros on the lid (solve.jl:2-10) and only the
    hull pressures are integrated (solve.jl:47-55).
    """
    names = list(dofs.keys())
    radiating = names if radiating is None else list(radiating)
    influenced = names if influenced is None else list(influenced)
    k = omega * omega / g
    nh = mesh.nfaces
    full = mesh if lid_mesh is None else _combine(mesh, lid_mesh)
    S, D = assemble_matrices(full, k, gfs=gfs, direct=direct, nthreads=nthreads)
    rhs = [radiation_bc(mesh.normals, dofs[d], omega) for d in radiating]
    rhs += [airy_bc(mesh.centers, mesh.normals, omega, k, b, g) for b in betas]
    if not rhs:
        return (np.zeros((len(influenced), 0)),) * 2 + (np.zeros((len(influenced), 0), complex),) * 3
    B = pad_hull_bc(np.stack(rhs, axis=1), full.nfaces)
    phi, _ = solve(D, S, B, direct=direct, lapack=lapack)
    p = (1j * rho * omega * phi)[:nh]
    F = np.array([[integrate_dof_pressure(mesh.normals, mesh.areas, dofs[d], p[:, c]) for c in range(B.shape[1])]
                  for d in influenced])
    nr = len(radiating)
    Fr = F[:, :nr]
    A = Fr.real / omega ** 2
    Bd = Fr.imag / omega
    Fd = F[:, nr:]
    Fk = np.array([[integrate_dof_pressure(mesh.normals, mesh.areas, dofs[d],
                                           airy_pressure(mesh.centers, omega, k, b, rho, g)) for b in betas]
                   for d in influenced]).reshape(len(influenced), len(betas))
    return A, Bd, Fd, Fk, Fd + Fk


def encountered_values(omega, beta, forward_speed, g=9.81):
    """compute_encountered_values (waves.jl:136-151) -> (omega_e, k_e, beta_e)."""
    k = omega * omega / g
    if forward_speed == 0:
        return omega, k, beta
    doppler = omega - k * forward_speed * np.cos(beta)
    oe = abs(doppler)
    return oe, oe * oe / g, (beta if doppler >= 0 else beta + np.pi)


def gradient_of_motion(n, dof_name):
    """evaluate_gradient_of_motion (bodies.jl:54-66): d(dof)/dx for rigid dofs."""
    d = np.zeros((n, 3))
    if dof_name == "Pitch":
        d[:, 2] = 1.0
    elif dof_name == "Yaw":
        d[:, 1] = -1.0
    return d


def forward_speed_group(mesh, dofs, omega, beta, forward_speed, radiating=(), diffraction=True, influenced=None,
                        rho=1000.0, g=9.81, gfs=DEFAULT_WU, lid_mesh=None, lapack=True):
    """solve(problem, IndirectBEM()) (solve.jl:35-65) for the radiation problems of
    ``radiating`` and (optionally) the diffraction problem at one (omega, beta, U):
    encountered frequency and wavenumber (waves.jl:136-151), radiation condition with the
    U * n . d(dof)/dx term (waves.jl:183-199), Airy condition with the encountered heading
    (waves.jl:243-282), indirect solve, pressure i rho omega_e phi + rho U (K sigma)
    with K assembled for the fixed normal [1, 0, 0] (solve.jl:35-45).  Returns
    (omega_e, [force dict per problem]) in the order radiating..., diffraction."""
    names = list(dofs.keys())
    influenced = names if influenced is None else list(influenced)
    oe, ke, be = encountered_values(omega, beta, forward_speed, g)
    k = omega * omega / g
    n = mesh.nfaces
    rhs = []
    for d in radiating:
        bc = -1j * oe * np.einsum("ij,ij->i", mesh.normals, dofs[d])
        if forward_speed != 0:
            bc = bc + forward_speed * np.einsum("ij,ij->i", mesh.normals, gradient_of_motion(n, d))
        rhs.append(bc)
    if diffraction:
        c = np.asarray(mesh.centers)
        wbar = c[:, 0] * np.cos(be) + c[:, 1] * np.sin(be)
        cih = np.exp(k * c[:, 2])
        amp = g * k / omega * np.exp(1j * k * wbar)
        v = np.stack([amp * np.cos(beta) * cih, amp * np.sin(beta) * cih, -1j * amp * cih], axis=1)
        rhs.append(-np.einsum("ij,ij->i", v, mesh.normals))
    full = mesh if lid_mesh is None else _combine(mesh, lid_mesh)
    S, D = assemble_matrices(full, ke, gfs=gfs, direct=False)
    B = pad_hull_bc(np.stack(rhs, axis=1), full.nfaces)
    phi, src = solve(D, S, B, direct=False, lapack=lapack)
    p = 1j * rho * oe * phi
    if forward_speed != 0:
        _, K = assemble_matrices(full, ke, gfs=gfs, direct=False, fixed_normal=[1.0, 0.0, 0.0])
        p = p + rho * forward_speed * (K @ src)
    p = p[:n]
    out = [{d: integrate_dof_pressure(mesh.normals, mesh.areas, dofs[d], p[:, q]) for d in influenced}
           for q in range(B.shape[1])]
    return oe, out


class _Panels:
    """Concatenated panel arrays of hull + lid (combine_meshes, meshes.jl:56-92)."""

    def __init__(self, meshes):
        self.panel_vertices = np.concatenate([np.asarray(m.panel_vertices) for m in meshes])
        self.centers = np.concatenate([np.asarray(m.centers) for m in meshes])
        self.normals = np.concatenate([np.asarray(m.normals) for m in meshes])
        self.areas = np.concatenate([np.asarray(m.areas) for m in meshes])
        self.radii = np.concatenate([np.asarray(m.radii) for m in meshes])
        self.nfaces = len(self.areas)


def _combine(hull, lid):
    return _Panels([hull, lid])


def num_threads():
    return lib().or_num_threads()
