"""Device-side handles and thin wrappers over the C-ABI calls."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MH_MEM_DEVICE, MH_MEM_HOST, ptr_and_mem


class DeviceMesh:
    """An mh_mesh: one body's panels resident on the device of `ctx`."""

    def __init__(self, ctx: _lib.Context, mesh, n_hull=None):
        self.ctx = ctx
        self.n = mesh.nfaces
        V = np.ascontiguousarray(mesh.panel_vertices, dtype=np.float64)
        C = np.ascontiguousarray(mesh.centers, dtype=np.float64)
        N = np.ascontiguousarray(mesh.normals, dtype=np.float64)
        A = np.ascontiguousarray(mesh.areas, dtype=np.float64)
        R = np.ascontiguousarray(mesh.radii, dtype=np.float64)
        h = ctypes.c_void_p()
        ctx.check(ctx._L.mh_mesh_create(ctx.handle, self.n, V.ctypes.data, C.ctypes.data, N.ctypes.data,
                                        A.ctypes.data, R.ctypes.data, MH_MEM_HOST, ctypes.byref(h)),
                  "mh_mesh_create")
        self._h = h
        self.n_hull = self.n
        if n_hull is not None and n_hull != self.n:
            ctx.check(ctx._L.mh_mesh_set_lid(self._h, int(n_hull)), "mh_mesh_set_lid")
            self.n_hull = int(n_hull)

    @classmethod
    def from_device_arrays(cls, ctx, n, V, C, N, A, R):
        """Build from device buffers (objects with __cuda_array_interface__)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.n = int(n)
        ptrs = [ptr_and_mem(x) for x in (V, C, N, A, R)]
        if any(m != MH_MEM_DEVICE for _, m in ptrs):
            raise TypeError("from_device_arrays needs device arrays")
        h = ctypes.c_void_p()
        ctx.check(ctx._L.mh_mesh_create(ctx.handle, self.n, *[p for p, _ in ptrs], MH_MEM_DEVICE, ctypes.byref(h)),
                  "mh_mesh_create")
        self._h = h
        return self

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.ctx._L.mh_mesh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _c128(a, shape=None, order="F"):
    a = np.asarray(a, dtype=np.complex128)
    if shape is not None:
        a = a.reshape(shape, order=order)
    return np.asfortranarray(a)


def assemble(ctx, dmesh: DeviceMesh, k: float, gfs: int, direct: bool, include_identity: bool, fixed_normal=None):
    n = dmesh.n
    S = np.empty((n, n), dtype=np.complex128, order="F")
    D = np.empty((n, n), dtype=np.complex128, order="F")
    fx = None
    if fixed_normal is not None:
        fx = np.ascontiguousarray(np.asarray(fixed_normal, dtype=np.float64).reshape(3))
    ctx.check(ctx._L.mh_assemble_matrices(ctx.handle, dmesh.handle, float(k), int(gfs), int(bool(direct)),
                                          int(bool(include_identity)), fx.ctypes.data if fx is not None else None,
                                          S.ctypes.data, D.ctypes.data, MH_MEM_HOST), "assemble_matrices")
    return S, D


def linsolve(ctx, A, B, precision=_lib.MH_PREC_FP64, adjoint=False):
    A = _c128(A)
    n = A.shape[0]
    if A.shape != (n, n):
        raise ValueError(f"A must be square, got {A.shape}")
    Bv = np.asarray(B, dtype=np.complex128)
    vec = Bv.ndim == 1
    if Bv.shape[0] != n:
        raise ValueError(f"dimension mismatch: A is {n}x{n}, b has {Bv.shape[0]} rows")
    Bm = np.asfortranarray(Bv.reshape(n, -1, order="F"))
    X = np.empty_like(Bm, order="F")
    fn = ctx._L.mh_linsolve_adjoint if adjoint else ctx._L.mh_linsolve
    ctx.check(fn(ctx.handle, n, Bm.shape[1], A.ctypes.data, Bm.ctypes.data, X.ctypes.data, int(precision),
                 MH_MEM_HOST), "linsolve")
    return X[:, 0].copy() if vec else X


def solve_linear(ctx, D, S, bc, direct=True, precision=_lib.MH_PREC_FP64):
    D = _c128(D)
    S = _c128(S)
    n = D.shape[0]
    b = np.asarray(bc, dtype=np.complex128)
    vec = b.ndim == 1
    if b.shape[0] != n or S.shape != (n, n) or D.shape != (n, n):
        raise ValueError("dimension mismatch between D, S and bc")
    B = np.asfortranarray(b.reshape(n, -1, order="F"))
    phi = np.empty_like(B, order="F")
    src = None if direct else np.empty_like(B, order="F")
    ctx.check(ctx._L.mh_solve(ctx.handle, n, B.shape[1], D.ctypes.data, S.ctypes.data, B.ctypes.data,
                              int(bool(direct)), phi.ctypes.data, None if direct else src.ctypes.data,
                              int(precision), MH_MEM_HOST), "solve")
    if vec:
        return phi[:, 0].copy(), (None if direct else src[:, 0].copy())
    return phi, src


def solve_pullback(ctx, D, S, bc, phi_bar, direct=True, sources_bar=None, precision=_lib.MH_PREC_FP64):
    """mh_solve_pullback with host buffers: (phi, sources, D_bar, S_bar, bc_bar)."""
    D = _c128(D)
    S = _c128(S)
    n = D.shape[0]
    b = np.asarray(bc, dtype=np.complex128)
    vec = b.ndim == 1
    if b.shape[0] != n or S.shape != (n, n) or D.shape != (n, n):
        raise ValueError("dimension mismatch between D, S and bc")
    B = np.asfortranarray(b.reshape(n, -1, order="F"))
    Pb = np.asfortranarray(np.asarray(phi_bar, dtype=np.complex128).reshape(B.shape, order="F"))
    Sb = None if sources_bar is None else np.asfortranarray(
        np.asarray(sources_bar, dtype=np.complex128).reshape(B.shape, order="F"))
    phi = np.empty_like(B, order="F")
    src = None if direct else np.empty_like(B, order="F")
    Dbar = np.empty((n, n), dtype=np.complex128, order="F")
    Sbar = np.empty((n, n), dtype=np.complex128, order="F")
    bcbar = np.empty_like(B, order="F")
    ctx.check(ctx._L.mh_solve_pullback(ctx.handle, n, B.shape[1], D.ctypes.data, S.ctypes.data, B.ctypes.data,
                                       int(bool(direct)), Pb.ctypes.data, None if Sb is None else Sb.ctypes.data,
                                       int(precision), phi.ctypes.data, None if direct else src.ctypes.data,
                                       Dbar.ctypes.data, Sbar.ctypes.data, bcbar.ctypes.data, MH_MEM_HOST),
              "solve pullback")
    if vec:
        return phi[:, 0].copy(), (None if direct else src[:, 0].copy()), Dbar, Sbar, bcbar[:, 0].copy()
    return phi, src, Dbar, Sbar, bcbar


def wu_wave_terms(ctx, hh, vv):
    hh = np.ascontiguousarray(np.asarray(hh, dtype=np.float64).ravel())
    vv = np.ascontiguousarray(np.asarray(vv, dtype=np.float64).ravel())
    m = hh.size
    out = np.empty((m, 3), dtype=np.complex128)
    ctx.check(ctx._L.mh_wu_wave_terms(ctx.handle, m, hh.ctypes.data, vv.ctypes.data, out.ctypes.data, MH_MEM_HOST),
              "wu wave terms")
    return out


def fixpoint_points(ctx, x):
    """exp(-|x|), log|x|, 1/|x|, sqrt|x| as the Wu kernels evaluate them on the integer pipe (m x 4)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
    out = np.empty((x.size, 4), dtype=np.float64)
    ctx.check(ctx._L.mh_fixpoint_points(ctx.handle, x.size, x.ctypes.data, out.ctypes.data, MH_MEM_HOST),
              "fixed-point points")
    return out


def bessel01_points(ctx, x):
    """J0, J1, Y0, Y1 as the Wu kernels evaluate them (m x 4; Y is NaN below x = 3)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
    out = np.empty((x.size, 4), dtype=np.float64)
    ctx.check(ctx._L.mh_bessel01_points(ctx.handle, x.size, x.ctypes.data, out.ctypes.data, MH_MEM_HOST),
              "Bessel points")
    return out


def exact_wave_terms(ctx, r, z, rtol=1e-12, atol=1e-14):
    r = np.ascontiguousarray(np.asarray(r, dtype=np.float64).ravel())
    z = np.ascontiguousarray(np.asarray(z, dtype=np.float64).ravel())
    m = r.size
    out = np.empty((m, 2), dtype=np.complex128)
    ctx.check(ctx._L.mh_exact_wave_terms(ctx.handle, m, r.ctypes.data, z.ctypes.data, float(rtol), float(atol),
                                         out.ctypes.data, MH_MEM_HOST), "exact wave terms")
    return out


def hydro_sweep(ctx, dmesh: DeviceMesh, omegas, rho, g, gfs, direct, dofs, rad_idx, inf_idx, betas,
                precision=_lib.MH_PREC_FP64, out=None):
    """mh_hydrodynamic_coefficients with host buffers; returns the five arrays."""
    om = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
    be = np.ascontiguousarray(np.asarray(betas, dtype=np.float64).ravel())
    dofs = np.ascontiguousarray(np.asarray(dofs, dtype=np.float64))
    ri = np.ascontiguousarray(np.asarray(rad_idx, dtype=np.int32).ravel())
    ii = np.ascontiguousarray(np.asarray(inf_idx, dtype=np.int32).ravel())
    nw, nb, nr, ni = om.size, be.size, ri.size, ii.size
    nd = dofs.shape[0] if dofs.size else 0
    A = np.empty((ni, nr, nw), dtype=np.float64, order="F")
    B = np.empty_like(A)
    Fd = np.empty((ni, nw, nb), dtype=np.complex128, order="F")
    Fk = np.empty_like(Fd)
    Fe = np.empty_like(Fd)
    p = lambda a: a.ctypes.data if a.size else None
    ctx.check(ctx._L.mh_hydrodynamic_coefficients(
        ctx.handle, dmesh.handle, nw, om.ctypes.data, float(rho), float(g), int(gfs), int(bool(direct)), nd,
        p(dofs), nr, p(ri), ni, p(ii), nb, p(be), int(precision), p(A), p(B), p(Fd), p(Fk), p(Fe), MH_MEM_HOST),
        "hydrodynamic_coefficients")
    return A, B, Fd, Fk, Fe


def hydro_frequency_derivative(ctx, dmesh: DeviceMesh, omegas, rho, g, gfs, direct, dofs, rad_idx, inf_idx, betas):
    """mh_hydro_frequency_derivative with host buffers; returns the five arrays and their
    omega-derivatives (ten arrays, layouts of hydro_sweep)."""
    om = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
    be = np.ascontiguousarray(np.asarray(betas, dtype=np.float64).ravel())
    dofs = np.ascontiguousarray(np.asarray(dofs, dtype=np.float64))
    ri = np.ascontiguousarray(np.asarray(rad_idx, dtype=np.int32).ravel())
    ii = np.ascontiguousarray(np.asarray(inf_idx, dtype=np.int32).ravel())
    nw, nb, nr, ni = om.size, be.size, ri.size, ii.size
    nd = dofs.shape[0] if dofs.size else 0
    out = []
    for _ in range(2):
        A = np.empty((ni, nr, nw), dtype=np.float64, order="F")
        out += [A, np.empty_like(A)] + [np.empty((ni, nw, nb), dtype=np.complex128, order="F") for _ in range(3)]
    p = lambda a: a.ctypes.data if a.size else None
    ctx.check(ctx._L.mh_hydro_frequency_derivative(
        ctx.handle, dmesh.handle, nw, om.ctypes.data, float(rho), float(g), int(gfs), int(bool(direct)), nd,
        p(dofs), nr, p(ri), ni, p(ii), nb, p(be), *[p(a) for a in out], MH_MEM_HOST), "hydro_frequency_derivative")
    return out


def batch_hydro(ctx, dmeshes, omegas_per_body, rho, g, gfs, direct, dofs_per_body, rad_idx, inf_idx, betas,
                precision=_lib.MH_PREC_FP64, n_streams=0):
    """mh_batch_hydrodynamic_coefficients with host buffers; returns per-body lists of the five arrays."""
    nb_ = len(dmeshes)
    nws = np.asarray([len(o) for o in omegas_per_body], dtype=np.int64)
    om = np.ascontiguousarray(np.concatenate([np.asarray(o, dtype=np.float64) for o in omegas_per_body]))
    be = np.ascontiguousarray(np.asarray(betas, dtype=np.float64).ravel())
    ri = np.ascontiguousarray(np.asarray(rad_idx, dtype=np.int32).ravel())
    ii = np.ascontiguousarray(np.asarray(inf_idx, dtype=np.int32).ravel())
    dofs = [np.ascontiguousarray(np.asarray(d, dtype=np.float64)) for d in dofs_per_body]
    nd = dofs[0].shape[0] if dofs and dofs[0].size else 0
    mesh_arr = (ctypes.c_void_p * nb_)(*[m.handle.value for m in dmeshes])
    dof_arr = (ctypes.c_void_p * nb_)(*[d.ctypes.data for d in dofs])
    W, nr, ni, nbeta = int(nws.sum()), ri.size, ii.size, be.size
    A = np.empty(ni * nr * W)
    B = np.empty_like(A)
    Fd = np.empty(ni * W * nbeta, dtype=np.complex128)
    Fk = np.empty_like(Fd)
    Fe = np.empty_like(Fd)
    p = lambda a: a.ctypes.data if a.size else None
    ctx.check(ctx._L.mh_batch_hydrodynamic_coefficients(
        ctx.handle, nb_, mesh_arr, nws.ctypes.data, om.ctypes.data, float(rho), float(g), int(gfs), int(bool(direct)),
        nd, dof_arr, nr, p(ri), ni, p(ii), nbeta, p(be), int(precision), int(n_streams), p(A), p(B), p(Fd), p(Fk),
        p(Fe), MH_MEM_HOST), "batch_hydrodynamic_coefficients")
    out = []
    w0 = 0
    for nw in nws:
        nw = int(nw)
        a = A[ni * nr * w0:ni * nr * (w0 + nw)].reshape((ni, nr, nw), order="F")
        b = B[ni * nr * w0:ni * nr * (w0 + nw)].reshape((ni, nr, nw), order="F")
        sl = slice(ni * nbeta * w0, ni * nbeta * (w0 + nw))
        fd, fk, fe = (x[sl].reshape((ni, nw, nbeta), order="F") for x in (Fd, Fk, Fe))
        out.append((a, b, fd, fk, fe))
        w0 += nw
    return out


def hydro_vjp(ctx, dmesh: DeviceMesh, omegas, rho, g, gfs, dofs, rad_idx, inf_idx, abar, bbar, betas=(), fbar=None,
              precision=_lib.MH_PREC_FP64, direct=True):
    """mh_hydro_vjp with host buffers: cotangents abar, bbar of shape (n_inf, n_rad, n_omega),
    fbar complex (n_inf, n_omega, n_beta).

    Returns (J, gc (n,3), gn (n,3), ga (n,), gv (n,4,3), gd (n_dofs,n,3))."""
    om = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
    be = np.ascontiguousarray(np.asarray(betas, dtype=np.float64).ravel())
    dofs = np.ascontiguousarray(np.asarray(dofs, dtype=np.float64))
    ri = np.ascontiguousarray(np.asarray(rad_idx, dtype=np.int32).ravel())
    ii = np.ascontiguousarray(np.asarray(inf_idx, dtype=np.int32).ravel())
    shape = (ii.size, ri.size, om.size)
    ab = np.asfortranarray(np.asarray(abar, dtype=np.float64).reshape(shape))
    bb = np.asfortranarray(np.asarray(bbar, dtype=np.float64).reshape(shape))
    fb = np.asfortranarray(np.zeros((ii.size, om.size, be.size), dtype=np.complex128) if fbar is None else
                           np.asarray(fbar, dtype=np.complex128).reshape((ii.size, om.size, be.size)))
    n = dmesh.n
    J = ctypes.c_double()
    gc = np.empty((n, 3))
    gn = np.empty((n, 3))
    ga = np.empty(n)
    gv = np.empty((n, 4, 3))
    gd = np.empty((dofs.shape[0], n, 3))
    p = lambda a: a.ctypes.data if a.size else None
    ctx.check(ctx._L.mh_hydro_vjp(
        ctx.handle, dmesh.handle, om.size, om.ctypes.data, float(rho), float(g), int(gfs), int(bool(direct)),
        dofs.shape[0], dofs.ctypes.data, ri.size, p(ri), ii.size, ii.ctypes.data, be.size, p(be), p(ab), p(bb), p(fb),
        int(precision), ctypes.byref(J), gc.ctypes.data, gn.ctypes.data, ga.ctypes.data, gv.ctypes.data,
        gd.ctypes.data, MH_MEM_HOST), "hydro_vjp")
    return J.value, gc, gn, ga, gv, gd


def hydro_gradient(ctx, dmesh: DeviceMesh, omegas, rho, g, gfs, dofs, obj_idx, precision=_lib.MH_PREC_FP64,
                   direct=True):
    """mh_hydro_gradient with host buffers.

    Returns (J, gc (n,3), gn (n,3), ga (n,), gv (n,4,3), gd (n_obj,n,3)): the objective
    J = sum_omega sum_h A_hh + B_hh and its gradient w.r.t. the panel fields, the Birk
    corners and the objective dof fields."""
    om = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64).ravel())
    dofs = np.ascontiguousarray(np.asarray(dofs, dtype=np.float64))
    oi = np.ascontiguousarray(np.asarray(obj_idx, dtype=np.int32).ravel())
    n = dmesh.n
    J = ctypes.c_double()
    gc = np.empty((n, 3))
    gn = np.empty((n, 3))
    ga = np.empty(n)
    gv = np.empty((n, 4, 3))
    gd = np.empty((oi.size, n, 3))
    ctx.check(ctx._L.mh_hydro_gradient(
        ctx.handle, dmesh.handle, om.size, om.ctypes.data, float(rho), float(g), int(gfs), int(bool(direct)),
        dofs.shape[0], dofs.ctypes.data, oi.size, oi.ctypes.data, int(precision), ctypes.byref(J), gc.ctypes.data, gn.ctypes.data, ga.ctypes.data,
        gv.ctypes.data, gd.ctypes.data, MH_MEM_HOST), "hydro_gradient")
    return J.value, gc, gn, ga, gv, gd
