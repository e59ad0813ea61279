"""Reverse-mode gradient (mh_hydro_gradient) against central finite differences.

Two truncated cylinders side by side; the objective is the summed diagonal added
mass + radiation damping of the objective dofs over a few frequencies.  The
finite differences use the device sweep (itself pinned against the oracle) with
h = 1e-6 along per-body affine vertex moves.  Affine moves keep every panel
planar: the Birk self term zeroes the solid-angle part of an in-plane field
point, so along a move that bends a panel out of its plane the primal is not
smooth at h = 0 and no derivative exists to compare with.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-6
OMEGAS = (0.6, 1.1, 1.7)
RTOL = 1e-6  # central differences at h = 1e-6 carry ~1e-9 relative rounding and h^2 truncation


def _geometry(mh):
    m1 = mh.vertical_cylinder_mesh(1.0, 1.6, 10, 4, 2)
    m2 = mh.vertical_cylinder_mesh(1.0, 1.6, 10, 4, 2, center=(4.0, 0.5))
    return m1, m2


def _body(mh, V1, V2, m1, m2, dofs):
    b1 = mh.FloatingBody(mh.StaticArraysMesh(V1, m1.faces), dofs, rotation_center=(0.0, 0.0, -0.5), body_name="c1")
    b2 = mh.FloatingBody(mh.StaticArraysMesh(V2, m2.faces), dofs, rotation_center=(4.0, 0.5, -0.5),
                         body_name="c2")
    return b1 + b2


def _objective(mh, ctx, body, obj, F):
    r = mh.hydrodynamic_coefficients(body, {"wave_frequencies": OMEGAS, "radiating_dofs": obj,
                                            "influenced_dofs": obj}, F, ctx=ctx, rho=1025.0, g=9.81)
    A, B = r["added_mass"][..., 0], r["radiation_damping"][..., 0]
    return sum(A[h, h, w] + B[h, h, w] for h in range(len(obj)) for w in range(len(OMEGAS)))


def _affine_moves(V1, V2, rng):
    """Per-body affine vertex moves that keep z = 0 at z = 0 (no panel leaves the water)."""
    moves = []
    for which in (0, 1):
        M = rng.standard_normal((3, 3))
        M[2, :2] = 0.0
        t = np.array([rng.standard_normal(), rng.standard_normal(), 0.0])
        d1 = V1 @ M.T + t if which == 0 else np.zeros_like(V1)
        d2 = V2 @ M.T + t if which == 1 else np.zeros_like(V2)
        moves.append((d1, d2))
    moves.append((np.zeros_like(V1), np.tile([1.0, 0.0, 0.0], (len(V2), 1))))  # spacing
    moves.append((V1 * [0.0, 0.0, 1.0], np.zeros_like(V2)))                      # draft of body 1
    return moves


@pytest.mark.parametrize("gf,obj", [("wu_heave", ["c1__Heave", "c2__Heave"]),
                                    ("wu_pitch", ["c1__Pitch", "c2__Heave"]),
                                    ("rankine", ["c1__Heave"])])
def test_gradient_matches_finite_differences(mh, ctx, gf, obj):
    F = mh.DirectBEM() if gf.startswith("wu") else mh.DirectBEM((mh.Rankine(), mh.RankineReflectedNegative()))
    m1, m2 = _geometry(mh)
    dofs = ["Heave", "Pitch"]
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, dofs)
    J, grad = mh.hydro_gradient(body, OMEGAS, obj, F, ctx=ctx, rho=1025.0, g=9.81)
    J_sweep = _objective(mh, ctx, body, obj, F)
    assert abs(J - J_sweep) <= 1e-12 * abs(J_sweep)
    n1 = m1.nvertices
    rng = np.random.default_rng(11)
    for d1, d2 in _affine_moves(m1.vertices, m2.vertices, rng):
        jp = _objective(mh, ctx, _body(mh, m1.vertices + H * d1, m2.vertices + H * d2, m1, m2, dofs), obj, F)
        jm = _objective(mh, ctx, _body(mh, m1.vertices - H * d1, m2.vertices - H * d2, m1, m2, dofs), obj, F)
        fd = (jp - jm) / (2 * H)
        ad = float(np.sum(grad[:n1] * d1) + np.sum(grad[n1:] * d2))
        scale = np.abs(grad).sum() * max(np.abs(d1).max(), np.abs(d2).max())
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * scale), (ad, fd)


def _oracle_objective(oracle, body, obj, gfs, direct):
    J = 0.0
    for om in OMEGAS:
        A, B, _, _, _ = oracle.hydro_one_frequency(body.mesh, body.dofs, om, rho=1025.0, g=9.81, radiating=obj,
                                                   influenced=obj, gfs=gfs, direct=direct)
        J += float(np.trace(A) + np.trace(B))
    return J


@pytest.mark.parametrize("gf", ["Wu", "ExactGuevelDelhommeau"])
@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("obj", [["c1__Heave", "c2__Heave"], ["c1__Pitch", "c2__Heave"]])
def test_gradient_matches_oracle_finite_differences(mh, oracle, ctx, obj, direct, gf):
    """The device adjoint against central differences of the CPU oracle (not of the device sweep):
    the two-cylinder mesh of 120 panels, the same affine moves; DirectBEM and IndirectBEM, the Wu
    and the exact Guevel-Delhommeau wave terms.  h = 1e-6: the moves are large affine maps, whose
    h^2 truncation already reaches 2e-5 at h = 1e-5; the oracle's quadrature noise (1e-13 of J)
    over h stays near 1e-7."""
    m1, m2 = _geometry(mh)
    dofs = ["Heave", "Pitch"]
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, dofs)
    assert body.mesh.nfaces <= 150
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(gf)
    gfs = oracle.DEFAULT_WU if gf == "Wu" else oracle.DEFAULT_EGD
    h = H
    J, grad = mh.hydro_gradient(body, OMEGAS, obj, F, ctx=ctx, rho=1025.0, g=9.81)
    J_oracle = _oracle_objective(oracle, body, obj, gfs, direct)
    assert abs(J - J_oracle) <= 1e-8 * abs(J_oracle)
    n1 = m1.nvertices
    rng = np.random.default_rng(23)
    for d1, d2 in _affine_moves(m1.vertices, m2.vertices, rng):
        jp = _oracle_objective(oracle, _body(mh, m1.vertices + h * d1, m2.vertices + h * d2, m1, m2, dofs), obj,
                               gfs, direct)
        jm = _oracle_objective(oracle, _body(mh, m1.vertices - h * d1, m2.vertices - h * d2, m1, m2, dofs), obj,
                               gfs, direct)
        fd = (jp - jm) / (2 * h)
        ad = float(np.sum(grad[:n1] * d1) + np.sum(grad[n1:] * d2))
        scale = np.abs(grad).sum() * max(np.abs(d1).max(), np.abs(d2).max())
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * scale), (ad, fd)


@pytest.mark.parametrize("direct", [True, False])
def test_vjp_with_full_cotangents_matches_oracle(mh, oracle, ctx, direct):
    """General cotangents of A, B and the excitation forces, IndirectBEM and DirectBEM, against
    central differences of the oracle's sweep along one affine move."""
    m1, m2 = _geometry(mh)
    dofs = ["Heave", "Pitch"]
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, dofs)
    names = list(body.dofs)
    rng = np.random.default_rng(31)
    betas = [0.0, 1.1]
    ab = rng.standard_normal((4, 4, len(OMEGAS)))
    bb = rng.standard_normal((4, 4, len(OMEGAS)))
    fb = rng.standard_normal((4, len(OMEGAS), 2)) + 1j * rng.standard_normal((4, len(OMEGAS), 2))
    F = (mh.DirectBEM if direct else mh.IndirectBEM)()
    J, grad = mh.hydro_vjp(body, OMEGAS, names, names, ab, bb, F, ctx=ctx, rho=1025.0, g=9.81,
                           wave_directions=betas, excitation_force_bar=fb)

    def objective(b):
        tot = 0.0
        for w, om in enumerate(OMEGAS):
            A, B, _, _, Fe = oracle.hydro_one_frequency(b.mesh, b.dofs, om, rho=1025.0, g=9.81, betas=betas,
                                                        direct=direct)
            tot += np.sum(ab[:, :, w] * A) + np.sum(bb[:, :, w] * B)
            tot += np.sum(fb[:, w, :].real * Fe.real + fb[:, w, :].imag * Fe.imag)
        return float(tot)

    assert abs(J - objective(body)) <= 1e-8 * abs(J)
    M = rng.standard_normal((3, 3))
    M[2, :2] = 0.0
    d1 = m1.vertices @ M.T
    d2 = np.zeros_like(m2.vertices)
    jp = objective(_body(mh, m1.vertices + H * d1, m2.vertices, m1, m2, dofs))
    jm = objective(_body(mh, m1.vertices - H * d1, m2.vertices, m1, m2, dofs))
    fd = (jp - jm) / (2 * H)
    ad = float(np.sum(grad[:m1.nvertices] * d1))
    assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * np.abs(grad).sum() * np.abs(d1).max()), (ad, fd)


def test_gradient_rejects_unsupported(mh, ctx):
    m1, m2 = _geometry(mh)
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, ["Heave"])
    both = (mh.Rankine(), mh.RankineReflected(), mh.GFWu(), mh.ExactGuevelDelhommeau())
    with pytest.raises(ValueError):
        mh.hydro_gradient(body, OMEGAS, ["c1__Heave"], mh.DirectBEM(both), ctx=ctx)
    with pytest.raises(ValueError):
        mh.hydro_gradient(body, OMEGAS, ["c1__Heave"], mh.DirectBEM("Surrogate"), ctx=ctx)


def _soup(mh, V4, C, N, A, R):
    """A mesh whose panels own their corners and carry the given (independent) fields."""
    n = len(C)
    return mh.StaticArraysMesh(V4.reshape(-1, 3), np.arange(4 * n).reshape(n, 4) + 1, C, N, A, R)


def _inplane(v, N):
    """Component of v (n, ..., 3) orthogonal to each panel normal N (n, 3)."""
    if v.ndim == 3:
        return v - np.einsum("iqk,ik->iq", v, N)[..., None] * N[:, None, :]
    return v - np.sum(v * N, axis=1)[:, None] * N


@pytest.mark.parametrize("wu", [True, False])
def test_panel_terms_match_finite_differences(mh, ctx, wu):
    """Each per-panel term of mh_hydro_gradient alone: areas, normals, in-plane centre
    moves, in-plane corner moves and dof fields, perturbed independently.  In-plane
    moves keep every self and coplanar pair in the plane of its panel; a triangle's
    repeated corner moves with its twin (moved apart, the zero-length edge the Birk
    integral skips would open: a kink, not a derivative)."""
    from importlib import import_module
    dev = import_module("marinehydro_gb300._device")
    m1, m2 = _geometry(mh)
    mesh = m1 + m2
    body = mh.FloatingBody(mesh, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, -0.5))
    dofs = body.dof_array(["Heave", "Pitch"])
    obj = [0, 1]
    gfs = mh.gf_flags((mh.Rankine(), mh.RankineReflected()) + ((mh.GFWu(),) if wu else ()))
    V4, C, N, A, R = mesh.panel_vertices, mesh.centers, mesh.normals, mesh.areas, mesh.radii

    def J(V4_, C_, N_, A_, dofs_):
        sm = _soup(mh, V4_, C_, N_, A_, R)
        a, b, *_ = dev.hydro_sweep(ctx, sm.device_mesh(ctx), OMEGAS, 1025.0, 9.81, gfs, True, dofs_, obj, obj, [])
        return sum(a[h, h, w] + b[h, h, w] for h in range(2) for w in range(len(OMEGAS)))

    sm0 = _soup(mh, V4, C, N, A, R)
    J0, gc, gn, ga, gv, gd = dev.hydro_gradient(ctx, sm0.device_mesh(ctx), OMEGAS, 1025.0, 9.81, gfs, dofs, obj)
    assert abs(J0 - J(V4, C, N, A, dofs)) <= 1e-12 * abs(J0)
    rng = np.random.default_rng(17)
    z = np.zeros_like
    dAr = rng.standard_normal(A.shape) * A
    dN = rng.standard_normal(N.shape)
    dC = _inplane(rng.standard_normal(C.shape), N)
    dV = _inplane(rng.standard_normal(V4.shape), N)
    tri = np.all(V4[:, 3] == V4[:, 2], axis=1)  # a triangle's repeated corner moves with its twin
    dV[tri, 3] = dV[tri, 2]
    dD = np.zeros_like(dofs)
    dD[obj] = rng.standard_normal(dofs[obj].shape)
    cases = {"areas": ((z(V4), z(C), z(N), dAr, z(dofs)), np.sum(ga * dAr)),
             "normals": ((z(V4), z(C), dN, z(A), z(dofs)), np.sum(gn * dN)),
             "centers": ((z(V4), dC, z(N), z(A), z(dofs)), np.sum(gc * dC)),
             "corners": ((dV, z(C), z(N), z(A), z(dofs)), np.sum(gv * dV)),
             "dofs": ((z(V4), z(C), z(N), z(A), dD), np.sum(gd * dD[obj]))}
    bad = {}
    for name, (d, ad) in cases.items():
        plus = [x + H * dx for x, dx in zip((V4, C, N, A, dofs), d)]
        minus = [x - H * dx for x, dx in zip((V4, C, N, A, dofs), d)]
        fd = (J(*plus) - J(*minus)) / (2 * H)
        if not abs(ad - fd) <= RTOL * max(abs(fd), 1e-6 * abs(J0)):
            bad[name] = (ad, fd)
    assert not bad, bad


@pytest.mark.parametrize("precision", ["mixed", "fp64_tc"])
def test_other_precisions_match_fp64(mh, ctx, precision):
    """FP32 factors + refinement of both solves, or the FP64 LU with its update on the tensor
    cores: J and the gradient agree with the FP64 path."""
    m1, m2 = _geometry(mh)
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, ["Heave", "Pitch"])
    obj = ["c1__Heave", "c2__Pitch"]
    J64, g64 = mh.hydro_gradient(body, OMEGAS, obj, mh.DirectBEM(), ctx=ctx, rho=1025.0)
    J32, g32 = mh.hydro_gradient(body, OMEGAS, obj, mh.DirectBEM(precision=precision), ctx=ctx, rho=1025.0)
    assert abs(J32 - J64) <= 1e-12 * abs(J64)
    assert np.abs(g32 - g64).max() <= 1e-10 * np.abs(g64).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vjp_with_full_cotangents_matches_finite_differences(mh, ctx, precision):
    """mh_hydro_vjp with dense random cotangents on every (influenced, radiating, omega)
    entry of A and B, off-diagonal couplings and rotation dofs included."""
    F = mh.DirectBEM(precision=precision)
    m1, m2 = _geometry(mh)
    dofs = ["Surge", "Heave", "Pitch"]
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, dofs)
    rad = ["c1__Heave", "c2__Pitch", "c1__Surge", "c2__Heave", "c1__Pitch"]  # five columns: two kernel groups
    inf = ["c2__Heave", "c1__Pitch", "c1__Heave"]
    betas = [0.0, 1.1]
    rng = np.random.default_rng(5)
    ab = rng.standard_normal((3, 5, len(OMEGAS)))
    bb = rng.standard_normal((3, 5, len(OMEGAS)))
    # excitation forces are ~1e4 times larger than A, B here: scale their cotangents alike
    fb = 1e-4 * (rng.standard_normal((3, len(OMEGAS), 2)) + 1j * rng.standard_normal((3, len(OMEGAS), 2)))

    def objective(b):
        r = mh.hydrodynamic_coefficients(b, {"wave_frequencies": OMEGAS, "radiating_dofs": rad,
                                             "influenced_dofs": inf, "wave_directions": betas}, mh.DirectBEM(),
                                         ctx=ctx, rho=1025.0, g=9.81)
        fe = r["excitation_force"][..., 0]
        return float(np.sum(ab * r["added_mass"][..., 0]) + np.sum(bb * r["radiation_damping"][..., 0])
                     + np.sum(fb.real * fe.real) + np.sum(fb.imag * fe.imag))

    J, grad = mh.hydro_vjp(body, OMEGAS, rad, inf, ab, bb, F, ctx=ctx, rho=1025.0, g=9.81, wave_directions=betas,
                           excitation_force_bar=fb)
    J0 = objective(body)
    assert abs(J - J0) <= 1e-11 * np.abs(ab).sum() * 1e3 + 1e-12 * abs(J0)
    n1 = m1.nvertices
    for d1, d2 in _affine_moves(m1.vertices, m2.vertices, np.random.default_rng(17)):
        jp = objective(_body(mh, m1.vertices + H * d1, m2.vertices + H * d2, m1, m2, dofs))
        jm = objective(_body(mh, m1.vertices - H * d1, m2.vertices - H * d2, m1, m2, dofs))
        fd = (jp - jm) / (2 * H)
        ad = float(np.sum(grad[:n1] * d1) + np.sum(grad[n1:] * d2))
        scale = np.abs(grad).sum() * max(np.abs(d1).max(), np.abs(d2).max())
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * scale), (ad, fd)


def test_vjp_with_identity_cotangents_equals_gradient(mh, ctx):
    m1, m2 = _geometry(mh)
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, ["Heave", "Pitch"])
    obj = ["c1__Pitch", "c2__Heave"]
    J1, g1 = mh.hydro_gradient(body, OMEGAS, obj, ctx=ctx, rho=1025.0, g=9.81)
    eye = np.repeat(np.eye(2)[:, :, None], len(OMEGAS), axis=2)
    J2, g2 = mh.hydro_vjp(body, OMEGAS, obj, obj, eye, eye, ctx=ctx, rho=1025.0, g=9.81)
    assert J1 == pytest.approx(J2, rel=1e-14)
    assert np.abs(g1 - g2).max() <= 1e-13 * np.abs(g1).max()


def test_vjp_of_excitation_forces_alone(mh, ctx):
    """Only excitation cotangents (no radiating dofs): the diffraction solve, the Airy
    condition's and the Froude-Krylov pressure's dependence on the panel centres."""
    m1, m2 = _geometry(mh)
    dofs = ["Surge", "Heave", "Pitch"]
    body = _body(mh, m1.vertices, m2.vertices, m1, m2, dofs)
    inf = ["c1__Surge", "c2__Heave", "c1__Pitch"]
    betas = [0.3, 2.0]
    rng = np.random.default_rng(23)
    fb = rng.standard_normal((3, len(OMEGAS), 2)) + 1j * rng.standard_normal((3, len(OMEGAS), 2))

    def objective(b):
        r = mh.hydrodynamic_coefficients(b, {"wave_frequencies": OMEGAS, "influenced_dofs": inf,
                                             "wave_directions": betas}, ctx=ctx, rho=1025.0, g=9.81)
        fe = r["excitation_force"][..., 0]
        return float(np.sum(fb.real * fe.real) + np.sum(fb.imag * fe.imag))

    J, grad = mh.hydro_vjp(body, OMEGAS, [], inf, ctx=ctx, rho=1025.0, g=9.81, wave_directions=betas,
                           excitation_force_bar=fb)
    assert abs(J - objective(body)) <= 1e-11 * abs(J)
    n1 = m1.nvertices
    for d1, d2 in _affine_moves(m1.vertices, m2.vertices, np.random.default_rng(29)):
        jp = objective(_body(mh, m1.vertices + H * d1, m2.vertices + H * d2, m1, m2, dofs))
        jm = objective(_body(mh, m1.vertices - H * d1, m2.vertices - H * d2, m1, m2, dofs))
        fd = (jp - jm) / (2 * H)
        ad = float(np.sum(grad[:n1] * d1) + np.sum(grad[n1:] * d2))
        scale = np.abs(grad).sum() * max(np.abs(d1).max(), np.abs(d2).max())
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * scale), (ad, fd)
