"""Irregular-frequency lid and forward speed on the GPU, against the CPU oracle.

Lid (solve.jl:2-28): the matrices cover hull + lid, the boundary conditions are zero on
the lid and only hull pressures enter the forces.  Forward speed (solve.jl:35-45,
waves.jl:136-199, problems_and_results.jl:262-363): encountered frequency and wavenumber,
the U n.d(dof)/dx term of the radiation condition, pressure i rho omega_e phi + rho U K sigma,
IndirectBEM only.  Bar: coefficients within 1e-8 of the oracle (relative to the largest
entry of each array).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_COEF = 1e-8


def close(a, b, rel=REL_COEF):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-300)


def _cylinder_with_lid(mh):
    hull = mh.vertical_cylinder_mesh(1.0, 1.0, n_theta=24, n_z=8, n_r=5)
    lid = mh.disc_lid_mesh(1.0, -0.15, n_theta=24, n_r=5)
    return hull, lid


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
@pytest.mark.parametrize("direct", [True, False])
def test_sweep_with_lid_matches_oracle(mh, oracle, ctx, direct, precision):
    hull, lid = _cylinder_with_lid(mh)
    dofs = ["Surge", "Heave", "Pitch"]
    body = mh.FloatingBody(hull, dofs, rotation_center=(0.0, 0.0, -0.5), lid_mesh=lid)
    oms = [1.5, 4.9]
    betas = [0.0, np.pi / 4]
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(precision=precision)
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": dofs,
                                              "wave_directions": betas}, F, ctx=ctx, rho=1025.0)
    for w, om in enumerate(oms):
        A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(hull, body.dofs, om, rho=1025.0, direct=direct, betas=betas,
                                                      lid_mesh=lid)
        assert close(res["added_mass"][:, :, w, 0], A)
        assert close(res["radiation_damping"][:, :, w, 0], B)
        assert close(res["diffraction_force"][:, w, :, 0], Fd)
        assert close(res["Froude_Krylov_force"][:, w, :, 0], Fk)
        assert close(res["excitation_force"][:, w, :, 0], Fe)


def test_lid_removes_irregular_frequency_on_gpu(mh, ctx):
    """Heave A, B of the a = T = 1 m cylinder around its irregular frequency (4.90 rad/s)."""
    hull, lid = _cylinder_with_lid(mh)
    oms = [4.8, 4.9, 5.0]
    params = {"wave_frequencies": oms, "radiating_dofs": ["Heave"]}
    r0 = mh.hydrodynamic_coefficients(mh.FloatingBody(hull, ["Heave"]), params, ctx=ctx, rho=1025.0)
    r1 = mh.hydrodynamic_coefficients(mh.FloatingBody(hull, ["Heave"], lid_mesh=lid), params, ctx=ctx, rho=1025.0)
    bump = lambda y: abs(y[1] - 0.5 * (y[0] + y[2]))
    A0, B0 = r0["added_mass"].ravel(), r0["radiation_damping"].ravel()
    A1, B1 = r1["added_mass"].ravel(), r1["radiation_damping"].ravel()
    assert bump(A0) > 0.02 * abs(A0[1]) and bump(B0) > 0.5 * abs(B0[1])
    assert bump(A1) < 1e-3 * abs(A1[1]) and bump(B1) < 0.05 * abs(B1[1])


def test_problem_solve_and_batch_with_lid_match_sweep(mh, ctx):
    hull, lid = _cylinder_with_lid(mh)
    body = mh.FloatingBody(hull, ["Heave", "Surge"], lid_mesh=lid)
    params = {"wave_frequencies": [2.2], "radiating_dofs": ["Heave"], "wave_directions": [0.3]}
    res = mh.hydrodynamic_coefficients(body, params, ctx=ctx, rho=1025.0)
    r = mh.solve(mh.RadiationProblem(body, 2.2, "Heave", ["Heave", "Surge"], rho=1025.0), ctx=ctx)
    d = mh.solve(mh.DiffractionProblem(body, 2.2, 0.3, ["Heave", "Surge"], rho=1025.0), ctx=ctx)
    a = mh.added_mass(r)
    assert a["Heave"] == pytest.approx(res["added_mass"][0, 0, 0, 0], rel=1e-10)
    fe = mh.excitation_force(d)
    assert abs(fe["Heave"] - res["excitation_force"][0, 0, 0, 0]) <= 1e-10 * abs(fe["Heave"])
    plain = mh.FloatingBody(mh.vertical_cylinder_mesh(1.5, 2.0, 16, 6, 4), ["Heave", "Surge"])
    out = mh.batch_hydrodynamic_coefficients([body, plain], [params, params], ctx=ctx, rho=1025.0)
    ref1 = mh.hydrodynamic_coefficients(plain, params, ctx=ctx, rho=1025.0)
    for key in ("added_mass", "radiation_damping", "excitation_force"):
        assert close(out[0][key], res[key], 1e-10)
        assert close(out[1][key], ref1[key], 1e-10)


def test_device_rejects_lid_at_free_surface(mh, ctx):
    hull = mh.vertical_cylinder_mesh(1.0, 1.0, n_theta=12, n_z=4, n_r=3)
    surface = mh.disc_lid_mesh(1.0, 0.0, n_theta=12, n_r=3)
    both = mh.combine_meshes([hull, surface])
    dm = mh.api._device.DeviceMesh(ctx, both)
    assert ctx._L.mh_mesh_set_lid(dm.handle, hull.nfaces) == 1  # MH_ERR_ARG
    assert b"below the free surface" in ctx._L.mh_last_error(ctx.handle)
    assert ctx._L.mh_mesh_set_lid(dm.handle, 0) == 1
    assert ctx._L.mh_mesh_set_lid(dm.handle, both.nfaces) == 0  # no lid


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_forward_speed_coefficients_match_oracle(mh, oracle, ctx, precision):
    """forward_speeds = [0, 0.8] m/s, two headings, IndirectBEM, hemisphere with 3 dofs."""
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    dofs = ["Surge", "Heave", "Pitch"]
    body = mh.FloatingBody(mesh, dofs, body_name="sphere")
    oms = [1.2, 2.0]
    betas = [0.0, 2.0]
    Us = [0.0, 0.8]
    params = {"wave_frequencies": oms, "radiating_dofs": dofs, "wave_directions": betas, "forward_speeds": Us}
    res = mh.hydrodynamic_coefficients(body, params, mh.IndirectBEM(precision=precision), ctx=ctx, rho=1025.0)
    assert res["added_mass"].shape == (3, 3, 2, 2, 2)
    assert res["excitation_force"].shape == (3, 2, 2, 2)
    for iU, U in enumerate(Us):
        for iw, om in enumerate(oms):
            for ib, beta in enumerate(betas):
                oe, forces = oracle.forward_speed_group(mesh, body.dofs, om, beta, U, radiating=dofs, rho=1025.0)
                F = np.array([[f[d] for d in dofs] for f in forces])  # [problem, influenced]
                A = F[:3].real.T / oe ** 2
                B = F[:3].imag.T / oe
                assert close(res["added_mass"][:, :, iw, iU, ib], A)
                assert close(res["radiation_damping"][:, :, iw, iU, ib], B)
                assert close(res["diffraction_force"][:, iw, ib, iU], F[3])
    # zero speed equals the plain sweep, for every heading
    plain = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": dofs,
                                                "wave_directions": betas}, mh.IndirectBEM(precision=precision),
                                         ctx=ctx, rho=1025.0)
    for ib in range(2):
        assert close(res["added_mass"][:, :, :, 0, ib], plain["added_mass"][..., 0], 1e-12)
    assert close(res["excitation_force"][..., 0], plain["excitation_force"][..., 0], 1e-12)
    with pytest.raises(ValueError, match="direct method"):
        mh.hydrodynamic_coefficients(body, params, mh.DirectBEM(), ctx=ctx)


def test_forward_speed_problem_solve_matches_oracle(mh, oracle, ctx):
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    hull, lid = _cylinder_with_lid(mh)
    for m, lm in ((mesh, None), (hull, lid)):
        body = mh.FloatingBody(m, ["Heave", "Pitch"], lid_mesh=lm)
        r = mh.solve(mh.RadiationProblem(body, 1.6, "Pitch", ["Heave", "Pitch"], beta=0.5, forward_speed=1.1,
                                         rho=1025.0), mh.IndirectBEM(), ctx=ctx)
        d = mh.solve(mh.DiffractionProblem(body, 1.6, 0.5, ["Heave", "Pitch"], forward_speed=1.1, rho=1025.0),
                     mh.IndirectBEM(), ctx=ctx)
        oe, forces = oracle.forward_speed_group(m, body.dofs, 1.6, 0.5, 1.1, radiating=["Pitch"], rho=1025.0,
                                                lid_mesh=lm)
        assert r.problem.encountered_omega == pytest.approx(oe, rel=1e-15)
        for dname in ("Heave", "Pitch"):
            assert abs(r.forces[dname] - forces[0][dname]) <= REL_COEF * abs(forces[0]["Pitch"])
            assert abs(d.forces[dname] - forces[1][dname]) <= REL_COEF * max(abs(forces[1]["Heave"]), 1.0)
