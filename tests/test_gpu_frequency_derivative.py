"""d/d omega of the hydrodynamic coefficients (mh_hydro_frequency_derivative).

The reference differentiates hydrodynamic_coefficients in omega with ForwardDiff and
checks it against central finite differences (test/outputs_differentiation.jl:39-150,
solve_problem_differentiation.jl:89-110, diffraction_differentiation.jl:63-78).  Here the
forward-mode device derivative is checked against central differences of the GPU sweep
and of the CPU oracle (h = 1e-5 omega: truncation ~h^2, rounding ~1e-11), bar 1e-6 of the
largest entry of each array, for the Wu and the exact Guevel-Delhommeau wave terms; the
coefficients themselves equal the plain sweep's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("added_mass", "radiation_damping", "diffraction_force", "Froude_Krylov_force", "excitation_force")


def close(a, b, rel):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-300)


def _fd(fn, om, h):
    hi, lo = fn(om + h), fn(om - h)
    return {k: (hi[k] - lo[k]) / (2 * h) for k in KEYS}


@pytest.mark.parametrize("direct", [True, False])
def test_derivative_matches_central_differences(mh, ctx, direct):
    mesh = mh.hemisphere_mesh(1.0, 8, 16)
    dofs = ["Surge", "Heave", "Pitch"]
    body = mh.FloatingBody(mesh, dofs, rotation_center=(0.0, 0.0, -0.3))
    F = mh.DirectBEM() if direct else mh.IndirectBEM()
    for om in (0.7, 1.9, 3.1):
        params = {"wave_frequencies": [om], "radiating_dofs": dofs, "wave_directions": [0.0, 0.9]}
        res = mh.hydrodynamic_coefficients_derivative(body, params, F, ctx=ctx, rho=1025.0)
        plain = mh.hydrodynamic_coefficients(body, params, F, ctx=ctx, rho=1025.0)
        for k in KEYS:
            assert close(res[k], plain[k], 1e-12), k
        fd = _fd(lambda w: mh.hydrodynamic_coefficients(body, dict(params, wave_frequencies=[w]), F, ctx=ctx,
                                                        rho=1025.0), om, 1e-5 * om)
        for k in KEYS:
            assert close(res["d_" + k], fd[k], 1e-6), (om, k)


def test_derivative_with_lid_and_several_frequencies(mh, ctx):
    hull = mh.vertical_cylinder_mesh(1.0, 1.0, n_theta=20, n_z=6, n_r=4)
    lid = mh.disc_lid_mesh(1.0, -0.15, n_theta=20, n_r=4)
    body = mh.FloatingBody(hull, ["Heave", "Surge"], lid_mesh=lid)
    oms = [1.0, 2.5, 4.0]
    params = {"wave_frequencies": oms, "radiating_dofs": ["Heave", "Surge"], "wave_directions": [0.4]}
    res = mh.hydrodynamic_coefficients_derivative(body, params, ctx=ctx, rho=1025.0)
    assert res["d_added_mass"].shape == (2, 2, 3, 1)
    for w, om in enumerate(oms):
        h = 1e-5 * om
        fd = _fd(lambda x: mh.hydrodynamic_coefficients(body, dict(params, wave_frequencies=[x]), ctx=ctx, rho=1025.0),
                 om, h)
        assert close(res["d_added_mass"][:, :, w], fd["added_mass"][:, :, 0], 1e-6)
        assert close(res["d_radiation_damping"][:, :, w], fd["radiation_damping"][:, :, 0], 1e-6)
        assert close(res["d_excitation_force"][:, w], fd["excitation_force"][:, 0], 1e-6)


@pytest.mark.parametrize("gf,direct", [("Wu", True), ("ExactGuevelDelhommeau", True),
                                       ("ExactGuevelDelhommeau", False)])
def test_derivative_matches_oracle_differences(mh, oracle, ctx, gf, direct):
    """The device derivative against central differences of the CPU oracle, with the Wu term and
    with the exact Guevel-Delhommeau term (the latter as ForwardDiff over omega with
    ExactGuevelDelhommeau in test/outputs_differentiation.jl:70-84); h = 1e-5 omega."""
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    body = mh.FloatingBody(mesh, ["Heave", "Surge"])
    om, h = 1.4, 1.4e-5
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(gf)
    gfs = oracle.DEFAULT_WU if gf == "Wu" else oracle.DEFAULT_EGD
    res = mh.hydrodynamic_coefficients_derivative(body, {"wave_frequencies": [om], "radiating_dofs": ["Heave", "Surge"],
                                                         "wave_directions": [0.0]}, F, ctx=ctx, rho=1025.0)
    hi = oracle.hydro_one_frequency(mesh, body.dofs, om + h, rho=1025.0, betas=[0.0], lapack=True, gfs=gfs,
                                    direct=direct)
    lo = oracle.hydro_one_frequency(mesh, body.dofs, om - h, rho=1025.0, betas=[0.0], lapack=True, gfs=gfs,
                                    direct=direct)
    dA, dB, dFd, dFk, dFe = [(a - b) / (2 * h) for a, b in zip(hi, lo)]
    assert close(res["d_added_mass"][:, :, 0, 0], dA, 1e-6)
    assert close(res["d_radiation_damping"][:, :, 0, 0], dB, 1e-6)
    assert close(res["d_diffraction_force"][:, 0, :, 0], dFd, 1e-6)
    assert close(res["d_Froude_Krylov_force"][:, 0, :, 0], dFk, 1e-6)
    assert close(res["d_excitation_force"][:, 0, :, 0], dFe, 1e-6)


def test_derivative_rejects_other_green_functions(mh, ctx):
    body = mh.FloatingBody(mh.hemisphere_mesh(1.0, 4, 8), ["Heave"])
    with pytest.raises(ValueError, match="frequency derivative covers"):
        mh.hydrodynamic_coefficients_derivative(body, {"wave_frequencies": [1.0], "radiating_dofs": ["Heave"]},
                                                mh.DirectBEM("Surrogate"), ctx=ctx)
