"""Arrays of bodies (combine_floatingbodies, bodies.jl:165-225) through the GPU sweep.

The reference's two-body test (test/consistency_with_Capytaine.jl:300-423) compares a
combined body's 12 x 12 coefficients with Capytaine at rtol 0.1; here the combined
body's sweep matches the CPU oracle at 1e-8, interaction terms included, and a batch of
two arrays matches their separate sweeps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DOFS = ["Surge", "Sway", "Heave", "Roll", "Pitch", "Yaw"]


def _array(mh, sep):
    m1 = mh.vertical_cylinder_mesh(1.0, 2.0, 16, 5, 3)
    m2 = mh.vertical_cylinder_mesh(1.0, 2.0, 16, 5, 3, center=(sep, 1.0))
    b1 = mh.FloatingBody(m1, DOFS, rotation_center=(0.0, 0.0, -1.0), body_name="cyl")
    b2 = mh.FloatingBody(m2, DOFS, rotation_center=(sep + 1.0, 1.0, 0.0), body_name="cyl")
    return b1 + b2


def test_two_body_array_matches_oracle(mh, oracle, ctx):
    body = _array(mh, 5.0)
    names = list(body.dofs)
    assert len(names) == 12
    oms = [0.8, 1.6]
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": names,
                                              "wave_directions": [0.0, 0.7]}, ctx=ctx, rho=1025.0)
    assert res["added_mass"].shape == (12, 12, 2, 1)
    for w, om in enumerate(oms):
        A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(body.mesh, body.dofs, om, rho=1025.0, betas=[0.0, 0.7])
        for got, ref in ((res["added_mass"][:, :, w, 0], A), (res["radiation_damping"][:, :, w, 0], B),
                         (res["excitation_force"][:, w, :, 0], Fe)):
            assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max()
    # the bodies interact: heave of body 2 is felt by body 1
    a = res["added_mass"][:, :, 0, 0]
    assert abs(a[names.index("cyl__Heave"), names.index("cyl_2__Heave")]) > 1e-3 * abs(a[2, 2])


def test_batch_of_arrays_matches_separate_sweeps(mh, ctx):
    arrays = [_array(mh, 5.0), _array(mh, 8.0)]
    params = [{"wave_frequencies": [0.9, 1.7], "radiating_dofs": list(arrays[0].dofs)}] * 2
    out = mh.batch_hydrodynamic_coefficients(arrays, params, ctx=ctx, rho=1025.0)
    for b, p, o in zip(arrays, params, out):
        ref = mh.hydrodynamic_coefficients(b, p, ctx=ctx, rho=1025.0)
        assert np.abs(o["added_mass"] - ref["added_mass"]).max() <= 1e-10 * np.abs(ref["added_mass"]).max()
