"""Size-independent physical properties of the GPU sweep at full size (no oracle needed):

* Haskind's relation in deep water, B_jj = k omega / (4 pi rho g^2) * integral over the
  headings of |X_j(beta)|^2 (X the excitation force per unit wave amplitude): it ties the
  radiation solve to the diffraction solve and the Froude-Krylov force.  For an
  axisymmetric body, heave: B_33 = k omega |X_3|^2 / (2 rho g^2); surge:
  B_11 = k omega |X_1(0)|^2 / (4 rho g^2).
* Reciprocity: the added-mass and damping matrices are symmetric.
Both hold for the continuous problem; the panel method meets them to its discretisation
error.  Measured on a GB300 with these meshes: Haskind to 0.3 % on the cylinder up to
omega = 1.3 rad/s and to 0.5 % on the barge at 0.9-1.2 rad/s (1.5-2 % where the damping
itself is small: heave of the deep cylinder at 1.6 rad/s, roll of the barge), symmetry
to 0.23 %.  The tolerances below leave a factor of about two.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHO, G = 1025.0, 9.81


def test_haskind_on_the_2000_panel_cylinder(mh, ctx):
    mesh = mh.config2_cylinder()
    assert mesh.nfaces == 2000
    body = mh.FloatingBody(mesh, ["Surge", "Heave"])
    oms = [0.5, 0.8, 1.1]
    r = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": ["Surge", "Heave"],
                                            "wave_directions": [0.0]}, ctx=ctx, rho=RHO, g=G)
    for w, om in enumerate(oms):
        k = om * om / G
        B = r["radiation_damping"][:, :, w, 0]
        X = r["excitation_force"][:, w, 0, 0]
        heave = k * om * abs(X[1]) ** 2 / (2 * RHO * G * G)
        surge = k * om * abs(X[0]) ** 2 / (4 * RHO * G * G)
        assert heave == pytest.approx(B[1, 1], rel=0.006), om
        assert surge == pytest.approx(B[0, 0], rel=0.006), om


def test_haskind_and_reciprocity_on_a_barge(mh, ctx):
    mesh = mh.barge_mesh(20.0, 8.0, 4.0, 40, 16, 8)
    dofs = ["Surge", "Sway", "Heave", "Roll", "Pitch", "Yaw"]
    body = mh.FloatingBody(mesh, dofs, rotation_center=(0.0, 0.0, -1.0))
    betas = np.linspace(0.0, 2 * np.pi, 36, endpoint=False)
    oms = [0.9, 1.2]
    r = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": dofs,
                                            "wave_directions": list(betas)}, ctx=ctx, rho=RHO, g=G)
    for w, om in enumerate(oms):
        k = om * om / G
        A = r["added_mass"][:, :, w, 0]
        B = r["radiation_damping"][:, :, w, 0]
        X = r["excitation_force"][:, w, :, 0]
        for j in (0, 1, 2, 4, 5):  # surge, sway, heave, pitch, yaw
            haskind = k * om / (4 * np.pi * RHO * G * G) * np.mean(np.abs(X[j]) ** 2) * 2 * np.pi
            assert haskind == pytest.approx(B[j, j], rel=0.01), (om, dofs[j])
        assert np.abs(A - A.T).max() <= 0.005 * np.abs(A).max()
        assert np.abs(B - B.T).max() <= 0.005 * np.abs(B).max()
