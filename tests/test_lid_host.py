"""Irregular-frequency lid: host logic and the oracle's lid restatement (CPU only).

The reference checks its lid method against Capytaine (test/irregular_frequency_removal.jl,
rtol 0.3), which cannot run here.  The oracle's hull + lid solve is pinned instead by the
physics the lid exists for: a truncated vertical cylinder of radius a and draft T has its
first irregular frequency at the wavenumber K = (j01/a) coth(j01 T/a), j01 = 2.4048 the first
zero of J0 (the interior Dirichlet eigenmode J0(j01 r/a) sinh(j01 (z+T)/a) meets the
free-surface condition there); without a lid the heave coefficients spike at that frequency,
with a lid below the free surface they do not.
"""
import numpy as np
import pytest


def _cylinder_with_lid(mh, up=True):
    hull = mh.vertical_cylinder_mesh(1.0, 1.0, n_theta=24, n_z=8, n_r=5)
    lid = mh.disc_lid_mesh(1.0, -0.15, n_theta=24, n_r=5, normal_up=up)
    return hull, lid


def test_lid_mesher_geometry(mh):
    _, lid = _cylinder_with_lid(mh)
    assert np.allclose(lid.normals, [0.0, 0.0, 1.0])
    assert np.allclose(lid.centers[:, 2], -0.15)
    # the polygonal disc: 24-gon of radius 1
    assert lid.areas.sum() == pytest.approx(0.5 * 24 * np.sin(2 * np.pi / 24), rel=1e-12)
    down = mh.disc_lid_mesh(1.0, -0.15, n_theta=24, n_r=5, normal_up=False)
    assert np.allclose(down.normals, [0.0, 0.0, -1.0])
    assert np.allclose(down.areas, lid.areas)


def test_body_with_lid_host_logic(mh):
    hull, lid = _cylinder_with_lid(mh)
    body = mh.FloatingBody(hull, ["Heave", "Pitch"], body_name="cyl", lid_mesh=lid)
    mesh, n_hull = body.mesh_including_lid()
    assert n_hull == hull.nfaces and mesh.nfaces == hull.nfaces + lid.nfaces
    assert np.array_equal(mesh.centers[:n_hull], hull.centers)
    assert np.array_equal(mesh.centers[n_hull:], lid.centers)
    assert mesh.n_hull == n_hull
    d = body.padded_dof_array(["Heave", "Pitch"])
    assert d.shape == (2, mesh.nfaces, 3)
    assert np.array_equal(d[:, :n_hull], body.dof_array(["Heave", "Pitch"]))
    assert not d[:, n_hull:].any()
    # no lid: the hull itself
    plain = mh.FloatingBody(hull, ["Heave"])
    assert plain.mesh_including_lid() == (hull, hull.nfaces)
    # combine_floatingbodies keeps the lids (bodies.jl:205-209)
    both = mh.combine_floatingbodies([body, body])
    assert both.lid_mesh.nfaces == 2 * lid.nfaces
    assert mh.combine_floatingbodies([plain, plain]).lid_mesh is None
    with pytest.raises(ValueError, match="hydro_gradient does not cover bodies with a lid"):
        mh.hydro_gradient(body, [1.0], ["Heave"])


def test_lid_at_the_free_surface_is_rejected(mh):
    hull = mh.vertical_cylinder_mesh(1.0, 1.0, n_theta=12, n_z=4, n_r=3)
    surface_lid = mh.disc_lid_mesh(1.0, 0.0, n_theta=12, n_r=3)
    with pytest.raises(ValueError, match="below the free surface"):
        mh.FloatingBody(hull, ["Heave"], lid_mesh=surface_lid)


def test_oracle_lid_removes_the_irregular_frequency(oracle, mh):
    """Heave A and B at 4.8, 4.9, 5.0 rad/s; the first irregular frequency of this
    cylinder (a = T = 1 m) is at k = 2.4048 coth(2.4048) m^-1, omega = 4.90 rad/s."""
    hull, lid = _cylinder_with_lid(mh)
    body = mh.FloatingBody(hull, ["Heave"])
    k_irr = 2.404825557695773 / np.tanh(2.404825557695773)
    assert np.sqrt(9.81 * k_irr) == pytest.approx(4.90, abs=0.01)
    oms = [4.8, 4.9, 5.0]
    curves = {}
    for name, lm in (("none", None), ("lid", lid)):
        A, B = [], []
        for om in oms:
            a, b, *_ = oracle.hydro_one_frequency(hull, body.dofs, om, rho=1025.0, lapack=True, lid_mesh=lm)
            A.append(a[0, 0])
            B.append(b[0, 0])
        curves[name] = (np.array(A), np.array(B))
    bump = lambda y: abs(y[1] - 0.5 * (y[0] + y[2]))
    A0, B0 = curves["none"]
    A1, B1 = curves["lid"]
    assert bump(A0) > 0.02 * abs(A0[1]) and bump(B0) > 1.0 * abs(B0[1]) * 0.5
    assert bump(A1) < 1e-3 * abs(A1[1]) and bump(B1) < 0.05 * abs(B1[1])
    # away from the spike the lid changes the coefficients only by the discretisation
    assert abs(A1[0] - A0[0]) < 0.01 * abs(A0[0])
