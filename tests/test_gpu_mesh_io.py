"""User meshes through the GPU path: a WAMIT GDF file with x = 0 / y = 0 symmetry and
Capytaine-style 0-based vertex/face arrays with 3-index triangles, each solved on the
device and checked against the CPU oracle on the same mesh (S, D at 1e-10, coefficients
at 1e-8)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_SD = 1e-10
REL_COEF = 1e-8


def _check_against_oracle(mh, oracle, ctx, mesh, oms, dofs):
    k = oms[0] ** 2 / 9.81
    S, D = mh.assemble_matrices(mh.default_greens_functions("Wu"), mesh, k, ctx=ctx)
    So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_WU)
    assert np.linalg.norm(S - So) <= REL_SD * np.linalg.norm(So)
    assert np.linalg.norm(D - Do) <= REL_SD * np.linalg.norm(Do)
    body = mh.FloatingBody(mesh, dofs, rotation_center=(0.0, 0.0, -0.3), body_name="user")
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": dofs,
                                              "wave_directions": [0.0, 0.6]}, ctx=ctx, rho=1025.0)
    for w, om in enumerate(oms):
        A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(mesh, body.dofs, om, rho=1025.0, betas=[0.0, 0.6])
        for got, ref in ((res["added_mass"][:, :, w, 0], A), (res["radiation_damping"][:, :, w, 0], B),
                         (res["excitation_force"][:, w, :, 0], Fe)):
            assert np.abs(got - ref).max() <= REL_COEF * np.abs(ref).max()


def test_gdf_with_symmetry_matches_oracle(mh, oracle, ctx, tmp_path):
    full = mh.hemisphere_mesh(1.0, 6, 16)
    P = full.panel_vertices
    quarter = P[np.all(P[:, :, 0] >= -1e-15, axis=1) & np.all(P[:, :, 1] >= -1e-15, axis=1)]
    path = tmp_path / "quarter_sphere.gdf"
    with open(path, "w") as f:
        f.write("quarter of a floating hemisphere\n1.0 9.81\n1 1\n%d\n" % len(quarter))
        for panel in quarter:
            for v in panel:
                f.write(" ".join(repr(float(x)) for x in v) + "\n")
    mesh = mh.read_gdf(path)
    assert mesh.nfaces == full.nfaces
    _check_against_oracle(mh, oracle, ctx, mesh, [0.7, 1.5], ["Surge", "Heave", "Pitch"])


def test_capytaine_arrays_with_triangles_match_oracle(mh, oracle, ctx):
    m = mh.vertical_cylinder_mesh(1.2, 2.0, 14, 5, 3)
    faces0 = m.faces - 1
    tri = faces0[:, 2] == faces0[:, 3]
    assert tri.any()
    # quads as 4 indices; the bottom's centre fan as 3-index triangles, listed separately
    V = m.vertices
    quads = mh.mesh_from_arrays(V, faces0[~tri])
    tris = mh.mesh_from_arrays(V, faces0[tri][:, :3])
    mesh = mh.combine_meshes([quads, tris])
    _check_against_oracle(mh, oracle, ctx, mesh, [1.1], ["Heave", "Roll"])
