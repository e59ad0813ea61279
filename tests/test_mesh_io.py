"""Mesh interop on the host: Capytaine-style vertex/face arrays (meshes.jl:113-142) and WAMIT
GDF files, read into the reference's StaticArraysMesh layout (1-based faces, derived fields
by meshes.jl:461-489)."""
import types

import numpy as np
import pytest


def _same_mesh(a, b, tol=0.0):
    for name in ("centers", "normals", "areas", "radii"):
        x, y = getattr(a, name), getattr(b, name)
        assert x.shape == y.shape, name
        assert np.abs(x - y).max() <= tol, name
    assert np.abs(a.panel_vertices - b.panel_vertices).max() <= tol


def test_arrays_zero_and_one_based(mh):
    m = mh.vertical_cylinder_mesh(1.0, 2.0, 8, 3, 2)
    a0 = mh.mesh_from_arrays(m.vertices, m.faces - 1)            # Capytaine / Mesh: 0-based
    a1 = mh.mesh_from_arrays(m.vertices, m.faces, index_base=1)  # StaticArraysMesh: 1-based
    _same_mesh(a0, m)
    _same_mesh(a1, m)
    with pytest.raises(ValueError, match="out of range"):
        mh.mesh_from_arrays(m.vertices, m.faces, index_base=0)  # 1-based indices read as 0-based


def test_triangles_as_three_index_faces_and_repeated_vertices(mh):
    V = np.array([[0.0, 0.0, -1.0], [1.0, 0.0, -1.0], [1.0, 1.0, -1.0], [0.0, 1.0, -1.0]])
    tri3 = mh.mesh_from_arrays(V, [[0, 1, 2], [0, 2, 3]])
    quad = mh.mesh_from_arrays(V, [[0, 1, 2, 2], [0, 2, 3, 3]])
    _same_mesh(tri3, quad)
    assert np.allclose(tri3.areas, [0.5, 0.5])
    assert np.allclose(tri3.centers[0], [2 / 3, 1 / 3, -1.0])
    # Capytaine's triangles may close on their first vertex: same fields
    closed = mh.mesh_from_arrays(V, [[0, 1, 2, 0]])
    assert np.allclose(closed.areas, [0.5]) and np.allclose(closed.centers[0], tri3.centers[0])
    with pytest.raises(ValueError, match="no normal"):
        mh.mesh_from_arrays(V, [[0, 0, 1, 2]])


def test_capytaine_attributes_are_used_as_given(mh):
    m = mh.hemisphere_mesh(1.0, 4, 8)
    obj = types.SimpleNamespace(vertices=m.vertices, faces=m.faces - 1, faces_centers=m.centers + 1e-3,
                                faces_normals=m.normals, faces_areas=m.areas, faces_radiuses=m.radii)
    got = mh.mesh_from_capytaine(obj)
    assert np.array_equal(got.centers, m.centers + 1e-3)  # Capytaine's own fields, not recomputed
    assert np.array_equal(got.faces, m.faces)
    bare = mh.mesh_from_capytaine(types.SimpleNamespace(vertices=m.vertices, faces=m.faces - 1))
    _same_mesh(bare, m)


def test_gdf_round_trip(mh, tmp_path):
    m = mh.barge_mesh(10.0, 4.0, 2.0, 5, 2, 2)
    p = tmp_path / "barge.gdf"
    mh.write_gdf(p, m)
    r = mh.read_gdf(p)
    assert r.nfaces == m.nfaces and r.nvertices == len(np.unique(m.vertices, axis=0))  # equal corners merged
    _same_mesh(r, m)


def test_gdf_symmetry_expands_to_the_full_body(mh, tmp_path):
    full = mh.barge_mesh(8.0, 4.0, 2.0, 4, 2, 2)
    P = full.panel_vertices
    quarter = P[np.all(P[:, :, 0] >= 0, axis=1) & np.all(P[:, :, 1] >= 0, axis=1)]
    p = tmp_path / "quarter.gdf"
    with open(p, "w") as f:
        f.write("quarter barge\n1.0 9.81\n1 1\n%d\n" % len(quarter))
        for panel in quarter:
            f.write(" ".join(repr(float(x)) for x in panel.ravel()) + "\n")  # 12 numbers on one line
    r = mh.read_gdf(p)
    assert r.nfaces == full.nfaces
    key = lambda m: np.lexsort(np.round(m.centers, 12).T)
    for name in ("centers", "normals", "areas", "radii"):
        assert np.allclose(getattr(r, name)[key(r)], getattr(full, name)[key(full)], atol=1e-14), name


def test_gdf_symmetry_with_triangles(mh, tmp_path):
    """A hemisphere (triangles at the pole) stored as the quarter x >= 0, y >= 0."""
    full = mh.hemisphere_mesh(1.0, 4, 8)  # azimuthal bands split at x = 0 and y = 0
    P = full.panel_vertices
    quarter = P[np.all(P[:, :, 0] >= -1e-15, axis=1) & np.all(P[:, :, 1] >= -1e-15, axis=1)]
    p = tmp_path / "q.gdf"
    with open(p, "w") as f:
        f.write("quarter sphere\n1.0 9.81\n1 1\n%d\n" % len(quarter))
        for panel in quarter:
            for v in panel:
                f.write(" ".join(repr(float(x)) for x in v) + "\n")
    r = mh.read_gdf(p)
    assert r.nfaces == full.nfaces
    assert np.isclose(r.areas.sum(), full.areas.sum(), rtol=1e-14)
    assert np.all(np.sum(r.normals * (r.centers - [0, 0, 0]), axis=1) > 0)  # outward everywhere


def test_gdf_rejects_a_short_file(mh, tmp_path):
    p = tmp_path / "bad.gdf"
    p.write_text("t\n1 9.81\n0 0\n2\n0 0 -1 1 0 -1 1 1 -1 0 1 -1\n")
    with pytest.raises(ValueError, match="NPAN"):
        mh.read_gdf(p)
