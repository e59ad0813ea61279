"""face_fields_jacobian (complex step through meshes.face_fields) against central
differences of face_fields itself: the chain from panel fields to vertices that the
reverse-mode gradient uses."""
import numpy as np


def _fd_columns(mh, mesh, h=1e-6):
    """Directional derivatives of (centers, normals, areas) along random vertex moves,
    by central differences of face_fields, and the same from the Jacobian."""
    rng = np.random.default_rng(3)
    faces0 = mesh.faces - 1
    dC, dN, dA = mh.face_fields_jacobian(mesh.panel_vertices)
    out = []
    for _ in range(3):
        dV = rng.standard_normal(mesh.vertices.shape)
        cp, npl, ap, _ = mh.face_fields(mesh.vertices + h * dV, faces0)
        cm, nm, am, _ = mh.face_fields(mesh.vertices - h * dV, faces0)
        d12 = dV[faces0].reshape(-1, 12)
        out.append(((cp - cm) / (2 * h), np.einsum("ikq,iq->ik", dC, d12)))
        out.append(((npl - nm) / (2 * h), np.einsum("ikq,iq->ik", dN, d12)))
        out.append(((ap - am) / (2 * h), np.einsum("iq,iq->i", dA, d12)))
    return out


def test_jacobian_quads_and_triangles(mh):
    # the hemisphere has a ring of triangles (repeated last vertex) at the pole
    for mesh in (mh.hemisphere_mesh(1.3, 5, 8), mh.vertical_cylinder_mesh(2.0, 3.0, 8, 3, 2)):
        for fd, jac in _fd_columns(mh, mesh):
            assert np.abs(fd - jac).max() <= 1e-7 * max(1.0, np.abs(jac).max())


def test_rotation_metadata_follows_combination(mh):
    a = mh.FloatingBody(mh.vertical_cylinder_mesh(1.0, 2.0, 6, 2, 1), ["Heave", "Pitch"], rotation_center=(0, 0, -1),
                        body_name="a")
    b = mh.FloatingBody(mh.vertical_cylinder_mesh(1.0, 2.0, 6, 2, 1, center=(5.0, 0.0)), ["Yaw"], body_name="b")
    c = a + b
    na = a.mesh.nfaces
    assert c.rotations == {"a__Pitch": (1, (0.0, 0.0, -1.0), 0, na), "b__Yaw": (2, (0.0, 0.0, 0.0), na, c.mesh.nfaces)}
