"""combine_floatingbodies / `+` (bodies.jl:138-225): host logic, CPU only."""
import numpy as np


def test_combined_dofs_are_named_and_padded(mh):
    m1 = mh.vertical_cylinder_mesh(1.0, 2.0, 12, 4, 3)
    m2 = mh.vertical_cylinder_mesh(1.0, 2.0, 12, 4, 3, center=(6.0, 0.0))
    b1 = mh.FloatingBody(m1, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, -1.0), body_name="float one")
    b2 = mh.FloatingBody(m2, ["Heave", "Pitch"], rotation_center=(6.0, 0.0, -1.0), body_name="float one")
    both = b1 + b2
    assert list(both.dofs) == ["float_one__Heave", "float_one__Pitch", "float_one_2__Heave", "float_one_2__Pitch"]
    assert both.body_name == "float_one+float_one_2"
    n1 = m1.nfaces
    assert both.mesh.nfaces == n1 + m2.nfaces
    assert np.array_equal(both.dofs["float_one__Pitch"][:n1], b1.dofs["Pitch"])
    assert not both.dofs["float_one__Pitch"][n1:].any()
    assert np.array_equal(both.dofs["float_one_2__Heave"][n1:], b2.dofs["Heave"])
    assert not both.dofs["float_one_2__Heave"][:n1].any()
    # faces of the second mesh are offset by the first mesh's vertex count (meshes.jl:79-81)
    assert both.mesh.faces[n1:].min() == m1.nvertices + 1
    assert np.array_equal(both.mesh.centers[n1:], m2.centers)
