"""Floating bodies and rigid-body dof fields (bodies.jl)."""
from __future__ import annotations

import numpy as np

from .meshes import StaticArraysMesh, combine_meshes

TRANSLATIONS = ("Surge", "Sway", "Heave")
ROTATIONS = ("Roll", "Pitch", "Yaw")


def translational_dofs(mesh: StaticArraysMesh, name: str) -> np.ndarray:
    """translational_dofs (bodies.jl:74-86): a unit vector on every panel."""
    dof = np.zeros((mesh.nfaces, 3))
    dof[:, TRANSLATIONS.index(name)] = 1.0
    return dof


def rotational_dofs(mesh: StaticArraysMesh, name: str, rotation_center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """rotational_dofs (bodies.jl:103-118): axis x (center_i - rotation_center)."""
    if name not in ROTATIONS:
        raise ValueError(f"unknown rotational dof {name}")
    axis = np.zeros(3)
    axis[ROTATIONS.index(name)] = 1.0
    return np.cross(axis, mesh.centers - np.asarray(rotation_center, dtype=float))


def evaluate_gradient_of_motion(mesh: StaticArraysMesh, name: str) -> np.ndarray:
    """evaluate_gradient_of_motion (bodies.jl:54-66), forward-speed problems only."""
    if name not in TRANSLATIONS + ROTATIONS:
        raise ValueError("forward speed problems are only developed for rigid body dofs")
    d = np.zeros((mesh.nfaces, 3))
    if name == "Pitch":
        d[:, 2] = 1.0
    elif name == "Yaw":
        d[:, 1] = -1.0
    return d


class FloatingBody:
    """FloatingBody (bodies.jl:9-51): mesh, optional lid, named dof fields (n x 3).

    The dof fields live on the hull panels.  A lid (irregular-frequency removal) is a
    mesh of panels inside the body's waterplane, below the free surface; the solve
    runs on hull + lid with zero boundary conditions on the lid (solve.jl:2-28).
    """

    def __init__(self, mesh: StaticArraysMesh, dofs=None, rotation_center=None, body_name: str = "body",
                 lid_mesh=None):
        if lid_mesh is not None and not np.all(np.asarray(lid_mesh.centers)[:, 2] < -1e-8):
            raise ValueError("a lid must lie below the free surface (every lid panel centre at z < -1e-8); "
                             "at z = 0 the wave Green functions are singular at the lid's self pairs")
        self.mesh = mesh
        self.lid_mesh = lid_mesh
        self._with_lid = None
        self.body_name = body_name
        # rigid rotation dofs: name -> (axis index, rotation centre, first panel, end panel); their
        # fields follow the panel centres, which the gradient chain needs
        self.rotations = {}
        if dofs is None:
            dofs = {}
        if isinstance(dofs, dict):
            self.dofs = {str(k): np.ascontiguousarray(np.asarray(v, dtype=float)) for k, v in dofs.items()}
        else:  # rigid dof names
            rc = (0.0, 0.0, 0.0) if rotation_center is None else rotation_center
            self.dofs = {}
            for name in dofs:
                name = str(name)
                self.dofs[name] = (translational_dofs(mesh, name) if name in TRANSLATIONS
                                   else rotational_dofs(mesh, name, rc))
                if name in ROTATIONS:
                    self.rotations[name] = (ROTATIONS.index(name), tuple(float(x) for x in rc), 0, mesh.nfaces)
        for k, v in self.dofs.items():
            if v.shape != (mesh.nfaces, 3):
                raise ValueError(f"dof {k} must have shape ({mesh.nfaces}, 3)")

    def __add__(self, other):
        return combine_floatingbodies([self, other])

    def mesh_including_lid(self):
        """_mesh_including_lid (solve.jl:22-28): (hull + lid mesh, number of hull panels).

        The hull panels come first, so the hull mask is `index < n_hull`; the combined
        mesh carries `n_hull` to its device copy (mh_mesh_set_lid)."""
        if self.lid_mesh is None:
            return self.mesh, self.mesh.nfaces
        if self._with_lid is None:
            m = combine_meshes([self.mesh, self.lid_mesh])
            m.n_hull = self.mesh.nfaces
            self._with_lid = m
        return self._with_lid, self.mesh.nfaces

    def padded_dof_array(self, names=None) -> np.ndarray:
        """dof_array on hull + lid panels: zeros on the lid."""
        d = self.dof_array(names)
        if self.lid_mesh is None or d.size == 0:
            return d
        out = np.zeros((d.shape[0], self.mesh.nfaces + self.lid_mesh.nfaces, 3))
        out[:, :self.mesh.nfaces] = d
        return out

    def dof_array(self, names=None) -> np.ndarray:
        names = list(self.dofs) if names is None else list(names)
        return np.ascontiguousarray(np.stack([self.dofs[n] for n in names])) if names else np.zeros((0, 0, 3))


def _unique_names(names):
    """make_body_name_list_unique (bodies.jl:138-163)."""
    seen, out = {}, []
    for s in names:
        if s not in seen:
            out.append(s)
            seen[s] = 2
        else:
            c = seen[s]
            new = f"{s}_{c}"
            while new in seen or new in names:
                c += 1
                new = f"{s}_{c}"
            out.append(new)
            seen[s] = c + 1
            seen[new] = 1
    return out


def combine_floatingbodies(bodies, new_body_name: str | None = None) -> FloatingBody:
    """combine_floatingbodies (bodies.jl:165-225): one mesh, dofs named body__dof, zero on other bodies."""
    names = _unique_names([b.body_name.replace(" ", "_") for b in bodies])
    mesh = combine_meshes([b.mesh for b in bodies])
    total = mesh.nfaces
    dofs, rotations = {}, {}
    off = 0
    for b, nm in zip(bodies, names):
        for k, v in b.dofs.items():
            d = np.zeros((total, 3))
            d[off:off + b.mesh.nfaces] = v
            dofs[f"{nm}__{k}"] = d
        for k, (ax, rc, p0, p1) in getattr(b, "rotations", {}).items():
            rotations[f"{nm}__{k}"] = (ax, rc, off + p0, off + p1)
        off += b.mesh.nfaces
    lids = [b.lid_mesh for b in bodies if b.lid_mesh is not None]  # bodies.jl:205-209
    out = FloatingBody(mesh, dofs, body_name=new_body_name or "+".join(names),
                       lid_mesh=combine_meshes(lids) if lids else None)
    out.rotations = rotations
    return out
