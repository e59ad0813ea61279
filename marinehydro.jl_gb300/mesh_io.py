"""Meshes from other programs: Capytaine-style vertex/face arrays and WAMIT GDF files.

The reference takes user meshes as Capytaine's arrays (meshes.jl:113-142): vertices
(nv, 3), 0-based faces (nf, 4) in which a triangle repeats one of its vertices, and the
per-face fields Capytaine computed (``faces_centers``, ``faces_normals``,
``faces_areas``, ``faces_radiuses``); ``Mesh(...)`` keeps the faces 0-based and
``StaticArraysMesh(mesh::PyObject)`` adds 1 (meshes.jl:127-140).  Here the same arrays
(or any object carrying Capytaine's attribute names) become a ``StaticArraysMesh``
without Python Capytaine; where the per-face fields are not given they are derived from
the vertices with the reference's own formulas (meshes.jl:461-489).

GDF is WAMIT's low-order panel format, which most marine meshers write: a title line,
``ULEN GRAV``, ``ISX ISY`` (geometric symmetry about x = 0 and y = 0: only the part with
x >= 0 / y >= 0 is stored), ``NPAN``, then 4 vertices (12 numbers) per panel in any
line layout, ordered so that the normal by the right-hand rule points into the fluid.
Panels carry their own corners, so vertices shared by panels are merged on exact
coordinate equality when the file is read.
"""
from __future__ import annotations

import numpy as np

from .meshes import StaticArraysMesh, face_fields


def _pad_faces(faces) -> np.ndarray:
    f = np.asarray(faces)
    if f.ndim != 2 or f.shape[1] not in (3, 4):
        raise ValueError(f"faces must have shape (nfaces, 3) or (nfaces, 4), got {f.shape}")
    if not np.issubdtype(f.dtype, np.integer):
        if not np.all(f == np.round(f)):
            raise ValueError("faces must hold integer vertex indices")
        f = f.astype(np.int64)
    if f.shape[1] == 3:  # a triangle repeats its last vertex
        f = np.concatenate([f, f[:, 2:3]], axis=1)
    return f.astype(np.int64)


def mesh_from_arrays(vertices, faces, index_base: int = 0, centers=None, normals=None, areas=None,
                     radii=None) -> StaticArraysMesh:
    """A mesh from vertex/face arrays.

    ``faces`` (nf, 4) or (nf, 3) index ``vertices`` (nv, 3) from ``index_base`` (0 for
    Capytaine's arrays and the reference's ``Mesh``, 1 for its ``StaticArraysMesh``); a
    triangle is a quad with a repeated vertex, or a 3-index face.  The corner order is
    kept as given (the Birk panel integral skips zero-length edges wherever they are).
    Per-face fields not given are derived from the vertices (meshes.jl:461-489); a face
    whose first three corners span no area has no normal and is rejected.
    """
    if index_base not in (0, 1):
        raise ValueError("index_base must be 0 or 1")
    V = np.asarray(vertices, dtype=np.float64)
    if V.ndim != 2 or V.shape[1] != 3:
        raise ValueError(f"vertices must have shape (nvertices, 3), got {V.shape}")
    if not np.all(np.isfinite(V)):
        raise ValueError("vertices must be finite")
    F0 = _pad_faces(faces) - index_base
    if F0.size and (F0.min() < 0 or F0.max() >= len(V)):
        raise ValueError(f"face indices out of range for {len(V)} vertices with index_base={index_base}")
    if centers is None or normals is None or areas is None or radii is None:
        a, b, c = V[F0[:, 0]], V[F0[:, 1]], V[F0[:, 2]]
        bad = np.linalg.norm(np.cross(b - a, c - a), axis=1) == 0.0
        if np.any(bad):
            raise ValueError(f"faces {np.flatnonzero(bad)[:8].tolist()} have no normal: their first three corners "
                             "span no area (put a triangle's repeated vertex last)")
        c_, n_, a_, r_ = face_fields(V, F0)
        centers = c_ if centers is None else centers
        normals = n_ if normals is None else normals
        areas = a_ if areas is None else areas
        radii = r_ if radii is None else radii
    return StaticArraysMesh(V, F0 + 1, centers, normals, areas, radii)


def mesh_from_capytaine(mesh) -> StaticArraysMesh:
    """``StaticArraysMesh(mesh::PyObject)`` (meshes.jl:127-140) for any object with Capytaine's
    attributes: ``vertices``, 0-based ``faces`` and, when present, ``faces_centers``,
    ``faces_normals``, ``faces_areas``, ``faces_radiuses`` (used as given)."""
    get = lambda name: (np.asarray(getattr(mesh, name)) if getattr(mesh, name, None) is not None else None)
    return mesh_from_arrays(get("vertices"), get("faces"), 0, get("faces_centers"), get("faces_normals"),
                            get("faces_areas"), get("faces_radiuses"))


def _merge_vertices(corners: np.ndarray):
    """(np, 4, 3) corners -> (vertices, 0-based faces), merging exactly equal coordinates."""
    flat = corners.reshape(-1, 3)
    verts, inv = np.unique(flat, axis=0, return_inverse=True)
    return verts, inv.reshape(-1, 4)


def _mirrored(P: np.ndarray, axis: int) -> np.ndarray:
    """Mirror images of panels (np, 4, 3) in the plane x_axis = 0, with the corner order reversed
    so that the normal still points into the fluid.  A triangle (a quad with a repeated
    corner) is rotated so that its first three corners are distinct."""
    M = P.copy()
    M[:, :, axis] *= -1.0
    M = M[:, [0, 3, 2, 1]]
    for rot in range(4):
        a, b, c = M[:, 0], M[:, 1], M[:, 2]
        bad = np.linalg.norm(np.cross(b - a, c - a), axis=1) == 0.0
        if not bad.any():
            break
        M[bad] = M[bad][:, [1, 2, 3, 0]]
    return M


def read_gdf(path) -> StaticArraysMesh:
    """Read a WAMIT GDF file (low-order panels), expanding its x = 0 / y = 0 symmetries."""
    with open(path) as f:
        lines = f.read().splitlines()
    if len(lines) < 4:
        raise ValueError(f"{path}: a GDF file has a title line, ULEN GRAV, ISX ISY and NPAN before the panels")
    try:
        ulen = float(lines[1].split()[0])
        isx, isy = (int(x) for x in lines[2].split()[:2])
        npan = int(lines[3].split()[0])
        nums = np.array([float(x) for ln in lines[4:] for x in ln.replace(",", " ").split()], dtype=np.float64)
    except (IndexError, ValueError) as exc:
        raise ValueError(f"{path}: malformed GDF header or panel data ({exc})") from None
    if npan < 1 or nums.size < 12 * npan:
        raise ValueError(f"{path}: NPAN = {npan} needs {12 * npan} panel coordinates, found {nums.size}")
    if ulen <= 0:
        raise ValueError(f"{path}: ULEN must be positive")
    corners = nums[:12 * npan].reshape(npan, 4, 3)
    if isx == 1:
        corners = np.concatenate([corners, _mirrored(corners, 0)])
    if isy == 1:
        corners = np.concatenate([corners, _mirrored(corners, 1)])
    V, F0 = _merge_vertices(corners)
    return mesh_from_arrays(V, F0, 0)


def write_gdf(path, mesh: StaticArraysMesh, ulen: float = 1.0, grav: float = 9.81,
              title: str = "MarineHydro GB300 mesh") -> None:
    """Write every panel of `mesh` (no symmetry) as a WAMIT GDF file; values in full precision."""
    P = mesh.panel_vertices
    with open(path, "w") as f:
        f.write(f"{title}\n{float(ulen)!r} {float(grav)!r}\n0 0\n{len(P)}\n")
        for panel in P:
            for v in panel:
                f.write(" ".join(repr(float(x)) for x in v) + "\n")
