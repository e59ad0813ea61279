"""Panel meshes (the reference's StaticArraysMesh / Mesh data layout) and synthetic meshers.

``StaticArraysMesh`` mirrors meshes.jl:42-51: vertices, 1-based quad faces (a
triangle repeats its last vertex), and per-face centers, normals, areas, radii.
``Mesh`` (meshes.jl:12-40) is the same data with 0-based faces.  Derived face
fields follow meshes.jl:461-489: the center is the area-weighted centroid of the
triangles (a,b,c) and (a,c,d), the normal is normalize((b-a) x (c-a)), the radius
is |a - center| and the area is the sum of the two triangle areas.

The meshers build the bodies of the benchmark configurations (lat-long
hemispheres, truncated vertical cylinders, rectangular barges, seeded random
bodies), all with outward normals (into the fluid) and vertices below z = 0.
They replace the reference's Capytaine loaders (meshes.jl:113-142), which need
Python Capytaine through PyCall.
"""
from __future__ import annotations

import numpy as np


class StaticArraysMesh:
    """Panel mesh; ``faces`` are 1-based (Julia convention), shape (nfaces, 4)."""

    def __init__(self, vertices, faces, centers=None, normals=None, areas=None, radii=None):
        self.vertices = np.ascontiguousarray(np.asarray(vertices, dtype=np.float64).reshape(-1, 3))
        self.faces = np.ascontiguousarray(np.asarray(faces, dtype=np.int64).reshape(-1, 4))
        if self.faces.size and (self.faces.min() < 1 or self.faces.max() > len(self.vertices)):
            raise ValueError("faces must hold 1-based vertex indices")
        if centers is None or normals is None or areas is None or radii is None:
            c, n, a, r = face_fields(self.vertices, self.faces - 1)
            centers = c if centers is None else centers
            normals = n if normals is None else normals
            areas = a if areas is None else areas
            radii = r if radii is None else radii
        self.centers = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
        self.normals = np.ascontiguousarray(np.asarray(normals, dtype=np.float64).reshape(-1, 3))
        self.areas = np.ascontiguousarray(np.asarray(areas, dtype=np.float64).reshape(-1))
        self.radii = np.ascontiguousarray(np.asarray(radii, dtype=np.float64).reshape(-1))
        nf = len(self.faces)
        for name, arr, shape in (("centers", self.centers, (nf, 3)), ("normals", self.normals, (nf, 3)),
                                 ("areas", self.areas, (nf,)), ("radii", self.radii, (nf,))):
            if arr.shape != shape:
                raise ValueError(f"{name} must have shape {shape}, got {arr.shape}")
        self._handles = {}

    @property
    def nfaces(self) -> int:
        return len(self.faces)

    @property
    def nvertices(self) -> int:
        return len(self.vertices)

    @property
    def panel_vertices(self) -> np.ndarray:
        """(nfaces, 4, 3) gathered corners, the layout the C-ABI takes."""
        return np.ascontiguousarray(self.vertices[self.faces - 1])

    def __add__(self, other):
        return combine_meshes([self, other])

    def device_mesh(self, ctx):
        """The mh_mesh handle of this mesh on context `ctx` (uploaded once)."""
        from ._device import DeviceMesh

        h = self._handles.get(id(ctx))
        if h is None:
            h = DeviceMesh(ctx, self, getattr(self, "n_hull", None))
            self._handles[id(ctx)] = h
        return h


def Mesh(vertices, faces0, centers=None, normals=None, areas=None, radii=None) -> StaticArraysMesh:
    """Dense-`Mesh` constructor (0-based faces, meshes.jl:12-40) -> StaticArraysMesh."""
    return StaticArraysMesh(vertices, np.asarray(faces0) + 1, centers, normals, areas, radii)


def smesh(mesh: StaticArraysMesh) -> StaticArraysMesh:
    return mesh


def face_fields(vertices: np.ndarray, faces0: np.ndarray):
    """Center, normal, area, radius per face (meshes.jl:461-489)."""
    a = vertices[faces0[:, 0]]
    b = vertices[faces0[:, 1]]
    c = vertices[faces0[:, 2]]
    d = vertices[faces0[:, 3]]
    area1 = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    area2 = 0.5 * np.linalg.norm(np.cross(c - a, d - a), axis=1)
    c1 = (a + b + c) / 3
    c2 = (a + c + d) / 3
    center = (c1 * area1[:, None] + c2 * area2[:, None]) / (area1 + area2)[:, None]
    nrm = np.cross(b - a, c - a)
    nrm = nrm / np.linalg.norm(nrm, axis=1)[:, None]
    radius = np.linalg.norm(a - center, axis=1)
    return center, nrm, area1 + area2, radius


def _corner_fields(a, b, c, d, degenerate2):
    """face_fields on corner arrays, written with analytic operations only (no abs), so
    that a complex step through it differentiates it.  A triangle stored as a quad
    (c == d) has a second triangle of area 0 whatever the shared vertex does: such
    panels (``degenerate2``) keep area2 = 0 instead of differentiating |0|."""
    def norm(x):
        return np.sqrt(np.sum(x * x, axis=-1))
    nrm = np.cross(b - a, c - a)
    area1 = 0.5 * norm(nrm)
    area2 = np.where(degenerate2, 0.0, 0.5 * norm(np.cross(c - a, d - a)))
    center = (((a + b + c) / 3) * area1[:, None] + ((a + c + d) / 3) * area2[:, None]) / (area1 + area2)[:, None]
    return center, nrm / norm(nrm)[:, None], area1 + area2


def face_fields_jacobian(panel_vertices: np.ndarray, step: float = 1e-30):
    """Jacobians of (center, normal, area) w.r.t. the 12 corner coordinates of each panel
    (corner q, axis x -> column 3q + x), by complex step: exact to rounding.
    Returns dC (n,3,12), dN (n,3,12), dA (n,12)."""
    V = np.asarray(panel_vertices, dtype=np.float64)
    n = V.shape[0]
    dC = np.empty((n, 3, 12))
    dN = np.empty((n, 3, 12))
    dA = np.empty((n, 12))
    deg2 = np.all(np.cross(V[:, 2] - V[:, 0], V[:, 3] - V[:, 0]) == 0.0, axis=-1)
    for col in range(12):
        Vc = V.astype(np.complex128)
        Vc[:, col // 3, col % 3] += 1j * step
        c, nv, ar = _corner_fields(Vc[:, 0], Vc[:, 1], Vc[:, 2], Vc[:, 3], deg2)
        dC[:, :, col] = c.imag / step
        dN[:, :, col] = nv.imag / step
        dA[:, col] = ar.imag / step
    return dC, dN, dA


def combine_meshes(meshes) -> StaticArraysMesh:
    """combine_meshes (meshes.jl:56-92): concatenate, offsetting face indices."""
    verts, faces, cs, ns, as_, rs = [], [], [], [], [], []
    off = 0
    for m in meshes:
        verts.append(m.vertices)
        faces.append(m.faces + off)
        off += m.nvertices
        cs.append(m.centers)
        ns.append(m.normals)
        as_.append(m.areas)
        rs.append(m.radii)
    return StaticArraysMesh(np.concatenate(verts), np.concatenate(faces), np.concatenate(cs), np.concatenate(ns),
                            np.concatenate(as_), np.concatenate(rs))


# ---------------------------------------------------------------------------
# structured meshers
# ---------------------------------------------------------------------------
def _assemble(vert_list, quad_list) -> StaticArraysMesh:
    V = np.asarray(vert_list, dtype=np.float64)
    F = np.asarray(quad_list, dtype=np.int64) + 1
    return StaticArraysMesh(V, F)


def _ring_strip(rows, closed=True):
    """Quads between successive rows of vertex indices.  rows[p] is a list of
    indices (a single index = apex).  Corner order (p,q), (p+1,q), (p+1,q+1),
    (p,q+1); a strip meeting an apex becomes the triangle (a, apex, d, d)."""
    quads = []
    for p in range(len(rows) - 1):
        r0, r1 = rows[p], rows[p + 1]
        m = max(len(r0), len(r1))
        for q in range(m):
            qn = (q + 1) % m if closed else q + 1
            if not closed and q == m - 1:
                break
            if len(r1) == 1:
                quads.append((r0[q], r1[0], r0[qn], r0[qn]))
            elif len(r0) == 1:
                quads.append((r0[0], r1[q], r1[qn], r1[qn]))
            else:
                quads.append((r0[q], r1[q], r1[qn], r0[qn]))
    return quads


def hemisphere_mesh(radius=1.0, n_lat=10, n_lon=20, center=(0.0, 0.0, 0.0)) -> StaticArraysMesh:
    """Immersed half of a sphere centred at z=0: n_lat polar bands uniform in polar
    angle from the equator to the south pole, n_lon azimuthal bands.  The pole
    ring is triangles (repeated last vertex)."""
    cx, cy, cz = center
    verts = []
    rows = []
    for p in range(n_lat + 1):
        phi = p * (np.pi / 2) / n_lat
        if p == n_lat:
            rows.append([len(verts)])
            verts.append((cx, cy, cz - radius))
            continue
        row = []
        for q in range(n_lon):
            th = q * 2 * np.pi / n_lon
            row.append(len(verts))
            verts.append((cx + radius * np.cos(phi) * np.cos(th), cy + radius * np.cos(phi) * np.sin(th),
                          cz - radius * np.sin(phi)))
        rows.append(row)
    return _assemble(verts, _ring_strip(rows))


def vertical_cylinder_mesh(radius=5.0, draft=10.0, n_theta=40, n_z=40, n_r=10, center=(0.0, 0.0)) -> StaticArraysMesh:
    """Truncated vertical cylinder: side n_theta x n_z quads, flat bottom as an
    n_r-ring polar grid with an n_theta-triangle centre fan."""
    cx, cy = center
    verts = []
    rows = []
    for p in range(n_z + 1):
        z = -draft * p / n_z
        row = []
        for q in range(n_theta):
            th = q * 2 * np.pi / n_theta
            row.append(len(verts))
            verts.append((cx + radius * np.cos(th), cy + radius * np.sin(th), z))
        rows.append(row)
    quads = _ring_strip(rows)
    # bottom: rings from the rim inwards, then the centre point
    brows = [rows[-1]]
    for m in range(1, n_r):
        rr = radius * (n_r - m) / n_r
        row = []
        for q in range(n_theta):
            th = q * 2 * np.pi / n_theta
            row.append(len(verts))
            verts.append((cx + rr * np.cos(th), cy + rr * np.sin(th), -draft))
        brows.append(row)
    brows.append([len(verts)])
    verts.append((cx, cy, -draft))
    quads += _ring_strip(brows)
    return _assemble(verts, quads)


def disc_lid_mesh(radius=5.0, z=-0.5, n_theta=40, n_r=10, center=(0.0, 0.0), normal_up=True) -> StaticArraysMesh:
    """Horizontal disc at height z (below the free surface) for the lid of a vertical
    cylinder's irregular-frequency removal: an n_r-ring polar grid with an n_theta-triangle
    centre fan, normals +z (normal_up) or -z."""
    cx, cy = center
    verts = []
    rows = []
    for m in range(n_r):
        rr = radius * (n_r - m) / n_r
        row = []
        for q in range(n_theta):
            th = q * 2 * np.pi / n_theta
            row.append(len(verts))
            verts.append((cx + rr * np.cos(th), cy + rr * np.sin(th), z))
        rows.append(row)
    rows.append([len(verts)])
    verts.append((cx, cy, z))
    quads = _ring_strip(rows)  # rim inwards, counter-clockwise from above: normals -z
    if normal_up:
        quads = [(a, c, b, b) if c == d else (a, d, c, b) for a, b, c, d in quads]
    return _assemble(verts, quads)


def _rect(verts, quads, origin, u, v, nu, nv):
    """Grid on the parallelogram origin + s u + t v (normal along u x v)."""
    o = np.asarray(origin, float)
    u = np.asarray(u, float)
    v = np.asarray(v, float)
    base = len(verts)
    for i in range(nu + 1):
        for j in range(nv + 1):
            verts.append(tuple(o + u * (i / nu) + v * (j / nv)))
    idx = lambda i, j: base + i * (nv + 1) + j
    for i in range(nu):
        for j in range(nv):
            quads.append((idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)))


def barge_mesh(length=100.0, beam=20.0, draft=10.0, nl=40, nb=8, nd=4) -> StaticArraysMesh:
    """Rectangular barge [-L/2, L/2] x [-B/2, B/2] x [-T, 0]: bottom nl x nb,
    long sides nl x nd, ends nb x nd, outward normals."""
    L, B, T = length, beam, draft
    verts, quads = [], []
    _rect(verts, quads, (-L / 2, B / 2, -T), (L, 0, 0), (0, -B, 0), nl, nb)   # bottom, -z
    _rect(verts, quads, (-L / 2, B / 2, -T), (0, 0, T), (L, 0, 0), nd, nl)    # y = +B/2, +y
    _rect(verts, quads, (-L / 2, -B / 2, -T), (L, 0, 0), (0, 0, T), nl, nd)   # y = -B/2, -y
    _rect(verts, quads, (L / 2, -B / 2, -T), (0, B, 0), (0, 0, T), nb, nd)    # x = +L/2, +x
    _rect(verts, quads, (-L / 2, -B / 2, -T), (0, 0, T), (0, B, 0), nd, nb)   # x = -L/2, -x
    return _assemble(verts, quads)


def barge_resolution(length, beam, draft, target):
    """(nl, nb, nd) with near-square panels and a panel count close to `target`."""
    best = None
    area = length * beam + 2 * length * draft + 2 * beam * draft
    h0 = np.sqrt(area / target)
    for scale in np.linspace(0.7, 1.4, 141):
        h = h0 * scale
        nl = max(1, int(round(length / h)))
        nb = max(1, int(round(beam / h)))
        nd = max(1, int(round(draft / h)))
        n = nl * nb + 2 * nl * nd + 2 * nb * nd
        err = abs(n - target)
        if best is None or err < best[0]:
            best = (err, nl, nb, nd)
    return best[1:]


def cylinder_resolution(radius, draft, target):
    """(n_theta, n_z, n_r) with near-square side panels and about `target` panels."""
    best = None
    for nt in range(8, 400, 2):
        h = 2 * np.pi * radius / nt
        nz = max(1, int(round(draft / h)))
        nr = max(1, int(round(radius / h)))
        n = nt * nz + nt * nr
        err = abs(n - target)
        if best is None or err < best[0]:
            best = (err, nt, nz, nr)
    return best[1:]


def hemisphere_resolution(target):
    """(n_lat, n_lon) with n_lon = 2 n_lat (square-ish panels) and about `target` panels."""
    best = None
    for nl in range(2, 200):
        for nlon in (2 * nl, 2 * nl + 2, 2 * nl - 2):
            if nlon < 3:
                continue
            n = nl * nlon
            err = abs(n - target)
            if best is None or err < best[0]:
                best = (err, nl, nlon)
    return best[1:]


def random_body(rng: np.random.Generator, target_n: int):
    """One body of the seeded batching workload: a floating sphere (r in [0.5, 5] m),
    a vertical cylinder or a rectangular barge (L/B in [2, 6]); returns (kind, mesh)."""
    kind = ("sphere", "cylinder", "barge")[int(rng.integers(0, 3))]
    if kind == "sphere":
        r = float(rng.uniform(0.5, 5.0))
        nl, nlon = hemisphere_resolution(target_n)
        return kind, hemisphere_mesh(r, nl, nlon)
    if kind == "cylinder":
        r = float(rng.uniform(0.5, 5.0))
        d = float(rng.uniform(0.5, 2.0)) * r
        nt, nz, nr = cylinder_resolution(r, d, target_n)
        return kind, vertical_cylinder_mesh(r, d, nt, nz, nr)
    B = float(rng.uniform(2.0, 10.0))
    L = float(rng.uniform(2.0, 6.0)) * B
    T = float(rng.uniform(0.3, 0.8)) * B
    nl, nb, nd = barge_resolution(L, B, T, target_n)
    return kind, barge_mesh(L, B, T, nl, nb, nd)


def tiny_static_mesh() -> StaticArraysMesh:
    """The two-panel fixture of the reference's GPU tests (test/gpu.jl:36-57)."""
    vertices = [(-1.0, -1.0, -1.0), (0.0, -1.0, -1.0), (0.0, 0.0, -1.0), (-1.0, 0.0, -1.0), (1.0, -1.0, -1.0),
                (1.0, 0.0, -1.0)]
    faces = [(1, 2, 3, 4), (2, 5, 6, 3)]
    centers = [(-0.5, -0.5, -1.0), (0.5, -0.5, -1.0)]
    normals = [(0.0, 0.0, 1.0), (0.0, 0.0, 1.0)]
    return StaticArraysMesh(vertices, faces, centers, normals, [1.0, 1.0], [np.sqrt(0.5), np.sqrt(0.5)])


def config1_hemisphere() -> StaticArraysMesh:
    """200-panel immersed hemisphere, radius 1 m (10 latitude x 20 longitude bands)."""
    return hemisphere_mesh(1.0, 10, 20)


def config2_cylinder() -> StaticArraysMesh:
    """2000-panel truncated cylinder r = 5 m, draft 10 m (side 40 x 40, bottom 10 x 40)."""
    return vertical_cylinder_mesh(5.0, 10.0, 40, 40, 10)
