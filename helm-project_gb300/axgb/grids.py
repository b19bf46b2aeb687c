"""Seeded synthetic grids in the AXIS mesh layout.

Every generator returns a :class:`MeshArrays` holding exactly what
``axis::topology::UnstructuredMesh`` holds (``ax:include/axis/topology/
unstructured_mesh.hpp:68-76``):

* ``node_lonlat``  float64 ``[n_nodes, 2]`` (lon, lat) in degrees,
* ``conn_offsets`` int64 ``[n_cells + 1]`` (CSR offsets),
* ``conn_indices`` int64 ``[sum of vertex counts]`` (CSR node indices),

with cell vertices counter-clockwise seen from outside the sphere, which is
the orientation the great-circle clipper needs for its clip polygon
(``inside`` = ``dot(a x b, p) >= -1e-14``,
``ax:include/axis/detail/spherical_clipper.hpp:301-335``).

The reference ships no cubed-sphere, tripole or Voronoi generator (its
benchmarks read C96 tiles from disk, ``ax:tests_python/test_c96_benchmarks.py``);
these are written from the standard definitions of each grid.
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class MeshArrays:
    node_lonlat: np.ndarray  # float64 [n_nodes, 2]
    conn_offsets: np.ndarray  # int64 [n_cells + 1]
    conn_indices: np.ndarray  # int64 [nnz]
    name: str = ""
    # Structured shape (ni, nj) for lat-lon grids, used only by reports.
    shape: tuple | None = None

    @property
    def n_cells(self) -> int:
        return int(self.conn_offsets.shape[0] - 1)

    @property
    def n_nodes(self) -> int:
        return int(self.node_lonlat.shape[0])


def _quad_connectivity(ni: int, nj: int, node_offset: int = 0, nip1: int | None = None):
    """BL, BR, TR, TL winding of ``StructuredGrid::to_unstructured``
    (``ax:src/topology/structured_grid.cpp:257-260``), cells row-major with
    the i (x) index fastest."""
    if nip1 is None:
        nip1 = ni + 1
    j, i = np.meshgrid(np.arange(nj, dtype=np.int64), np.arange(ni, dtype=np.int64), indexing="ij")
    bl = i + j * nip1
    br = (i + 1) + j * nip1
    tr = (i + 1) + (j + 1) * nip1
    tl = i + (j + 1) * nip1
    idx = np.stack([bl, br, tr, tl], axis=-1).reshape(-1) + node_offset
    return idx


def regular_latlon(ni: int, nj: int, lon_start: float = 0.0, lat_start: float = -90.0,
                   dlon: float | None = None, dlat: float | None = None) -> MeshArrays:
    """Regular lat-lon mesh laid out exactly like ``make_regular_mesh``
    (``ax:python/axis_py.cpp:75-103``): ``(ni+1)*(nj+1)`` corner nodes at
    ``lon_start + i*dlon``, ``lat_start + j*dlat`` (a separate node column at
    lon 360), cells row-major, BL/BR/TR/TL."""
    if dlon is None:
        dlon = 360.0 / ni
    if dlat is None:
        dlat = 180.0 / nj
    ii = np.arange(ni + 1, dtype=np.float64)
    jj = np.arange(nj + 1, dtype=np.float64)
    lon = lon_start + ii * dlon
    lat = lat_start + jj * dlat
    lon2 = np.broadcast_to(lon[None, :], (nj + 1, ni + 1)).reshape(-1)
    lat2 = np.broadcast_to(lat[:, None], (nj + 1, ni + 1)).reshape(-1)
    node = np.stack([lon2, lat2], axis=1).copy()
    idx = _quad_connectivity(ni, nj)
    off = np.arange(0, 4 * ni * nj + 1, 4, dtype=np.int64)
    return MeshArrays(node, off, idx, name=f"latlon{ni}x{nj}", shape=(ni, nj))


def rectilinear(lon_edges, lat_edges) -> MeshArrays:
    """Rectilinear lat-lon mesh on given (strictly increasing) cell edges, in
    the node and cell layout of ``regular_latlon``: cell ``i + j*ni`` spans
    ``lon_edges[i:i+2]`` x ``lat_edges[j:j+2]``."""
    lon = np.asarray(lon_edges, dtype=np.float64)
    lat = np.asarray(lat_edges, dtype=np.float64)
    ni, nj = lon.size - 1, lat.size - 1
    lon2 = np.broadcast_to(lon[None, :], (nj + 1, ni + 1)).reshape(-1)
    lat2 = np.broadcast_to(lat[:, None], (nj + 1, ni + 1)).reshape(-1)
    node = np.stack([lon2, lat2], axis=1).copy()
    off = np.arange(0, 4 * ni * nj + 1, 4, dtype=np.int64)
    return MeshArrays(node, off, _quad_connectivity(ni, nj), name=f"rect{ni}x{nj}", shape=(ni, nj))


def equal_area_latlon(ni: int, nj: int, lon_start: float = 0.0, stretch: float = 0.0) -> MeshArrays:
    """Global rectilinear mesh with equal-area latitude bands (edges at
    asin of evenly spaced sines) and, for ``stretch`` > 0, longitudes packed
    toward ``lon_start + 180``: a non-uniform grid on both axes."""
    lat = np.degrees(np.arcsin(np.linspace(-1.0, 1.0, nj + 1)))
    lat[0], lat[-1] = -90.0, 90.0
    t = np.linspace(0.0, 1.0, ni + 1)
    lon = lon_start + 360.0 * (t + stretch * np.sin(2.0 * np.pi * t) / (2.0 * np.pi))
    lon[0], lon[-1] = lon_start, lon_start + 360.0
    return rectilinear(lon, lat)


def latlon_deg(res_deg: float) -> MeshArrays:
    """Global lat-lon grid with cell edges on integer multiples of ``res_deg``
    (lon 0..360, lat -90..90)."""
    ni = int(round(360.0 / res_deg))
    nj = int(round(180.0 / res_deg))
    return regular_latlon(ni, nj, 0.0, -90.0, res_deg, res_deg)


# Right-handed (normal, u, v) frames of the six cube faces: u x v = normal,
# so a cell (i,j)->(i+1,j)->(i+1,j+1)->(i,j+1) is counter-clockwise seen from
# outside.
_CUBE_FACES = (
    ((1, 0, 0), (0, 1, 0), (0, 0, 1)),
    ((0, 1, 0), (-1, 0, 0), (0, 0, 1)),
    ((-1, 0, 0), (0, -1, 0), (0, 0, 1)),
    ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
    ((0, 0, 1), (0, 1, 0), (-1, 0, 0)),
    ((0, 0, -1), (0, 1, 0), (1, 0, 0)),
)


def _xyz_to_lonlat_deg(p: np.ndarray) -> np.ndarray:
    r = np.sqrt(np.einsum("ij,ij->i", p, p))
    lon = np.degrees(np.arctan2(p[:, 1], p[:, 0]))
    lon = np.where(lon < 0.0, lon + 360.0, lon)
    lon = np.where(lon >= 360.0, lon - 360.0, lon)
    lat = np.degrees(np.arcsin(np.clip(p[:, 2] / r, -1.0, 1.0)))
    return np.stack([lon, lat], axis=1)


def cubed_sphere(n: int) -> MeshArrays:
    """Gnomonic equiangular cubed sphere C<n>: 6 tiles of n x n cells, nodes
    welded across tile edges (each shared cube-edge point is one node).

    Tangent-plane coordinates are ``t_i = tan(pi/4 * (2i - n)/n)`` with the
    face edges forced to exactly +-1, so the unnormalised cube point of a
    shared node is bit-identical from both faces and welding is exact.
    Cells are ordered tile-major, then j, then i."""
    k = np.arange(n + 1, dtype=np.float64)
    t = np.tan((np.pi / 4.0) * ((2.0 * k - n) / n))
    t[0] = -1.0
    t[-1] = 1.0
    if n % 2 == 0:
        t[n // 2] = 0.0
    pts = []
    for nrm, u, v in _CUBE_FACES:
        nrm = np.asarray(nrm, dtype=np.float64)
        u = np.asarray(u, dtype=np.float64)
        v = np.asarray(v, dtype=np.float64)
        tj, ti = np.meshgrid(t, t, indexing="ij")  # [j, i]
        p = nrm[None, None, :] + ti[..., None] * u[None, None, :] + tj[..., None] * v[None, None, :]
        pts.append(p.reshape(-1, 3))
    allp = np.concatenate(pts, axis=0)
    # exact weld on the unnormalised cube point
    uniq, inv = np.unique(allp, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    # keep node order = order of first appearance, for locality
    first = np.full(uniq.shape[0], np.iinfo(np.int64).max, dtype=np.int64)
    np.minimum.at(first, inv, np.arange(inv.shape[0], dtype=np.int64))
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.shape[0])
    node_xyz = uniq[order]
    node_of = rank[inv]
    node = _xyz_to_lonlat_deg(node_xyz)
    per_face = (n + 1) * (n + 1)
    idx_local = _quad_connectivity(n, n)
    idx = np.concatenate([node_of[f * per_face + idx_local] for f in range(6)])
    off = np.arange(0, 4 * 6 * n * n + 1, 4, dtype=np.int64)
    return MeshArrays(node, off, idx.astype(np.int64), name=f"C{n}")


def tripole(ni: int = 1440, nj: int = 1080, seed: int = 4, jitter: float = 0.1) -> MeshArrays:
    """Curvilinear tripole-style ocean grid of ni x nj cells.

    South of ``lat_fold`` the grid is a Mercator-like lat-lon; north of it the
    rows bend towards two poles placed at seeded land points (longitudes
    ``lon_p`` and ``lon_p+180`` on the fold latitude), the bipolar cap of a
    tripole grid. Interior nodes are jittered by seeded uniform +-``jitter``
    of the local cell size. Nodes are not shared across the periodic seam
    (a separate node column at i = ni, as in the structured-grid layout), and
    the two cap rows meet the fold at the grid's top row.
    """
    rng = np.random.default_rng(seed)
    lon_p = float(rng.uniform(0.0, 180.0))
    lat_fold = 65.0
    lat_s = -78.0
    i = np.arange(ni + 1, dtype=np.float64)
    j = np.arange(nj + 1, dtype=np.float64)
    s = i / ni  # [0,1] around the globe
    r = j / nj
    nj_cap = nj // 6
    j_fold = nj - nj_cap
    lat_rows = np.empty(nj + 1)
    lat_rows[: j_fold + 1] = lat_s + (lat_fold - lat_s) * (j[: j_fold + 1] / j_fold)
    lon = np.empty((nj + 1, ni + 1))
    lat = np.empty((nj + 1, ni + 1))
    lon[: j_fold + 1, :] = (lon_p + 360.0 * s)[None, :]
    lat[: j_fold + 1, :] = lat_rows[: j_fold + 1, None]
    # bipolar cap: rows are circles around the two poles; q in (0,1] runs
    # from the fold to the pole-to-pole seam.
    for jj in range(j_fold + 1, nj + 1):
        q = (jj - j_fold) / nj_cap
        phi = 2.0 * np.pi * s
        # latitude lifted towards the north pole along the centre line, the
        # two poles stay on the fold latitude
        lat[jj, :] = lat_fold + (90.0 - lat_fold) * q * np.abs(np.sin(phi / 2.0)) ** 1.0 * (1.0 - 0.0 * q)
        lon[jj, :] = lon_p + 360.0 * s
    # smooth warp of the cap so the top row folds onto itself (i <-> ni - i)
    jit_lon = rng.uniform(-jitter, jitter, size=(nj + 1, ni + 1)) * (360.0 / ni)
    jit_lat = rng.uniform(-jitter, jitter, size=(nj + 1, ni + 1)) * ((lat_fold - lat_s) / j_fold)
    jit_lon[:, 0] = 0.0
    jit_lon[:, -1] = 0.0
    jit_lat[:, 0] = 0.0
    jit_lat[:, -1] = 0.0
    jit_lon[0, :] = 0.0
    jit_lat[0, :] = 0.0
    jit_lon[-1, :] = 0.0
    jit_lat[-1, :] = 0.0
    lon = lon + jit_lon
    lat = np.clip(lat + jit_lat, -89.9, 89.9)
    # periodic seam: column ni duplicates column 0 exactly (shifted 360)
    lon[:, ni] = lon[:, 0] + 360.0
    lat[:, ni] = lat[:, 0]
    lon = np.mod(lon, 360.0)
    node = np.stack([lon.reshape(-1), lat.reshape(-1)], axis=1)
    idx = _quad_connectivity(ni, nj)
    off = np.arange(0, 4 * ni * nj + 1, 4, dtype=np.int64)
    return MeshArrays(node, off, idx, name=f"tripole{ni}x{nj}", shape=(ni, nj))


def _fibonacci_points(n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    th = np.pi * (1.0 + 5.0 ** 0.5) * i
    return np.stack([r * np.cos(th), r * np.sin(th), z], axis=1)


def _tangent_basis(p: np.ndarray):
    a = np.where(np.abs(p[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
    e1 = np.cross(a, p)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(p, e1)
    return e1, e2


def _delaunay(p: np.ndarray):
    """Spherical Delaunay triangles (convex hull), oriented counter-clockwise
    seen from outside, and their circumcentres (the Voronoi vertices)."""
    from scipy.spatial import ConvexHull
    tri = ConvexHull(p).simplices.astype(np.int64)
    a, b, c = p[tri[:, 0]], p[tri[:, 1]], p[tri[:, 2]]
    nrm = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", nrm, a) < 0.0
    tri[flip, 1], tri[flip, 2] = tri[flip, 2], tri[flip, 1].copy()
    nrm[flip] *= -1.0
    cc = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    return tri, cc


def _fans(p: np.ndarray, tri: np.ndarray, cc: np.ndarray):
    """For every point, its incident triangles in counter-clockwise order
    around it (seen from outside): CSR offsets and triangle ids."""
    n = p.shape[0]
    owner = tri.reshape(-1)
    tid = np.repeat(np.arange(tri.shape[0], dtype=np.int64), 3)
    e1, e2 = _tangent_basis(p)
    d = cc[tid] - p[owner]
    ang = np.arctan2(np.einsum("ij,ij->i", d, e2[owner]), np.einsum("ij,ij->i", d, e1[owner]))
    # one sort on owner + angle fraction in [0, 1): owner ids < 2^31 leave more
    # than 20 bits of the angle in the float64 key
    key = owner.astype(np.float64) + (ang + np.pi) * (0.999 / (2.0 * np.pi))
    order = np.argsort(key, kind="stable")
    off = np.zeros(n + 1, dtype=np.int64)
    off[1:] = np.cumsum(np.bincount(owner, minlength=n))
    return off, tid[order]


def voronoi(n: int = 2621442, seed: int = 5, jitter: float = 0.2, lloyd: int = 5) -> MeshArrays:
    """Spherical Voronoi mesh of n cells (5- to 7-gons).

    Generators: Fibonacci-sphere points, each moved by a seeded uniform
    random tangent offset of up to ``jitter`` times the mean spacing, then
    ``lloyd`` Lloyd iterations (every generator moved to the centroid of its
    cell). The Lloyd steps keep the initial Delaunay triangulation (the
    points move by a fraction of the spacing, so the fans of incident
    triangles stay valid to first order) and the final cells come from an
    exact convex hull of the relaxed generators. Cell vertices are the
    circumcentres of the Delaunay triangles, shared between cells, listed
    counter-clockwise seen from outside."""
    rng = np.random.default_rng(seed)
    p = _fibonacci_points(n)
    spacing = np.sqrt(4.0 * np.pi / n)
    e1, e2 = _tangent_basis(p)
    r = jitter * spacing * np.sqrt(rng.uniform(0.0, 1.0, n))
    t = rng.uniform(0.0, 2.0 * np.pi, n)
    p = p + (r * np.cos(t))[:, None] * e1 + (r * np.sin(t))[:, None] * e2
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    if lloyd > 0:
        tri, cc = _delaunay(p)
        off, fan = _fans(p, tri, cc)
        owner = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
        nxt = np.arange(fan.shape[0], dtype=np.int64) + 1
        last = off[1:] - 1
        nxt[last] = off[:-1]  # wrap around each fan
        for _ in range(lloyd):
            a, b = tri[:, 0], tri[:, 1]
            nrm = np.cross(p[b] - p[a], p[tri[:, 2]] - p[a])
            cc = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
            v0, v1 = cc[fan], cc[fan[nxt]]
            g = p[owner]
            w = np.linalg.norm(np.cross(v0 - g, v1 - g), axis=1)  # 2 x planar fan triangle area
            q = w[:, None] * (g + v0 + v1)
            cen = np.stack([np.bincount(owner, weights=q[:, d], minlength=n) for d in range(3)], axis=1)
            p = cen / np.linalg.norm(cen, axis=1, keepdims=True)
    tri, cc = _delaunay(p)
    off, fan = _fans(p, tri, cc)
    node = _xyz_to_lonlat_deg(cc)
    return MeshArrays(node, off, fan, name=f"voronoi{n}")


def with_degenerate_cells(m: MeshArrays, seed: int) -> MeshArrays:
    """A copy of m in which a tenth of the cells (with at least four
    vertices) repeat their first vertex in place of the second, and three
    cells are collapsed to a point: the cases of the reference's
    degenerate-cell scan (detail/degenerate_cell_handler.hpp:115-236)."""
    rng = np.random.default_rng(seed)
    idx, off = m.conn_indices.copy(), m.conn_offsets
    for c in rng.choice(m.n_cells, m.n_cells // 10, replace=False):
        if off[c + 1] - off[c] >= 4:
            idx[off[c] + 1] = idx[off[c]]
    for c in rng.choice(m.n_cells, 3, replace=False):
        idx[off[c]:off[c + 1]] = idx[off[c]]
    return MeshArrays(m.node_lonlat, off, idx, name=f"degenerate_{m.name}")


def triangulated(m: MeshArrays) -> MeshArrays:
    """m with every quadrilateral split into two triangles (v0 v1 v2, v0 v2 v3)."""
    off, idx = [0], []
    for c in range(m.n_cells):
        v = list(m.conn_indices[m.conn_offsets[c]:m.conn_offsets[c + 1]])
        parts = [[v[0], v[1], v[2]], [v[0], v[2], v[3]]] if len(v) == 4 else [v]
        for p in parts:
            idx += p
            off.append(len(idx))
    return MeshArrays(m.node_lonlat, np.array(off, np.int64), np.array(idx, np.int64), name=f"triangulated_{m.name}")


def cell_centroids_xyz(mesh: MeshArrays) -> np.ndarray:
    """Normalised mean of the unit-sphere vertex vectors of every cell: the
    cap centroid of ``compute_cell_centroid_xyz``
    (``ax:include/axis/detail/spherical_cap_filter.hpp:85-122``)."""
    lon = np.radians(mesh.node_lonlat[:, 0])
    lat = np.radians(mesh.node_lonlat[:, 1])
    cl = np.cos(lat)
    xyz = np.stack([cl * np.cos(lon), cl * np.sin(lon), np.sin(lat)], axis=1)
    off = mesh.conn_offsets
    nv = np.diff(off)
    cell_of = np.repeat(np.arange(mesh.n_cells), nv)
    s = np.zeros((mesh.n_cells, 3))
    np.add.at(s, cell_of, xyz[mesh.conn_indices])
    s /= nv[:, None]
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    return s
