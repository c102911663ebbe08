"""Block-structured Q2 (9-node) meshes of the cylinder-in-channel geometry.

The reference reads SALOME-made ``<Problem>_MESH.DTA`` files
(FEM_mod.F90:172-256) and ships none, so this module builds the same kind of
mesh itself: a cylinder of radius ``R`` centred at the origin inside a channel
``y in [-H, H]``, ``x in [x_in, x_out]``.

Layout: an O-grid ring from the cylinder to the square ``[-H, H]^2`` (``4*m``
elements around, ``nr`` radially, geometric grading towards the cylinder),
plus an upstream block ``[x_in, -H] x [-H, H]`` and a downstream block
``[H, x_out] x [-H, H]``, each ``m`` elements high.  The element count is
``m * (4*nr + nu + nd)``.

Local node order follows setQuadraticQuadrangle (Gauss_Quadrangle_mod.F90:
405-478): corners counter-clockwise from (-1,-1), then the mid-side nodes of
eta=-1, xi=+1, eta=+1, xi=-1, then the centre.  Every element is mapped with a
positive Jacobian.

Arrays use the reference's own layouts (Fortran column-major):
``conn`` is Connectivity(Nel, 9) -> C array [9, Nel] of 1-based node ids,
``xyz`` is Xi_Mesh(Nnodes, 3) -> C array [3, Nnodes].
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# local (i, j) lattice offsets of the 9 nodes inside an element's 3x3 sub-lattice,
# i along xi, j along eta
_LOCAL_IJ = np.array([(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)])

# edge id (1..4, Gauss_Quadrangle_mod.F90:264-276) -> its three local nodes (0-based)
EDGE_NODES = {1: (0, 1, 4), 2: (1, 2, 5), 3: (2, 3, 6), 4: (3, 0, 7)}


@dataclasses.dataclass
class Mesh:
    conn: np.ndarray          # int32 [9, Nel], 1-based node ids (Connectivity(Nel, 9) in memory order)
    xyz: np.ndarray           # float64 [3, Nnodes] (Xi_Mesh(Nnodes, 3) in memory order)
    boundary_nodes: dict      # name -> sorted int array of 0-based node ids
    outlet_edges: np.ndarray  # int32 [n, 2]: (element 0-based, edge id 1..4) on x = x_out
    params: dict

    @property
    def nel(self) -> int:
        return int(self.conn.shape[1])

    @property
    def nnodes(self) -> int:
        return int(self.xyz.shape[1])

    def element_nodes(self) -> np.ndarray:
        """[Nel, 9] 0-based node ids (row per element)."""
        return np.ascontiguousarray(self.conn.T - 1)


def _grade(n2: int, ratio: float) -> np.ndarray:
    """2*n+1 points on [0, 1], geometric element sizes with last/first = ratio;
    mid nodes sit at the parametric midpoint of each element."""
    n = n2 // 2
    if n == 1 or abs(ratio - 1.0) < 1e-12:
        edges = np.linspace(0.0, 1.0, n + 1)
    else:
        q = ratio ** (1.0 / (n - 1))
        h = q ** np.arange(n)
        edges = np.concatenate([[0.0], np.cumsum(h)]) / h.sum()
    pts = np.empty(2 * n + 1)
    pts[0::2] = edges
    pts[1::2] = 0.5 * (edges[:-1] + edges[1:])
    return pts


def _square_point(sig: np.ndarray, H: float) -> np.ndarray:
    """Point on the square [-H, H]^2 perimeter, sig in [0, 4) counter-clockwise
    from (H, -H) ... so that side 0 is x = +H going up."""
    sig = np.mod(sig, 4.0)
    k = np.floor(sig).astype(int)
    u = sig - k
    out = np.empty(sig.shape + (2,))
    # side 0: right, (H,-H)->(H,H); 1: top, (H,H)->(-H,H); 2: left, (-H,H)->(-H,-H); 3: bottom
    s0 = k == 0
    out[s0, 0] = H
    out[s0, 1] = -H + 2 * H * u[s0]
    s1 = k == 1
    out[s1, 0] = H - 2 * H * u[s1]
    out[s1, 1] = H
    s2 = k == 2
    out[s2, 0] = -H
    out[s2, 1] = H - 2 * H * u[s2]
    s3 = k == 3
    out[s3, 0] = -H + 2 * H * u[s3]
    out[s3, 1] = -H
    return out


def choose_blocks(nel: int, exact: bool = True, x_in: float = -15.0, x_out: float = 25.0,
                  H: float = 2.0):
    """Pick (m, nr, nu, nd) with m*(4*nr + nu + nd) == nel.

    ``m`` is a divisor of ``nel`` close to sqrt(nel/20); with ``exact=False``
    the count is rounded to the nearest achievable one instead."""
    m0 = math.sqrt(nel / 20.0)
    best = None
    for m in range(max(2, int(m0 * 0.5)), int(m0 * 2.0) + 2):
        if nel % m and exact:
            continue
        cols = nel // m if exact else max(1, round(nel / m))
        nr = max(2, round(m * 1.0))
        rest = cols - 4 * nr
        if rest < 4:
            nr = max(2, (cols - 4) // 4)
            rest = cols - 4 * nr
        if rest < 4 or nr < 2:
            continue
        lu, ld = (-H - x_in), (x_out - H)
        nu = max(2, round(rest * lu / (lu + ld)))
        nd = rest - nu
        if nd < 2:
            continue
        score = abs(m - m0) + (0 if exact or m * cols == nel else abs(m * cols - nel))
        if best is None or score < best[0]:
            best = (score, m, nr, nu, nd)
    if best is None:
        raise ValueError(f"no block layout for {nel} elements (exact={exact})")
    return best[1:]


def build_cylinder_mesh(nel: int, exact: bool = True, R: float = 1.0, H: float = 2.0,
                        x_in: float = -15.0, x_out: float = 25.0, ring_ratio: float = 6.0,
                        channel_ratio: float = 6.0) -> Mesh:
    """Q2 mesh of the cylinder-in-channel geometry with ``nel`` elements."""
    m, nr, nu, nd = choose_blocks(nel, exact, x_in, x_out, H)
    coords = []     # list of [ny_nodes, nx_nodes, 2] lattices
    elements = []   # (lattice id, i0, j0) per element, lattice index (i along xi, j along eta)

    # upstream block: xi along x, eta along y; fine next to the square
    xs = x_in + (-H - x_in) * (1.0 - _grade(2 * nu, channel_ratio)[::-1])
    ys = np.linspace(-H, H, 2 * m + 1)
    lat_up = np.stack(np.meshgrid(xs, ys, indexing="ij"), axis=-1)       # [2nu+1, 2m+1, 2]
    # ring: xi radial (outwards), eta counter-clockwise around
    t = _grade(2 * nr, ring_ratio)
    sig = np.arange(8 * m + 1) / (2.0 * m)                               # 0..4 (wraps)
    q = _square_point(sig, H)
    ang = np.arctan2(q[:, 1], q[:, 0])
    c = np.stack([R * np.cos(ang), R * np.sin(ang)], axis=-1)
    lat_ring = c[None, :, :] + t[:, None, None] * (q - c)[None, :, :]    # [2nr+1, 8m+1, 2]
    # downstream block
    xs = H + (x_out - H) * _grade(2 * nd, channel_ratio)
    lat_dn = np.stack(np.meshgrid(xs, ys, indexing="ij"), axis=-1)
    coords = [lat_up, lat_ring, lat_dn]
    for j in range(m):
        for i in range(nu):
            elements.append((0, 2 * i, 2 * j))
    for j in range(4 * m):
        for i in range(nr):
            elements.append((1, 2 * i, 2 * j))
    for j in range(m):
        for i in range(nd):
            elements.append((2, 2 * i, 2 * j))

    # merge coincident lattice points (block interfaces, ring seam) by rounded coordinates
    key_to_id = {}
    node_xy = []
    lat_ids = []
    for lat in coords:
        ids = np.empty(lat.shape[:2], dtype=np.int64)
        for a in range(lat.shape[0]):
            for b in range(lat.shape[1]):
                x, y = lat[a, b]
                key = (round(float(x) * 1e8), round(float(y) * 1e8))
                nid = key_to_id.get(key)
                if nid is None:
                    nid = len(node_xy)
                    key_to_id[key] = nid
                    node_xy.append((float(x), float(y)))
                ids[a, b] = nid
        lat_ids.append(ids)
    conn0 = np.empty((len(elements), 9), dtype=np.int64)
    for e, (lid, i0, j0) in enumerate(elements):
        ids = lat_ids[lid]
        conn0[e] = ids[i0 + _LOCAL_IJ[:, 0], j0 + _LOCAL_IJ[:, 1]]

    # renumber nodes in order of first use by the elements
    order = np.full(len(node_xy), -1, dtype=np.int64)
    nxt = 0
    for nid in conn0.ravel():
        if order[nid] < 0:
            order[nid] = nxt
            nxt += 1
    xy = np.empty((nxt, 2))
    xy[order] = np.asarray(node_xy)
    conn0 = order[conn0]

    xyz = np.zeros((3, nxt))
    xyz[0] = xy[:, 0]
    xyz[1] = xy[:, 1]
    tol = 1e-6 * max(1.0, H)
    r = np.hypot(xy[:, 0], xy[:, 1])
    bnodes = {
        "Inlet": np.nonzero(np.abs(xy[:, 0] - x_in) < tol)[0],
        "Outlet": np.nonzero(np.abs(xy[:, 0] - x_out) < tol)[0],
        "Wall": np.nonzero(np.abs(np.abs(xy[:, 1]) - H) < tol)[0],
        "Cylinder": np.nonzero(np.abs(r - R) < tol)[0],
    }
    out_edges = []
    on_out = np.zeros(nxt, dtype=bool)
    on_out[bnodes["Outlet"]] = True
    for e in range(conn0.shape[0]):
        for ied, ln in EDGE_NODES.items():
            if on_out[conn0[e, list(ln)]].all():
                out_edges.append((e, ied))
    mesh = Mesh(conn=np.ascontiguousarray((conn0 + 1).T.astype(np.int32)),
                xyz=np.ascontiguousarray(xyz), boundary_nodes=bnodes,
                outlet_edges=np.asarray(out_edges, dtype=np.int32).reshape(-1, 2),
                params=dict(m=m, nr=nr, nu=nu, nd=nd, R=R, H=H, x_in=x_in, x_out=x_out))
    return mesh


def element_jacobian_signs(mesh: Mesh) -> np.ndarray:
    """Sign of detJ at the element centre (for mesh validity checks)."""
    en = mesh.element_nodes()
    x = mesh.xyz[0][en]
    y = mesh.xyz[1][en]
    # derivatives of the Q2 map at (0, 0): only mid-side nodes contribute
    dxdc = 0.5 * (x[:, 5] - x[:, 7])
    dydc = 0.5 * (y[:, 5] - y[:, 7])
    dxde = 0.5 * (x[:, 6] - x[:, 4])
    dyde = 0.5 * (y[:, 6] - y[:, 4])
    return np.sign(dxdc * dyde - dxde * dydc)


def write_dta(mesh: Mesh, path: str, edges_1d: bool = True) -> None:
    """Write a ``<Problem>_MESH.DTA`` file as readMeshFile (FEM_mod.F90:172-256)
    reads it: ``Nnodes Nel_total``, then ``id x y z`` per node, then
    ``id type n1..n_k`` per element with type = 100*dim + k.  The 2-D elements
    come last (the reader keeps the last Nel lines of its own dimension)."""
    lines = []
    en = mesh.element_nodes() + 1
    extra = []
    if edges_1d:
        for e, ied in mesh.outlet_edges:
            a, b, c = EDGE_NODES[int(ied)]
            extra.append((103, (en[e, a], en[e, b], en[e, c])))
    ntot = len(extra) + mesh.nel
    lines.append(f"{mesh.nnodes} {ntot}")
    for i in range(mesh.nnodes):
        lines.append(f"{i + 1} {mesh.xyz[0, i]:.17e} {mesh.xyz[1, i]:.17e} {mesh.xyz[2, i]:.17e}")
    k = 0
    for typ, nodes in extra:
        k += 1
        lines.append(f"{k} {typ} " + " ".join(str(int(n)) for n in nodes))
    for e in range(mesh.nel):
        k += 1
        lines.append(f"{k} 209 " + " ".join(str(int(n)) for n in en[e]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_dta(path: str, ndim: int = 2):
    """Read a ``_MESH.DTA`` file the way readMeshFile does; returns
    (conn [9, Nel] 1-based int32, xyz [3, Nnodes] float64)."""
    with open(path) as f:
        head = f.readline().split()
        nnodes, ntot = int(head[0]), int(head[1])
        xyz = np.zeros((3, nnodes))
        for i in range(nnodes):
            parts = f.readline().split()
            xyz[:, i] = [float(v) for v in parts[1:4]]
        rows = []
        for _ in range(ntot):
            parts = f.readline().split()
            typ = int(parts[1])
            if typ // 100 == ndim:
                rows.append([int(v) for v in parts[2:2 + typ % 100]])
    conn = np.ascontiguousarray(np.asarray(rows, dtype=np.int32).T)
    return conn, xyz


def rect_mesh(nx: int, ny: int, x0: float = 0.0, x1: float = 1.0, y0: float = 0.0,
              y1: float = 1.0, distort: float = 0.0, seed: int = 0) -> Mesh:
    """Structured Q2 mesh of a rectangle (small test meshes).  ``distort``
    moves interior lattice points randomly by up to that fraction of a
    half-cell, which makes the element maps non-affine."""
    xs = np.linspace(x0, x1, 2 * nx + 1)
    ys = np.linspace(y0, y1, 2 * ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    if distort:
        rng = np.random.default_rng(seed)
        hx = (x1 - x0) / (2 * nx)
        hy = (y1 - y0) / (2 * ny)
        X[1:-1, 1:-1] += distort * hx * rng.uniform(-1, 1, X[1:-1, 1:-1].shape)
        Y[1:-1, 1:-1] += distort * hy * rng.uniform(-1, 1, Y[1:-1, 1:-1].shape)
    ids = np.arange(X.size).reshape(X.shape)
    conn0 = []
    for j in range(ny):
        for i in range(nx):
            conn0.append(ids[2 * i + _LOCAL_IJ[:, 0], 2 * j + _LOCAL_IJ[:, 1]])
    conn0 = np.asarray(conn0, dtype=np.int64)
    xyz = np.zeros((3, X.size))
    xyz[0] = X.ravel()
    xyz[1] = Y.ravel()
    tol = 1e-12
    bnodes = {
        "Left": np.nonzero(np.abs(xyz[0] - x0) < tol)[0],
        "Right": np.nonzero(np.abs(xyz[0] - x1) < tol)[0],
        "Bottom": np.nonzero(np.abs(xyz[1] - y0) < tol)[0],
        "Top": np.nonzero(np.abs(xyz[1] - y1) < tol)[0],
    }
    out_edges = [(j * nx + nx - 1, 2) for j in range(ny)]
    return Mesh(conn=np.ascontiguousarray((conn0 + 1).T.astype(np.int32)), xyz=xyz,
                boundary_nodes=bnodes, outlet_edges=np.asarray(out_edges, dtype=np.int32),
                params=dict(nx=nx, ny=ny))
