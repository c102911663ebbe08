"""Mesh generator and the reference's mesh file format (no GPU).

* the cylinder-in-channel meshes have exactly the requested element counts
  of the benchmark configurations, lie in the channel, put the cylinder nodes
  on r = R, map every element with a positive Jacobian at all 3x3 Gauss
  points, and are conforming (every interior edge shared by two elements
  with the same three nodes, the boundary edges on the channel walls, inlet,
  outlet or cylinder);
* the local node order is setQuadraticQuadrangle's (Gauss_Quadrangle_mod.F90:
  413-421): corners counter-clockwise from (-1,-1), mid-sides of eta=-1,
  xi=+1, eta=+1, xi=-1, then the centre;
* ``write_dta`` / ``read_dta`` (readMeshFile, FEM_mod.F90:172-256) round-trip
  coordinates and connectivity bit for bit, and a reader of the 2-D elements
  skips the 1-D outlet-edge lines.
"""
import collections

import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import mesh as M

# 1-D Gauss points of the reference's 3-point rule (centre 0 + 1e-8)
_G = np.array([0.0 + 1e-8, np.sqrt(0.6), -np.sqrt(0.6)])


def _q2_shape_derivatives(c, e):
    """d/dxi and d/deta of the nine Q2 shape functions at (c, e) in the
    reference's local node order."""
    def l(t):
        return np.array([0.5 * t * (t - 1.0), 1.0 - t * t, 0.5 * t * (t + 1.0)])

    def dl(t):
        return np.array([t - 0.5, -2.0 * t, t + 0.5])

    # lattice index (0, 1, 2) <-> local coordinate (-1, 0, +1)
    ij = M._LOCAL_IJ
    lc, le, dlc, dle = l(c), l(e), dl(c), dl(e)
    dNc = dlc[ij[:, 0]] * le[ij[:, 1]]
    dNe = lc[ij[:, 0]] * dle[ij[:, 1]]
    return dNc, dNe


@pytest.mark.parametrize("nel", [2000, 20000, 40000])
def test_cylinder_mesh_counts_and_geometry(nel):
    mesh = M.build_cylinder_mesh(nel)
    assert mesh.nel == nel
    assert 4.0 * nel < mesh.nnodes <= 4.25 * nel      # ~4 nodes per Q2 element plus boundaries
    x, y = mesh.xyz[0], mesh.xyz[1]
    assert x.min() == pytest.approx(-15.0) and x.max() == pytest.approx(25.0)
    assert y.min() == pytest.approx(-2.0) and y.max() == pytest.approx(2.0)
    r = np.hypot(x, y)
    assert r.min() >= 1.0 - 1e-12
    cyl = mesh.boundary_nodes["Cylinder"]
    assert np.allclose(r[cyl], 1.0, atol=1e-12) and cyl.size > 0
    # every node is used, ids are 1-based
    assert mesh.conn.min() == 1 and mesh.conn.max() == mesh.nnodes
    assert np.unique(mesh.conn).size == mesh.nnodes
    assert np.all(M.element_jacobian_signs(mesh) > 0)


def test_positive_jacobian_at_every_gauss_point():
    mesh = M.build_cylinder_mesh(2000)
    en = mesh.element_nodes()
    x, y = mesh.xyz[0][en], mesh.xyz[1][en]
    for c in _G:
        for e in _G:
            dNc, dNe = _q2_shape_derivatives(c, e)
            det = (x @ dNc) * (y @ dNe) - (x @ dNe) * (y @ dNc)
            assert np.all(det > 0.0)


def test_mesh_is_conforming():
    mesh = M.build_cylinder_mesh(2000)
    en = mesh.element_nodes()
    edges = collections.defaultdict(list)
    for e in range(mesh.nel):
        for ied, (a, b, c) in M.EDGE_NODES.items():
            key = frozenset((en[e, a], en[e, b]))
            edges[key].append((e, en[e, c]))
    on = {name: set(v.tolist()) for name, v in mesh.boundary_nodes.items()}
    boundary = set().union(*on.values())
    n_boundary = 0
    for key, uses in edges.items():
        assert len(uses) in (1, 2)
        if len(uses) == 2:
            assert uses[0][1] == uses[1][1]          # the same mid-side node
        else:
            n_boundary += 1
            assert key <= boundary and uses[0][1] in boundary
    # outlet edges: the ones the generator lists, all on x = x_out
    outlet = [k for k, u in edges.items() if len(u) == 1 and k <= on["Outlet"]]
    assert len(outlet) == len(mesh.outlet_edges) == mesh.params["m"]
    assert n_boundary > 0


def test_local_node_order():
    mesh = M.rect_mesh(2, 1, 0.0, 2.0, 0.0, 1.0)
    en = mesh.element_nodes()[0]
    xy = mesh.xyz[:2, en].T
    expected = np.array([(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0),    # corners, CCW
                         (0.5, 0.0), (1.0, 0.5), (0.5, 1.0), (0.0, 0.5),    # mid-sides
                         (0.5, 0.5)])                                        # centre
    assert np.array_equal(xy, expected)
    assert tuple(M.EDGE_NODES[1]) == (0, 1, 4) and tuple(M.EDGE_NODES[4]) == (3, 0, 7)


def test_exact_false_allows_nearest_layout():
    mesh = M.build_cylinder_mesh(2013, exact=False)
    assert abs(mesh.nel - 2013) <= 0.05 * 2013
    with pytest.raises(ValueError):
        M.build_cylinder_mesh(7)


def test_dta_round_trip_is_bit_exact(tmp_path):
    mesh = M.build_cylinder_mesh(2000)
    path = tmp_path / "Cylinder_2D_MESH.DTA"
    M.write_dta(mesh, str(path))
    conn, xyz = M.read_dta(str(path))
    assert np.array_equal(conn, mesh.conn)
    assert np.array_equal(xyz, mesh.xyz)
    # the header counts the 1-D outlet edges too; a 1-D reader gets them back
    head = path.read_text().split("\n", 1)[0].split()
    assert int(head[0]) == mesh.nnodes
    assert int(head[1]) == mesh.nel + len(mesh.outlet_edges)
    edges, _ = M.read_dta(str(path), ndim=1)
    en = mesh.element_nodes() + 1
    for k, (e, ied) in enumerate(mesh.outlet_edges):
        a, b, c = M.EDGE_NODES[int(ied)]
        assert tuple(edges[:, k]) == (en[e, a], en[e, b], en[e, c])
