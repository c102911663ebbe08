"""The allocation-free residual entry point (vefem_assemble_residual_noalloc).

It serves callers that cannot call cudaMalloc when they assemble; its scratch
is a static device array.  Checked through the C ABI against the regular
entry point (vefem_assemble with VEFEM_RESIDUAL), bit for bit as the FP64
tests are, on two calls in a row (the second call reuses the scratch the
first one left behind).  This file is collected last on purpose, and it also
passes alone in a fresh process (the first call does the per-device set-up).
"""
import ctypes

import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


def _noalloc(L):
    f = L.vefem_assemble_residual_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("form", ["SQRT", "T"])
def test_noalloc_matches_regular_entry_point_twice(form):
    torch = pytest.importorskip("torch")
    B.build()
    L = V.load()
    f = _noalloc(L)
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 7)
    dev = torch.device("cuda:0")
    d_conn = torch.from_numpy(np.ascontiguousarray(mesh.conn)).to(dev)
    d_xyz = torch.from_numpy(np.ascontiguousarray(mesh.xyz)).to(dev)
    d_TL = torch.from_numpy(TL).to(dev)
    d_EU = torch.from_numpy(EU).to(dev)
    N = mesh.nnodes * 6 + phys.nex
    params = V.make_params(phys)
    outs = []
    for call in range(2):
        d_b = torch.zeros(N, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = f(ctypes.byref(params), mesh.nnodes, mesh.nel, d_conn.data_ptr(), d_xyz.data_ptr(),
               d_TL.data_ptr(), d_EU.data_ptr(), d_b.data_ptr(), None)
        assert rc == 0, L.vefem_last_error(None)
        outs.append(d_b.cpu().numpy())
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b_ref, _ = asm.set_equations_bulk(TL, EU, "MNR")
    asm.close()
    for b in outs:
        assert np.array_equal(b, b_ref)


def test_noalloc_rejects_oversized_mesh():
    B.build()
    L = V.load()
    f = _noalloc(L)
    phys = S.oldroyd_b(0.1, nex=0)
    params = V.make_params(phys)
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    rc = f(ctypes.byref(params), 400000, 40000, dummy, dummy, dummy, None, dummy, None)
    assert rc == 1
    assert b"exceeds the static scratch limit" in L.vefem_last_error(None)


def _fan_mesh(nsec: int):
    """``nsec`` kite-shaped 9-node quads around one centre node (node 1), so
    that node belongs to every element.  Returns conn [9, nel] (1-based) and
    xyz [3, nnodes]."""
    pts = [(0.0, 0.0)]

    def add(p):
        pts.append(p)
        return len(pts)            # 1-based id

    th = 2.0 * np.pi * np.arange(nsec) / nsec
    inner = [add((np.cos(t), np.sin(t))) for t in th]
    conn = []
    for k in range(nsec):
        a, b = inner[k], inner[(k + 1) % nsec]
        tm = 0.5 * (th[k] + th[k] + 2.0 * np.pi / nsec)
        c = add((2.0 * np.cos(tm), 2.0 * np.sin(tm)))
        P = {i: np.array(pts[i - 1]) for i in (1, a, b, c)}
        # corners counter-clockwise: centre, a, c, b; then mid-sides and centre
        m01 = add(tuple(0.5 * (P[1] + P[a])))
        m12 = add(tuple(0.5 * (P[a] + P[c])))
        m23 = add(tuple(0.5 * (P[c] + P[b])))
        m30 = add(tuple(0.5 * (P[b] + P[1])))
        mc = add(tuple(0.25 * (P[1] + P[a] + P[b] + P[c])))
        conn.append([1, a, c, b, m01, m12, m23, m30, mc])
    conn = np.ascontiguousarray(np.array(conn, dtype=np.int32).T)
    xy = np.array(pts).T
    xyz = np.ascontiguousarray(np.vstack([xy, np.zeros((1, xy.shape[1]))]))
    return conn, xyz


def _call_on_device(L, f, conn, xyz, phys, seed):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    nnodes, nel = xyz.shape[1], conn.shape[1]
    rng = np.random.default_rng(seed)
    TL = np.ascontiguousarray(rng.uniform(0.5, 1.0, (6, nnodes)))
    d_conn = torch.from_numpy(conn).to(dev)
    d_xyz = torch.from_numpy(xyz).to(dev)
    d_TL = torch.from_numpy(TL).to(dev)
    d_EU = torch.ones(1, dtype=torch.float64, device=dev)
    b0 = rng.standard_normal(nnodes * 6 + phys.nex)
    d_b = torch.from_numpy(b0.copy()).to(dev)
    params = V.make_params(phys)
    torch.cuda.synchronize()
    rc = f(ctypes.byref(params), nnodes, nel, d_conn.data_ptr(), d_xyz.data_ptr(),
           d_TL.data_ptr(), d_EU.data_ptr(), d_b.data_ptr(), None)
    return rc, b0, d_b.cpu().numpy()


def test_noalloc_rejects_crowded_node_leaving_b_unchanged():
    """A node shared by 33 elements (one more than the per-node limit) is
    found before anything is added: VEFEM_ERR_ARG and b untouched.  A fan of
    32 passes."""
    B.build()
    L = V.load()
    f = _noalloc(L)
    phys = S.oldroyd_b(0.1, nex=0)
    conn, xyz = _fan_mesh(33)
    rc, b0, b = _call_on_device(L, f, conn, xyz, phys, 3)
    assert rc == 1   # VEFEM_ERR_ARG
    assert b"more than 32 elements" in L.vefem_last_error(None)
    assert np.array_equal(b, b0)
    conn, xyz = _fan_mesh(32)
    rc, b0, b = _call_on_device(L, f, conn, xyz, phys, 4)
    assert rc == 0, L.vefem_last_error(None)
    assert not np.array_equal(b, b0)


def test_noalloc_rejects_bad_connectivity_leaving_b_unchanged():
    """A connectivity id of nnodes + 1 is caught on the device before any
    access through it: VEFEM_ERR_ARG, its message, and b untouched."""
    B.build()
    L = V.load()
    f = _noalloc(L)
    phys = S.oldroyd_b(0.1, nex=0)
    conn, xyz = _fan_mesh(8)
    conn = conn.copy()
    conn[4, 5] = xyz.shape[1] + 1
    rc, b0, b = _call_on_device(L, f, conn, xyz, phys, 5)
    assert rc == 1   # VEFEM_ERR_ARG
    assert b"connectivity id out of range" in L.vefem_last_error(None)
    assert np.array_equal(b, b0)

