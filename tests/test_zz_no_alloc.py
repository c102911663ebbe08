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
