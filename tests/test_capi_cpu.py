"""C-ABI checks that need no GPU: the library loads, exports every function
include/vefem.h declares, builds the preAllocatePetsc pattern like the numpy
restatement, and rejects bad arguments with an error code (never a crash)."""
import ctypes
import os
import re

import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return V.load()


def _declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(vefem_[a-z_0-9]+)\s*\(", text,
                                re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) >= set(V.EXPORTED)
    assert lib.vefem_abi_version() == 1


@pytest.mark.parametrize("nex", [0, 1])
def test_pattern_matches_numpy_restatement(lib, nex):
    mesh = M.build_cylinder_mesh(2000)
    r1, c1 = V.build_pattern(mesh.conn, mesh.nnodes, nex)
    r2, c2 = P.build_pattern(mesh.element_nodes(), mesh.nnodes, nex)
    assert np.array_equal(r1, r2)
    assert np.array_equal(c1, c2)
    # sorted columns in every row
    rows = np.repeat(np.arange(len(r1) - 1), np.diff(r1))
    assert np.all((np.diff(c1) > 0) | (np.diff(rows) > 0))


def test_create_rejects_bad_pattern_and_params(lib):
    mesh = M.rect_mesh(2, 2)
    phys = S.oldroyd_b(0.1, nex=1)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    # wrong size (nex mismatch)
    with pytest.raises(V.VefemError, match="pattern size"):
        V.BulkAssembler(mesh, S.oldroyd_b(0.1, nex=0), rowptr, colind)
    # a pattern that lacks an element block
    r2, c2 = P.build_pattern(mesh.element_nodes()[:1], mesh.nnodes, 1)
    with pytest.raises(V.VefemError, match="pattern"):
        V.BulkAssembler(mesh, phys, r2, c2)
    bad = S.oldroyd_b(0.1, nex=1)
    bad.form = "SQRT"
    p = V.make_params(bad)
    p.model = 9
    cm = V.c_mesh(mesh.nnodes, mesh.nel, mesh.conn.ctypes.data, mesh.xyz.ctypes.data, 0, None, None)
    cc = V.c_csr(len(rowptr) - 1, rowptr.ctypes.data, colind.ctypes.data)
    h = ctypes.c_void_p()
    assert lib.vefem_create(ctypes.byref(cm), ctypes.byref(cc), ctypes.byref(p), ctypes.byref(h)) == 1
    assert b"model" in lib.vefem_last_error(None)
    # connectivity out of range
    conn = mesh.conn.copy()
    conn[0, 0] = mesh.nnodes + 5
    cm2 = V.c_mesh(mesh.nnodes, mesh.nel, conn.ctypes.data, mesh.xyz.ctypes.data, 0, None, None)
    p = V.make_params(phys)
    assert lib.vefem_create(ctypes.byref(cm2), ctypes.byref(cc), ctypes.byref(p), ctypes.byref(h)) == 1


def test_no_gpu_fails_loudly(lib):
    """Without a usable GPU vefem_create reports a CUDA error; there is no CPU fallback."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    mesh = M.rect_mesh(2, 2)
    phys = S.oldroyd_b(0.1, nex=1)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    with pytest.raises(V.VefemError, match="CUDA|cuda|stream|device"):
        V.BulkAssembler(mesh, phys, rowptr, colind)
