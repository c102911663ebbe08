"""Golden fixtures (tests/golden/golden.json, made by tests/golden/make_golden.py):
the oracle must reproduce the recorded bits, and so must the CUDA library."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.mark.parametrize("entry", GOLD, ids=lambda e: f"{e['case']['model']}-{e['case']['form']}-{e['case']['VeN']}")
def test_oracle_reproduces_golden(entry):
    _, _, _, _, res, jac, ac = G.run_case(entry["case"])
    assert G.digest(res) == entry["res_sha256"]
    assert G.digest(jac) == entry["jac_sha256"]
    assert G.digest(ac) == entry["ac_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("entry", GOLD, ids=lambda e: f"{e['case']['model']}-{e['case']['form']}-{e['case']['VeN']}")
def test_library_reproduces_golden(entry):
    """Element outputs from the library's scatter of a mesh with disjoint elements equal
    the golden bits: assemble each element of the case on its own copy of the nodes."""
    from ve_flow_around_cylinder_fortran_gb300 import build as B
    from ve_flow_around_cylinder_fortran_gb300 import mesh as M
    from ve_flow_around_cylinder_fortran_gb300 import pattern as P
    from ve_flow_around_cylinder_fortran_gb300 import vefem as V
    B.build()
    c = entry["case"]
    mesh = G.case_mesh(c)
    phys = G.case_phys(c)
    from ve_flow_around_cylinder_fortran_gb300 import state as S
    TL, EU = S.portable_state(mesh.xyz, phys, c["seed"])
    # element-duplicated copy (like the reference's TL_Rank): node 9*e + i
    en = mesh.element_nodes()
    nel = mesh.nel
    dup = M.Mesh(conn=np.ascontiguousarray((np.arange(9 * nel).reshape(nel, 9) + 1).T.astype(np.int32)),
                 xyz=np.ascontiguousarray(mesh.xyz[:, en.ravel()]), boundary_nodes={},
                 outlet_edges=np.zeros((0, 2), np.int32), params={})
    TLd = np.ascontiguousarray(TL[:, en.ravel()])
    rowptr, colind = P.build_pattern(dup.element_nodes(), dup.nnodes, phys.nex)
    asm = V.BulkAssembler(dup, phys, rowptr, colind)
    b, vals = asm.set_equations_bulk(TLd, EU, "NRP")
    asm.close()
    res = b[:-1].reshape(nel, 9, 6)
    N = len(rowptr) - 1
    jac = np.zeros((nel, 9, 6, 9, 6))
    ac = np.zeros((nel, 9, 6, 1))
    for e in range(nel):
        for jnod in range(9):
            for jeq in range(6):
                row = (9 * e + jnod) * 6 + jeq
                s0 = rowptr[row]
                cols = colind[s0:rowptr[row + 1]]
                for inod in range(9):
                    for ieq in range(6):
                        k = np.searchsorted(cols, (9 * e + inod) * 6 + ieq)
                        jac[e, inod, ieq, jnod, jeq] = vals[s0 + k]
                assert cols[-1] == N - 1
                ac[e, jnod, jeq, 0] = vals[rowptr[row + 1] - 1]
    assert G.digest(res) == entry["res_sha256"]
    assert G.digest(jac) == entry["jac_sha256"]
    assert G.digest(ac) == entry["ac_sha256"]
