"""Edge cases of the element and scatter kernels: a single element, element
counts that leave ragged tails in every kernel's element batch (4 per FD
CTA, 8 per residual CTA, 1..8 per batched work item), instances of one
element in the batched form, and the stability assembly of one element.
Everything FP64 is compared bit for bit with the oracle, the FP32 Jacobian
within its tolerance."""
import numpy as np
import pytest

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


SHAPES = [(1, 1), (3, 1), (5, 1), (3, 3), (13, 1), (7, 3)]     # 1, 3, 5, 9, 13, 21 elements


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_ragged_element_counts_bitwise(shape, form):
    mesh = M.rect_mesh(*shape, 0.0, 1.0, 0.0, 1.0, distort=0.2, seed=3)
    phys = S.giesekus(0.1, 0.4, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, seed=5)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b, vals = asm.set_equations_bulk(TL, EU, "NRP")
    bo, vo = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    assert np.array_equal(b, bo) and np.array_equal(vals, vo)
    r, _ = asm.set_equations_bulk(TL, EU, "MNR")
    assert np.array_equal(r, bo)
    b32 = np.zeros_like(b)
    v32 = np.zeros(len(colind), np.float32)
    asm.assemble(TL, EU, V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT32, b32, v32)
    assert np.array_equal(b32, bo)
    assert np.max(np.abs(v32 - vo)) <= 2e-4 * np.max(np.abs(vo))
    asm.close()


def test_batched_with_single_element_instances():
    shapes = [(1, 1), (2, 1), (1, 1), (5, 3)]
    meshes = [M.rect_mesh(*s, 0.0, 1.0, 0.0, 1.0, distort=0.1, seed=i) for i, s in enumerate(shapes)]
    physs = [S.oldroyd_b(0.2 + 0.1 * i, 0.59, "SQRT", nex=0) for i in range(len(shapes))]
    pats = [V.build_pattern(m.conn, m.nnodes, 0) for m in meshes]
    states = [S.seeded_state(m.xyz, p, seed=i)[0] for i, (m, p) in enumerate(zip(meshes, physs))]
    bt = V.BatchAssembler(meshes, physs, pats)
    bt.set_tiles([8, 8, 8, 8, 8, 8])
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT64 | V.VEFEM_ZERO_FIRST
    bs = [np.zeros(len(rp) - 1) for rp, _ in pats]
    vs = [np.zeros(len(ci)) for _, ci in pats]
    bt.assemble(states, [np.zeros(1)] * len(shapes), flags, bs, vs)
    for m, p, (rp, ci), TL, b, v in zip(meshes, physs, pats, states, bs, vs):
        a = V.BulkAssembler(m, p, rp, ci)
        b1 = np.zeros(len(rp) - 1)
        v1 = np.zeros(len(ci))
        a.assemble(TL, None, flags, b1, v1)
        a.close()
        assert np.array_equal(b, b1) and np.array_equal(v, v1)
        bo, _ = O.assemble(p, m.conn, m.xyz, TL, np.zeros(0), rp, ci, jacobian=False)
        assert np.array_equal(b, bo)
    bt.close()


def test_stability_single_element():
    mesh = M.rect_mesh(1, 1, 0.0, 1.0, 0.0, 1.0, distort=0.2, seed=4)
    phys = S.oldroyd_b(0.5, 0.59, "T", nex=0)
    TL, _ = S.seeded_state(mesh.xyz, phys, seed=1)
    TLb = np.zeros((10, mesh.nnodes))
    TLb[0:2] = TL[0:2]
    TLb[3:7] = TL[2:6]
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 0)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    rp, ci = asm.stability_pattern()
    assert len(ci) == 90 * 90
    As, B_ = asm.stability_assemble(TLb, [1.5])
    _, _, A, Bo = O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, np.zeros_like(TLb), 1.5)
    en = mesh.element_nodes()[0]
    order = np.argsort(en)                       # pattern columns are sorted by node
    dense = A[0].reshape(90, 90).T               # row (jnod, jeq), column (inod, ieq)
    blk = dense.reshape(9, 10, 9, 10)[order][:, :, order].reshape(90, 90)
    got = np.zeros((90, 90))
    for r in range(90):
        got[r] = As[0][rp[r]:rp[r + 1]]
    assert np.max(np.abs(got - blk)) <= 1e-12 * np.max(np.abs(blk))
    asm.close()
