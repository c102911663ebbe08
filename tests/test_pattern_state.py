"""AIJ pattern, seeded states and boundary rows (no GPU).

* ``build_pattern`` freezes preAllocatePetsc's pattern (Petsc_mod.F90:629-743):
  a row of node r holds exactly the six unknowns of every node that shares an
  element with r, sorted, plus the arclength column when nex = 1, and the
  arclength row is dense;
* ``seeded_state`` draws the benchmark state: the masked parabolic inflow
  plus N(0, 0.01) noise, and SPD conformations (c = S^2 in the SQRT form,
  c = I + Wi/(1-beta) T in the T form); the same seed gives the same bits;
* ``boundary_conditions`` (setBoundaryEQs, Boundary_mod.F90:202-317):
  inlet u, v and stresses at the fully developed profile, outlet p = 0, walls
  and cylinder u = v = 0, each row once.
"""
import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import newton as N
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S


@pytest.mark.parametrize("nex", [0, 1])
def test_pattern_is_the_element_adjacency(nex):
    mesh = M.build_cylinder_mesh(40, exact=False)
    en = mesh.element_nodes()
    rowptr, colind = P.build_pattern(en, mesh.nnodes, nex)
    n_dof = mesh.nnodes * 6
    Nn = n_dof + nex
    assert rowptr.shape == (Nn + 1,) and rowptr[0] == 0 and rowptr[-1] == colind.size
    nbrs = [set() for _ in range(mesh.nnodes)]
    for e in range(mesh.nel):
        for a in en[e]:
            nbrs[a].update(en[e].tolist())
    for r in range(n_dof):
        cols = colind[rowptr[r]:rowptr[r + 1]]
        assert np.all(np.diff(cols) > 0)                       # sorted, unique
        expect = sorted(6 * b + q for b in nbrs[r // 6] for q in range(6))
        if nex:
            expect.append(n_dof)
        assert cols.tolist() == expect
    if nex:
        assert colind[rowptr[n_dof]:].tolist() == list(range(Nn))


def test_pattern_rejects_several_extra_unknowns():
    mesh = M.rect_mesh(2, 2)
    with pytest.raises(ValueError):
        P.build_pattern(mesh.element_nodes(), mesh.nnodes, 2)


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_seeded_state(form):
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, seed=3)
    TL2, _ = S.seeded_state(mesh.xyz, phys, seed=3)
    assert np.array_equal(TL, TL2)
    x, y = mesh.xyz[0], mesh.xyz[1]
    mask = np.clip((np.hypot(x, y) - 1.0) / 0.25, 0.0, 1.0)
    u0 = 1.5 * (1.0 - (y / 2.0) ** 2) * mask
    assert np.std(TL[0] - u0) == pytest.approx(0.01, rel=0.1)
    assert np.max(np.abs(TL[0] - u0)) < 0.07 and np.max(np.abs(TL[1])) < 0.07
    a, b, d = TL[3], TL[4], TL[5]
    if form == "SQRT":
        # c = S^2
        c11, c12, c22 = a * a + b * b, a * b + b * d, b * b + d * d
    else:
        k = phys.WiN / (1.0 - phys.BvN)
        c11, c12, c22 = 1.0 + k * a, k * b, 1.0 + k * d
    assert np.all(c11 > 0) and np.all(c11 * c22 - c12 * c12 > 0)
    # c = I + 0.1 A A^T with A ~ N(0, 0.1): trace - 2 ~ 0.1 * 4 * 0.01 on average
    assert np.mean(c11 + c22 - 2.0) == pytest.approx(0.004, rel=0.1)
    assert EU.tolist() == [1.0] and phys.Wi0 == phys.WiN


def test_boundary_rows():
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.3, 0.59, "SQRT", nex=1)
    rows, vals = N.boundary_conditions(mesh, phys)
    assert np.unique(rows).size == rows.size
    bn = mesh.boundary_nodes
    got = dict(zip(rows.tolist(), vals.tolist()))
    walls = set(bn["Wall"].tolist()) | set(bn["Cylinder"].tolist())
    for node in bn["Outlet"]:
        assert got[6 * node + 2] == 0.0
    for node in walls:
        assert got[6 * node] == 0.0 and got[6 * node + 1] == 0.0
    y = mesh.xyz[1]
    for node in bn["Inlet"]:
        if node in walls:
            continue           # the wall rows come later and win
        assert got[6 * node] == pytest.approx(1.5 * (1.0 - (y[node] / 2.0) ** 2), abs=1e-14)
        assert got[6 * node + 1] == 0.0
        for f in (3, 4, 5):
            assert 6 * node + f in got
        assert 6 * node + 2 not in got
    # Oldroyd-B fully developed inflow: c = [[1 + 2 (Wi g)^2, Wi g], [Wi g, 1]], g = du/dy
    node = bn["Inlet"][len(bn["Inlet"]) // 3]
    g = -3.0 * y[node] / 4.0
    c = np.array([[[1.0 + 2.0 * (0.3 * g) ** 2, 0.3 * g], [0.3 * g, 1.0]]])
    s = S.conformation_to_unknowns(c, phys)[:, 0]
    assert [got[6 * node + f] for f in (3, 4, 5)] == pytest.approx(s.tolist(), abs=1e-14)
