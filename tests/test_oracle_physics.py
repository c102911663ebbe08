"""Known-answer checks that pin the CPU oracle (a restatement of the reference
Fortran) to physics and to the reference's finite-difference semantics.

The reference ships no tests or golden vectors and cannot be built here
(Fortran + PETSc + MPI), so these are the oracle's pins:

* homogeneous-flow patch tests: a linear, divergence-free velocity with the
  constant stress that solves the textbook steady constitutive equation
  (Oldroyd-B, linear PTT, exponential PTT, Giesekus) in the conformation form
  ``-Wi (L c + c L^T) + F(c) = 0``, mapped to the reference's unknowns
  (T = (1-beta)/Wi (c - I) or S = c^(1/2)).  Every continuity and
  constitutive residual must vanish element by element, and the momentum
  residual must vanish at interior nodes after assembly;
* the forward-difference Jacobian, replayed column by column from plain
  residual evaluations with the reference's (x + eps) - eps restore
  (Equations_mod.F90:264-306), matches bit for bit;
* the FD Jacobian agrees with central differences;
* mirror symmetry y -> -y and invariance under translation.
"""
import numpy as np
import pytest
from scipy.optimize import fsolve

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S


def _homogeneous_conformation(model, eps, Wi, L):
    """Solve -Wi (L c + c L^T) + F(c) = 0 for symmetric 2x2 c (2-D, N = 2)."""
    I = np.eye(2)

    def F(c):
        tr = np.trace(c)
        if model == "L-PTT":
            return (1.0 + eps * (tr - 2.0)) * (c - I)
        if model == "e-PTT":
            return np.exp(eps * (tr - 2.0)) * (c - I)
        if model == "GIESEKUS":
            return (c - I) + eps * (c - I) @ (c - I)
        raise ValueError(model)

    def f(v):
        c = np.array([[v[0], v[1]], [v[1], v[2]]])
        r = -Wi * (L @ c + c @ L.T) + F(c)
        return [r[0, 0], r[0, 1], r[1, 1]]

    v = fsolve(f, [1.0, 0.0, 1.0], xtol=1e-15)
    c = np.array([[v[0], v[1]], [v[1], v[2]]])
    assert np.max(np.abs(f(v))) < 1e-13
    return c


def _affine_mesh():
    """Parallelogram elements: the reference's second derivatives
    (basis2D, Element_Calculations_mod.F90:352-355) drop the map's curvature
    terms, so a linear field has zero Laplacian only on affine elements."""
    mesh = M.rect_mesh(3, 3, -1.0, 2.0, -1.0, 1.5)
    A = np.array([[1.1, 0.35], [-0.2, 0.9]])
    xy = A @ mesh.xyz[:2] + np.array([[0.3], [-0.1]])
    mesh.xyz[:2] = xy
    return mesh


CASES = [("L-PTT", 0.0, "T"), ("L-PTT", 0.0, "SQRT"), ("L-PTT", 0.05, "T"),
         ("L-PTT", 0.05, "SQRT"), ("e-PTT", 0.05, "T"), ("e-PTT", 0.05, "SQRT"),
         ("GIESEKUS", 0.1, "T"), ("GIESEKUS", 0.1, "SQRT")]


@pytest.mark.parametrize("model,eps,form", CASES)
def test_homogeneous_flow_patch(model, eps, form):
    Wi, beta = 0.3, 0.59
    phys = S.Physics(model=model, form=form, WiN=Wi, Wi0=Wi, BvN=beta, VeN=eps, nex=0)
    # L_ij = du_i/dx_j, traceless
    L = np.array([[0.3, 0.5], [-0.2, -0.3]])
    c = _homogeneous_conformation(model, eps, Wi, L)
    mesh = _affine_mesh()
    x, y = mesh.xyz[0], mesh.xyz[1]
    n = mesh.nnodes
    TL = np.zeros((6, n))
    TL[0] = 0.7 + L[0, 0] * x + L[0, 1] * y
    TL[1] = -0.1 + L[1, 0] * x + L[1, 1] * y
    TL[2] = 0.0
    t = S.conformation_to_unknowns(np.repeat(c[None], n, axis=0), phys)
    TL[3:] = t
    res, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, np.zeros(0), jacobian=False)
    scale = np.max(np.abs(res[:, :, :2]))
    assert scale > 1e-3
    # continuity and constitutive residuals vanish element by element
    assert np.max(np.abs(res[:, :, 2:])) < 1e-12 * max(1.0, scale)
    # momentum vanishes at interior nodes after assembly
    rowptr, colind = P.build_pattern(mesh.element_nodes(), n, 0)
    b, _ = O.assemble(phys, mesh.conn, mesh.xyz, TL, np.zeros(0), rowptr, colind, jacobian=False)
    bnd = np.zeros(n, dtype=bool)
    for v in mesh.boundary_nodes.values():
        bnd[v] = True
    interior = np.nonzero(~bnd)[0]
    assert interior.size > 0
    bb = b.reshape(n, 6)
    # not 1e-12: the reference's 3-point rule has its centre point at 0 + 1e-8
    # (Gauss_Quadrangle_mod.F90:65,70), so integrals of grad(phi) carry O(1e-8) error
    assert np.max(np.abs(bb[interior, :2])) < 1e-7 * scale
    assert np.max(np.abs(bb[bnd, :2])) > 1e-6 * scale     # boundary tractions are not zero


def test_patch_detects_wrong_stress():
    """Sanity of the patch test itself: a stress off the constitutive solution
    leaves a constitutive residual."""
    Wi = 0.3
    phys = S.oldroyd_b(Wi, 0.59, "T", nex=0)
    mesh = M.rect_mesh(2, 2)
    L = np.array([[0.3, 0.5], [-0.2, -0.3]])
    c = _homogeneous_conformation("L-PTT", 0.0, Wi, L) + np.diag([0.01, 0.0])
    TL = np.zeros((6, mesh.nnodes))
    TL[0] = L[0, 0] * mesh.xyz[0] + L[0, 1] * mesh.xyz[1]
    TL[1] = L[1, 0] * mesh.xyz[0] + L[1, 1] * mesh.xyz[1]
    TL[3:] = S.conformation_to_unknowns(np.repeat(c[None], mesh.nnodes, axis=0), phys)
    res, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, np.zeros(0), jacobian=False)
    assert np.max(np.abs(res[:, :, 3:])) > 1e-4


def _single_element(seed=0, form="T", model="L-PTT", eps=0.0, nex=1):
    mesh = M.rect_mesh(1, 1, 0.0, 1.3, -0.2, 0.9, distort=0.4, seed=seed)
    phys = S.Physics(model=model, form=form, WiN=0.4, Wi0=0.4, BvN=0.59, VeN=eps, nex=nex)
    TL, EU = S.seeded_state(mesh.xyz + np.array([[2.0], [0.0], [0.0]]), phys, seed)
    return mesh, phys, TL, EU


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_fd_jacobian_replay_with_restore_residue(form):
    """The oracle's FD Jacobian equals a replay of storeBulk from single
    residual evaluations, including the (x+eps)-eps restore residue; values
    are chosen so that several restores do not give back x."""
    mesh, phys, TL, EU = _single_element(1, form)
    # values whose (x + eps) - eps != x: tiny numbers and numbers just below a power of two
    TL[2, 0] = 3.0e-13
    TL[2, 4] = 0.5 - 4.0e-9
    TL[4, 3] = -7.0e-12
    eps = phys.eps
    drift = (TL + eps) - eps
    assert np.count_nonzero(drift != TL) >= 3
    res0, jac, ac = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU)
    en = mesh.element_nodes()[0]
    cur = TL.copy()
    for inod in range(9):
        for ieq in range(6):
            g = en[inod]
            pert = cur.copy()
            pert[ieq, g] = cur[ieq, g] + eps
            r, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, pert, EU, jacobian=False)
            col = (r[0] - res0[0]) / eps
            assert np.array_equal(col, jac[0, inod, ieq]), (inod, ieq)
            cur[ieq, g] = (cur[ieq, g] + eps) - eps
    eu = EU.copy()
    eu[0] = EU[0] + eps
    r, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, cur, eu, jacobian=False)
    assert np.array_equal((r[0] - res0[0]) / eps, ac[0, :, :, 0])


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_fd_jacobian_matches_central_difference(form):
    mesh, phys, TL, EU = _single_element(2, form, "GIESEKUS", 0.1)
    res0, jac, ac = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU)
    en = mesh.element_nodes()[0]
    h = 1e-5
    scale = np.max(np.abs(jac))
    for inod, ieq in [(0, 0), (4, 1), (8, 2), (2, 3), (6, 4), (7, 5)]:
        tp = TL.copy()
        tm = TL.copy()
        tp[ieq, en[inod]] += h
        tm[ieq, en[inod]] -= h
        rp, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, tp, EU, jacobian=False)
        rm, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, tm, EU, jacobian=False)
        cd = (rp[0] - rm[0]) / (2 * h)
        assert np.max(np.abs(cd - jac[0, inod, ieq])) < 2e-5 * scale


def _mirror(mesh):
    """y -> -y with the element node order re-labelled so every map stays
    counter-clockwise: local (xi, eta) -> (xi, -eta)."""
    perm = [3, 2, 1, 0, 6, 5, 4, 7, 8]
    conn = np.ascontiguousarray(mesh.conn[perm])
    xyz = mesh.xyz.copy()
    xyz[1] = -xyz[1]
    return conn, xyz


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_mirror_symmetry(form):
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 4)
    sel = np.arange(0, mesh.nel, 97)
    res, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU, jacobian=False)
    conn_m, xyz_m = _mirror(mesh)
    TLm = TL.copy()
    TLm[1] = -TLm[1]
    TLm[4] = -TLm[4]
    resm, _, _ = O.element_outputs(phys, conn_m, xyz_m, TLm, EU, jacobian=False)
    perm = [3, 2, 1, 0, 6, 5, 4, 7, 8]
    sign = np.array([1, -1, 1, 1, -1, 1])
    scale = np.max(np.abs(res))
    # mirroring maps the 0 + 1e-8 quadrature point to -1e-8, which is not in the rule,
    # so the mirrored residual agrees to O(1e-8), not to rounding
    for e in sel:
        assert np.max(np.abs(resm[e] - res[e][perm] * sign)) < 1e-7 * scale


def test_translation_invariance():
    mesh = M.rect_mesh(2, 2, 0.0, 1.0, 0.0, 1.0, distort=0.3, seed=5)
    phys = S.giesekus(0.1, 0.5, 0.59, "T", nex=0)
    TL, EU = S.seeded_state(mesh.xyz + 1.5, phys, 5)
    res, _, _ = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU, jacobian=False)
    xyz2 = mesh.xyz.copy()
    xyz2[0] += 0.25
    xyz2[1] -= 0.5
    res2, _, _ = O.element_outputs(phys, mesh.conn, xyz2, TL, EU, jacobian=False)
    assert np.max(np.abs(res - res2)) < 1e-11 * np.max(np.abs(res))


def test_gauss_tables_partition_of_unity():
    t, w = O.gauss_tables()
    bfn, dfdc, dfde = t[0], t[1], t[2]
    assert np.allclose(bfn.sum(axis=1), 1.0, atol=1e-15)
    assert np.allclose(dfdc.sum(axis=1), 0.0, atol=1e-14)
    assert np.allclose(dfde.sum(axis=1), 0.0, atol=1e-14)
    assert abs(w.sum() - 4.0) < 1e-15
    # the 0 + 1e-8 "centre" point: basis of corner node 1 is tiny but not zero there
    assert 0 < abs(bfn[0, 0]) < 1e-8


def test_fd_jacobian_nan_at_exact_parallel_flow():
    """A quirk of the reference algorithm the restatement keeps: on element
    20478 of the 40,000-quad mesh at the fully developed Giesekus start
    (tests/golden/fd_nan_element.json, exact bits) the residual is finite but
    perturbing S12 at local nodes 1 and 3 by the FD step 1e-8 makes the
    residual NaN.  The SQRT form's LSCE coefficient holds the magnitude
    sqrt(0.5 Con_EQ : Con_EQ^T) with doubleDotProduct(A, B) = sum A_ij B_ji
    (Tools_mod.F90:262-278, Element_Calculations_mod.F90:762-768); Con_EQ
    vanishes for parallel flow, and after the perturbation the off-diagonal
    product of opposite signs dominates the sum, so the square root is of a
    negative number (here: tlsce NaN at the perturbed state)."""
    import json
    import os
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "fd_nan_element.json")))
    xyz = np.array([[float.fromhex(v) for v in r] for r in d["xyz"]])
    TL = np.array([[float.fromhex(v) for v in r] for r in d["TL"]])
    conn = np.arange(1, 10, dtype=np.int32).reshape(9, 1)
    phys = S.giesekus(0.1, 0.1, 0.59, "SQRT", nex=0)
    EU = np.zeros(0)
    res, jac, _ = O.element_outputs(phys, conn, xyz, TL, EU)
    assert np.all(np.isfinite(res))
    bad = np.argwhere(~np.isfinite(jac[0]))
    assert len(bad) == 90
    # the perturbed unknown (inod, ieq): S12 (field 4) of local nodes 1 and 3
    assert set(map(tuple, bad[:, :2])) == {(1, 4), (3, 4)}
    assert np.all(np.isfinite(O.gp_probe(phys, conn, xyz, TL, EU, 0)))
    TLp = TL.copy()
    TLp[4, 1] = TLp[4, 1] + 1.0e-8
    probe = O.gp_probe(phys, conn, xyz, TLp, EU, 0)
    assert np.all(np.isfinite(probe[:, 3:6]))          # Con_EQ 11/12/22 themselves finite
    assert np.any(np.isnan(probe[:, 8]))                # tlsce
