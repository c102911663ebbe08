"""Host sparse LU stand-in (linsolve.py): nested-dissection order, solves, and
the partial-pivoting fallback."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import linsolve as LS
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S


def test_nested_dissection_is_a_permutation():
    mesh = M.build_cylinder_mesh(300, exact=False)
    order = LS.nested_dissection(mesh.xyz[:2], mesh.element_nodes(), mesh.nnodes)
    assert np.array_equal(np.sort(order), np.arange(mesh.nnodes))


def _jacobian(nel=200, nex=1):
    mesh = M.build_cylinder_mesh(nel, exact=False)
    phys = S.oldroyd_b(0.3, 0.59, "T", nex=nex)
    TL, EU = S.seeded_state(mesh.xyz, phys, seed=0)
    rp, ci = P.build_pattern(mesh.element_nodes(), mesh.nnodes, nex)
    b, v = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rp, ci)
    N = len(rp) - 1
    # Dirichlet-like unit rows on the walls' velocities and a pinned last unknown
    rows = [nd * 6 + q for nd in mesh.boundary_nodes["Wall"] for q in (0, 1)] + [N - 1]
    for r in rows:
        s0, s1 = rp[r], rp[r + 1]
        v[s0:s1] = (ci[s0:s1] == r).astype(float)
    return mesh, rp, ci, v, b


def test_nd_solve_matches_reference_solve():
    mesh, rp, ci, v, b = _jacobian()
    A = sp.csr_matrix((v, ci, rp), shape=(len(rp) - 1,) * 2)
    x_ref = spla.spsolve(A.tocsc(), b)
    lu = LS.SparseLU(rp, ci, mesh).factor(v)
    x = lu.solve(b)
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    plain = LS.SparseLU(rp, ci, None).factor(v)
    assert np.linalg.norm(plain.solve(b) - x_ref) <= 1e-9 * np.linalg.norm(x_ref)


def test_zero_diagonal_is_handled():
    """Unit entries off the diagonal in two rows (zero diagonal pivots)."""
    mesh, rp, ci, v, b = _jacobian(60, nex=0)
    N = len(rp) - 1
    r0 = mesh.boundary_nodes["Wall"][0] * 6
    for r, c in ((r0, r0 + 1), (r0 + 1, r0)):
        s0, s1 = rp[r], rp[r + 1]
        v[s0:s1] = (ci[s0:s1] == c).astype(float)
    A = sp.csr_matrix((v, ci, rp), shape=(N, N))
    x = LS.SparseLU(rp, ci, mesh).factor(v).solve(b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


def test_singular_diagonal_factor_falls_back(monkeypatch):
    """When the diagonal-pivot factorisation reports an exactly singular factor,
    the matrix is refactorised with partial pivoting."""
    mesh, rp, ci, v, b = _jacobian(60, nex=0)
    real = LS.spla.splu

    def splu(A, permc_spec=None, diag_pivot_thresh=None, **kw):
        if diag_pivot_thresh == 0.0:
            raise RuntimeError("Factor is exactly singular")
        assert permc_spec == "COLAMD" and diag_pivot_thresh is None
        return real(A, permc_spec=permc_spec, **kw)
    monkeypatch.setattr(LS.spla, "splu", splu)
    lu = LS.SparseLU(rp, ci, mesh).factor(v)
    assert lu.pivoted and lu.refactorisations == 1
    A = sp.csr_matrix((v, ci, rp), shape=(len(rp) - 1,) * 2)
    assert np.linalg.norm(A @ lu.solve(b) - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("kind", ["numpy", "torch"])
def test_gmres_with_an_inexact_preconditioner(kind):
    """Right-preconditioned GMRES with the LU of a perturbed matrix as the
    preconditioner reaches the requested relative residual; with too few
    iterations it reports the residual it reached."""
    rng = np.random.default_rng(0)
    n = 300
    A = (sp.random(n, n, density=0.02, random_state=1) + 4.0 * sp.eye(n)).tocsr()
    P_ = (A + 0.3 * sp.random(n, n, density=0.01, random_state=2)).tocsc()
    lu = spla.splu(P_)
    b = rng.standard_normal(n)
    if kind == "numpy":
        mv, pre, rhs, back = (lambda v: A @ v), lu.solve, b, (lambda x: x)
    else:
        torch = pytest.importorskip("torch")
        At = torch.sparse_csr_tensor(torch.from_numpy(A.indptr).long(),
                                     torch.from_numpy(A.indices).long(),
                                     torch.from_numpy(A.data), size=A.shape)
        mv = lambda v: At @ v                                        # noqa: E731
        pre = lambda v: torch.from_numpy(lu.solve(v.numpy()))       # noqa: E731
        rhs, back = torch.from_numpy(b), (lambda x: x.numpy())
    x, its, rel = LS.gmres(mv, pre, rhs, 1e-10, 40)
    x = back(x)
    assert rel <= 1e-10 and its < 40
    assert np.linalg.norm(A @ x - b) <= 1e-9 * np.linalg.norm(b)
    _, its2, rel2 = LS.gmres(mv, pre, rhs, 1e-14, 2)
    assert its2 == 2 and rel2 > 1e-14
