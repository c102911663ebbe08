"""Linear-stability A/B assembly on the GPU against the stability oracle.

The GPU builds the element blocks from the derivative of the perturbation
coefficients (exact for the linear perturbation residual) and forms A(k) for
all wavenumbers from its quadratic dependence on k; the oracle takes the
reference's forward differences at each k.  Both are the same linear
operator up to rounding: tolerance 1e-12 of the largest entry (all T-form
models: Oldroyd-B, Giesekus, FENE-CR, FENE-P).  The leading eigenvalues of the
Dirichlet-constrained pencil (A, B) near a shift agree within 1e-8 relative,
on a seeded state and on a converged Wi = 0.7 base state on 2,000 quads at
four wavenumbers.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import build as B_
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    B_.build()
    V.load()


def _case(nel=80, model="oldroyd_b"):
    mesh = M.build_cylinder_mesh(nel, exact=False)
    if model == "oldroyd_b":
        phys = S.oldroyd_b(0.7, 0.59, "T", nex=0)
    elif model == "giesekus":
        phys = S.giesekus(0.2, 0.5, 0.59, "T", nex=0)
    else:
        phys = S.Physics(model={"fene_cr": "FENE-CR", "fene_p": "FENE-P"}[model], form="T",
                         WiN=0.5, Wi0=0.5, BvN=0.59, VeN=40.0, nex=0)
    TL, _ = S.seeded_state(mesh.xyz, phys, seed=2)
    TLb = np.zeros((10, mesh.nnodes))
    TLb[0:2] = TL[0:2]
    TLb[3:7] = TL[2:6]
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 0)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    return mesh, phys, TLb, asm


def _oracle_csr(mesh, phys, TLb, k, kz=True):
    _, _, A, B = O.stability_elements(phys, mesh.conn, mesh.xyz, TLb,
                                      np.zeros_like(TLb), k, kz=kz)
    en = mesh.element_nodes()
    N = mesh.nnodes * 10
    inod, ieq, jnod, jeq = np.meshgrid(np.arange(9), np.arange(10), np.arange(9), np.arange(10),
                                       indexing="ij")
    rows = (en[:, jnod] * 10 + jeq).reshape(-1)
    cols = (en[:, inod] * 10 + ieq).reshape(-1)
    mk = lambda X: sp.csr_matrix((X.reshape(-1), (rows, cols)), shape=(N, N))
    return mk(A), mk(B)


def _gpu_csr(asm, rp, ci, vals):
    N = len(rp) - 1
    return sp.csr_matrix((vals, ci, rp), shape=(N, N))


@pytest.mark.parametrize("model", ["oldroyd_b", "giesekus", "fene_cr", "fene_p"])
def test_matrices_match_oracle(model):
    mesh, phys, TLb, asm = _case(model=model)
    rp, ci = asm.stability_pattern()
    kws = [0.0, 0.5, 1.7, 4.0]
    As, B = asm.stability_assemble(TLb, kws)
    for k, a in zip(kws, As):
        Ao, Bo = _oracle_csr(mesh, phys, TLb, k)
        Ag = _gpu_csr(asm, rp, ci, a)
        scale = abs(Ao).max()
        assert abs(Ag - Ao).max() <= 1e-12 * scale, k
        assert abs(_gpu_csr(asm, rp, ci, B) - Bo).max() <= 1e-12 * abs(Bo).max()
    asm.close()


def test_as_written_and_add_semantics():
    mesh, phys, TLb, asm = _case()
    rp, ci = asm.stability_pattern()
    As, B = asm.stability_assemble(TLb, [2.0], flags=V.VEFEM_ZERO_FIRST | V.VEFEM_STAB_AS_WRITTEN)
    Ao, _ = _oracle_csr(mesh, phys, TLb, 2.0, kz=False)
    assert abs(_gpu_csr(asm, rp, ci, As[0]) - Ao).max() <= 1e-12 * abs(Ao).max()
    # ADD: a second call without zeroing doubles the values
    As2, B2 = asm.stability_assemble(TLb, [2.0], flags=V.VEFEM_STAB_AS_WRITTEN,
                                     As=[As[0].copy()], B=B.copy())
    assert np.array_equal(As2[0], 2 * As[0]) and np.array_equal(B2, 2 * B)
    asm.close()


def _dirichlet(mesh, A, B):
    """applyDirichletBCStability: inlet and outlet all unknowns, walls and the
    cylinder the velocities; A row -> unit row, B row -> zero row."""
    bn = mesh.boundary_nodes
    rows = []
    for nd in np.concatenate([bn["Inlet"], bn["Outlet"]]):
        rows += [nd * 10 + q for q in range(10)]
    for nd in np.concatenate([bn["Wall"], bn["Cylinder"]]):
        rows += [nd * 10 + q for q in range(3)]
    rows = np.unique(rows)
    d = np.ones(A.shape[0])
    d[rows] = 0.0
    Dm = sp.diags(d)
    return (Dm @ A + sp.diags(1.0 - d)).tocsc(), (Dm @ B).tocsc()


def test_leading_eigenvalues_match_oracle():
    from scipy.sparse.linalg import eigs
    mesh, phys, TLb, asm = _case(nel=60)
    rp, ci = asm.stability_pattern()
    k = 1.3
    As, B = asm.stability_assemble(TLb, [k])
    Ag, Bg = _dirichlet(mesh, _gpu_csr(asm, rp, ci, As[0]), _gpu_csr(asm, rp, ci, B))
    Ao, Bo = _dirichlet(mesh, *_oracle_csr(mesh, phys, TLb, k))
    sigma = 0.3
    ev = []
    for A_, B_m in ((Ag, Bg), (Ao, Bo)):
        w = eigs(A_, k=6, M=B_m, sigma=sigma, which="LM", return_eigenvectors=False,
                 v0=np.ones(A_.shape[0]), tol=1e-12)
        ev.append(np.sort_complex(w))
    assert np.all(np.isfinite(ev[0]))
    assert np.max(np.abs(ev[0] - ev[1]) / np.abs(ev[1])) < 1e-8
    asm.close()


def test_converged_base_leading_eigenvalues_2000():
    """The stability configuration of the benchmark on a converged base state:
    Oldroyd-B, beta 0.59, T form, Wi = 0.7 reached by Newton solves at
    Wi 0.1, 0.3, 0.5, 0.6, 0.7 (||R|| < 1e-10) on 2,000 quads; A(k) and B for
    four spanwise wavenumbers from the GPU and from the oracle's forward
    differences, Dirichlet rows applied, the 10 eigenvalues nearest the shift
    of each pencil agree within 1e-8 relative."""
    from scipy.sparse.linalg import eigs
    from ve_flow_around_cylinder_fortran_gb300 import newton as N
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, "T", nex=0)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 0)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    res = N.natural_continuation(asm, mesh, phys, [0.1, 0.3, 0.5, 0.6, 0.7], jacobian="fd64",
                                 tol=1e-10, linear_solver="frontal")
    assert all(r.converged for r in res)
    TL = res[-1].TL
    TLb = np.zeros((10, mesh.nnodes))
    TLb[0:2] = TL[0:2]
    TLb[3:7] = TL[2:6]
    import dataclasses
    pb = dataclasses.replace(phys, WiN=0.7, Wi0=0.7)
    asm.set_params(pb)
    rp, ci = asm.stability_pattern()
    kws = [0.5, 1.5, 2.5, 3.5]
    As, B = asm.stability_assemble(TLb, kws)
    worst = 0.0
    for k, a in zip(kws, As):
        Ag, Bg = _dirichlet(mesh, _gpu_csr(asm, rp, ci, a), _gpu_csr(asm, rp, ci, B))
        Ao, Bo = _dirichlet(mesh, *_oracle_csr(mesh, pb, TLb, k))
        ev = []
        for A_, B_m in ((Ag, Bg), (Ao, Bo)):
            w = eigs(A_, k=10, M=B_m, sigma=0.2, which="LM", return_eigenvectors=False,
                     v0=np.ones(A_.shape[0]), tol=1e-13, maxiter=5000)
            ev.append(np.sort_complex(w))
        assert np.all(np.isfinite(ev[0]))
        rel = np.max(np.abs(ev[0] - ev[1]) / np.abs(ev[1]))
        worst = max(worst, rel)
        print(f"k = {k}: leading eigenvalues {ev[0][:3]} ..., max rel. diff {rel:.2e}")
    asm.close()
    assert worst < 1e-8


def test_unsupported_forms_are_errors():
    mesh = M.build_cylinder_mesh(40, exact=False)
    phys = S.oldroyd_b(0.7, 0.59, "SQRT", nex=0)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 0)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    with pytest.raises(V.VefemError):
        asm.stability_assemble(np.zeros((10, mesh.nnodes)), [1.0])
    asm.close()
