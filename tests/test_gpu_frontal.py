"""GPU panel-frontal LU (frontal.py + csrc/vefem_frontal.cu) on Jacobians the
library assembles: the unpivoted Gauss-Jordan elimination against SuperLU and
against the pivoted per-panel LU, reproducible solves, the refusal of a
failing pivot (pivoted path, then the host), and the arclength continuation
driven by it."""
import numpy as np
import pytest
import scipy.sparse as sp

from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import continuation as C
from ve_flow_around_cylinder_fortran_gb300 import frontal as FR
from ve_flow_around_cylinder_fortran_gb300 import linsolve as LS
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import newton as N
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _system(nel, jac="fd64", arclength=True, seed=0):
    """Jacobian and residual of a perturbed fully developed state, with the
    Dirichlet rows and the lambda row (a dense arclength row, or pinned)."""
    mesh = M.build_cylinder_mesh(nel)
    phys = S.oldroyd_b(0.5, 0.59, "SQRT", nex=1)
    rp, ci = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rp, ci, outlet_edges=True)
    rows, values = N.boundary_conditions(mesh, phys)
    TL, EU = N.initial_state(mesh, phys)
    TLs, _ = S.seeded_state(mesh.xyz, phys, seed)
    TL = TL + 0.01 * (TLs - TL)
    dev = N.DeviceAssembly(asm, rows, values, jac, True)
    b, vals = dev(TL, EU, True)
    asm.close()
    lrow = C.LambdaRow(rp, ci)
    x = np.concatenate([TL.T.reshape(-1), EU])
    if arclength:
        rng = np.random.default_rng(seed)
        t = rng.standard_normal(len(x))
        lrow.mode, lrow.t, lrow.x_o, lrow.dS = "arclength", t / np.linalg.norm(t), x * 0.99, 0.1
    else:
        lrow.mode, lrow.target = "pinned", 1.0
    lrow(x, b, vals)
    A = sp.csr_matrix((vals, ci, rp), shape=(len(rp) - 1,) * 2)
    return mesh, rp, ci, vals, b, A


@pytest.mark.parametrize("arclength", [True, False])
@pytest.mark.parametrize("jac", ["fd64", "exact32"])
def test_native_frontal_matches_superlu_2000(jac, arclength):
    mesh, rp, ci, vals, b, A = _system(2000, jac, arclength)
    lu = FR.FrontalLU(rp, ci, mesh)
    lu.factor(vals)
    assert lu.mode == "native" and lu.fallbacks == 0
    x = lu.solve(b)
    x_ref = LS.SparseLU(rp, ci, mesh).factor(vals).solve(b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    # the same solve again: bit for bit (fixed summation order, no atomics)
    assert np.array_equal(lu.solve(b), x)
    assert lu.solve_path in (1, 2)
    lu.close()


@pytest.mark.parametrize("panel", [4, 16, 40])
def test_native_frontal_panel_sizes(panel):
    mesh, rp, ci, vals, b, A = _system(2000, "fd64", True, seed=3)
    lu = FR.FrontalLU(rp, ci, mesh, panel=panel).factor(vals)
    piv = FR.FrontalLU(rp, ci, mesh, panel=panel, method="pivoted").factor(vals)
    x, xp = lu.solve(b), piv.solve(b)
    assert lu.mode == "native" and piv.mode == "pivoted"
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert np.linalg.norm(x - xp) <= 1e-9 * np.linalg.norm(xp)
    assert 0.0 < lu.min_pivot <= 1.0
    lu.close()


def test_failing_pivot_is_refused():
    """A row that is zero except in the border column: the pivot block of its
    panel is singular, the unpivoted elimination refuses it (also after the
    symbolic phase is redone with delayed pressures), the pivoted path finds
    the same and the host SuperLU solves the bordered system."""
    mesh, rp, ci, vals, b, A = _system(500, "fd64", True)
    N_ = len(rp) - 1
    k = int(mesh.boundary_nodes["Wall"][5]) * 6
    s0, s1 = rp[k], rp[k + 1]
    vals[s0:s1] = (ci[s0:s1] == N_ - 1).astype(float)
    A = sp.csr_matrix((vals, ci, rp), shape=(N_, N_))
    lu = FR.FrontalLU(rp, ci, mesh).factor(vals)
    x = lu.solve(b)
    assert lu.resymbolised and lu.pivoted_factorisations == 2 and lu.fallbacks == 1
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    lu.close()


def test_arclength_continuation_with_frontal_solver():
    """The same continuation with the GPU frontal LU and with SuperLU: the
    same number of steps and Newton iterations, every point converged, and the
    points within 1e-6 of each other (the tangents, and hence the arclength
    steps, differ in the last bits, which moves each point along the branch
    by a few parts in 1e9 of the state)."""
    mesh = M.build_cylinder_mesh(300, exact=False)
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    TL, EU = N.initial_state(mesh, phys)
    rp, ci = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rp, ci, outlet_edges=True)
    cfg = C.ArclengthSettings(dArN=0.01, max_steps=12)
    runs = {}
    for solver in ("superlu", "frontal"):
        cont = C.ArclengthContinuation(asm, mesh, phys, "fd64", cfg, linear_solver=solver)
        runs[solver] = cont.run(TL, EU)
    asm.close()
    (r1, x1), (r2, x2) = runs["superlu"], runs["frontal"]
    assert len(r1) == len(r2) == 12
    assert [r.newton_iterations for r in r1] == [r.newton_iterations for r in r2]
    assert all(r.res_norm < 1e-10 for r in r2)
    for a, c in zip(x1, x2):
        assert np.linalg.norm(a - c) <= 1e-6 * np.linalg.norm(a)
