"""Pseudo-arclength continuation in Wi on the GPU assembly, and the learned
predictor against the tangent predictor it replaces.

* FD64 Jacobian: the continuation's iterates, step sizes and converged
  points equal the oracle-driven continuation's bit for bit (same residual
  and Jacobian bits, same host arithmetic).
* Learned predictor (cubic extrapolation in the POD space of the converged
  points, corrected by the library's MLP trained on the GPU): on the same
  branch it reaches the target Wi in fewer continuation steps and fewer
  Newton iterations than the tangent predictor, every point converged to
  ||R|| < 1e-10, and its branch agrees with the tangent run's.
"""
import numpy as np
import pytest

from oracle_assembly import OracleAssembly
from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import continuation as C
from ve_flow_around_cylinder_fortran_gb300 import learned as LP
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


def _setup(nel, phys):
    mesh = M.build_cylinder_mesh(nel, exact=False)
    TL, EU = N.initial_state(mesh, phys)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    return mesh, TL, EU, rowptr, colind


def test_gpu_arclength_equals_oracle_arclength():
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    mesh, TL, EU, rowptr, colind = _setup(150, phys)
    cfg = C.ArclengthSettings(dArN=0.01, max_steps=6)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    gpu = C.ArclengthContinuation(asm, mesh, phys, "fd64", cfg)
    r1, x1 = gpu.run(TL, EU)
    rows, values = N.boundary_conditions(mesh, phys)
    oa = OracleAssembly(phys, mesh, rowptr, colind, rows, values)
    cpu = C.ArclengthContinuation(asm, mesh, phys, "fd64", cfg, assembly=oa)
    r2, x2 = cpu.run(TL, EU)
    asm.close()
    assert len(r1) == len(r2) == 6
    for a, b in zip(r1, r2):
        assert (a.newton_iterations, a.factorisations, a.dS, a.lam, a.res_norm) == \
            (b.newton_iterations, b.factorisations, b.dS, b.lam, b.res_norm)
    for a, b in zip(x1, x2):
        assert np.array_equal(a, b)
    assert r1[-1].lam > 1.0


def _branch_lambda_interp(states, lam):
    """State on a branch at parameter lam by linear interpolation between the
    two converged points around it."""
    ls = np.array([s[-1] for s in states])
    k = int(np.searchsorted(ls, lam))
    w = (lam - ls[k - 1]) / (ls[k] - ls[k - 1])
    return (1 - w) * states[k - 1] + w * states[k]


def test_learned_predictor_gains_over_tangent():
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    mesh, TL, EU, rowptr, colind = _setup(300, phys)
    cfg = C.ArclengthSettings(dArN=0.01, lam_max=4.0, max_steps=400)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    plain = C.ArclengthContinuation(asm, mesh, phys, "exact32", cfg)
    rp, xp = plain.run(TL, EU)
    learn = C.ArclengthContinuation(asm, mesh, phys, "exact32", cfg)
    pred = LP.LearnedPredictor(n_modes=32, start=20)
    rl, xl = learn.run(TL, EU, predictor=pred)
    asm.close()
    pred.net.close()
    assert rp[-1].lam >= 4.0 and rl[-1].lam >= 4.0
    assert all(r.res_norm < 1e-10 for r in rp + rl)
    used = sum(r.predictor in ("learned", "extrapolation") for r in rl)
    steps_p, steps_l = len(rp), len(rl)
    newton_p = sum(r.newton_iterations for r in rp)
    newton_l = sum(r.newton_iterations for r in rl)
    print(f"tangent: {steps_p} steps, {newton_p} Newton iterations; "
          f"learned: {steps_l} steps, {newton_l} Newton iterations, learned prediction "
          f"taken {used} times")
    assert used >= 0.5 * (steps_l - pred.predict_from)
    assert steps_l < steps_p and newton_l < newton_p
    # the learned run's points lie on the tangent run's branch
    for x in xl[1:-1]:
        ref = _branch_lambda_interp(xp, x[-1])
        # linear interpolation between tangent-run points of relative step ~ 1e-2
        assert np.linalg.norm(x - ref) <= 2e-3 * np.linalg.norm(ref)
