"""Host logic of the arclength driver on the oracle assembly (no GPU): a
Newton step whose Jacobian cannot be factorised (SuperLU: exactly singular)
or whose residual is not finite fails that solve, and the emergency restart
(relaxation halved, emergencyNewtonRaphson) converges to the same point."""
import types

import numpy as np
import pytest

from oracle_assembly import OracleAssembly
from ve_flow_around_cylinder_fortran_gb300 import continuation as C
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import newton as N
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    from oracle import oracle as O
    O.build()


def _driver(max_steps=2):
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    mesh = M.build_cylinder_mesh(40, exact=False)
    TL, EU = N.initial_state(mesh, phys)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    rows, values = N.boundary_conditions(mesh, phys)
    asm = types.SimpleNamespace(rowptr=rowptr, colind=colind, N=len(rowptr) - 1,
                                nnodes=mesh.nnodes)
    oa = OracleAssembly(phys, mesh, rowptr, colind, rows, values)
    cfg = C.ArclengthSettings(dArN=0.01, max_steps=max_steps)
    return C.ArclengthContinuation(asm, mesh, phys, "fd64", cfg, assembly=oa), TL, EU


def test_singular_factorisation_restarts_newton():
    ref, TL, EU = _driver()
    r0, x0 = ref.run(TL, EU)
    cont, TL, EU = _driver()
    orig = cont.solver.factor
    calls = {"n": 0}

    def factor(vals):
        calls["n"] += 1
        if calls["n"] == 2:
            raise RuntimeError("Factor is exactly singular")
        return orig(vals)

    cont.solver.factor = factor
    r1, x1 = cont.run(TL, EU)
    assert cont.failed_factorisations == 1
    assert r1[0].emergencies == 1 and r0[0].emergencies == 0
    for a, b in zip(x0, x1):
        assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(a))
    assert all(r.res_norm < 1e-10 for r in r1)


def test_non_finite_residual_restarts_newton():
    cont, TL, EU = _driver(max_steps=1)
    orig = cont.dev
    calls = {"n": 0}

    def assemble(TL_, EU_, want):
        calls["n"] += 1
        b, v = orig(TL_, EU_, want)
        if calls["n"] == 2:
            b[0] = np.nan
        return b, v

    cont.dev = assemble
    cont.dev.set_values = orig.set_values
    r, x = cont.run(TL, EU)
    assert r[0].emergencies == 1 and r[0].res_norm < 1e-10


def test_persistent_singularity_stops_with_an_error():
    cont, TL, EU = _driver(max_steps=1)

    def factor(vals):
        raise RuntimeError("Factor is exactly singular")

    cont.solver.factor = factor
    with pytest.raises(RuntimeError, match="Newton failed at increment 1"):
        cont.run(TL, EU)
    assert cont.failed_factorisations == 7       # xF = 1, 1/2, ..., 1/64


def _branch_dev(xa, xb):
    """Largest relative distance of the points xb from the branch through the
    points xa (linear interpolation in lambda)."""
    la = np.array([x[-1] for x in xa])
    dev = 0.0
    for x in xb[1:-1]:
        k = int(np.searchsorted(la, x[-1]))
        if 0 < k < len(la):
            w = (x[-1] - la[k - 1]) / (la[k] - la[k - 1])
            ref = (1 - w) * xa[k - 1] + w * xa[k]
            dev = max(dev, float(np.linalg.norm(x - ref) / np.linalg.norm(ref)))
    return dev


def test_contraction_reuse_converges_on_the_same_branch_with_fewer_factorisations():
    """The chord policy (factorisations kept across steps while the chord
    iterations contract) converges every point to ||R|| < 1e-10 on the
    branch of the reference policy, with the reduced-space predictor, and
    factorises less often."""
    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    out = {}
    for reuse in ("reference", "contraction"):
        cont, TL, EU = _driver(max_steps=400)
        cont.cfg = C.ArclengthSettings(dArN=0.01, max_steps=400, lam_max=6.0, reuse=reuse,
                                       theta_max=0.6, factor_cost=30.0)
        pred = LP.LearnedPredictor(n_modes=32, start=20, device="cpu", net=object(),
                                   use_net=False)
        recs, xs = cont.run(TL, EU, predictor=pred)
        assert all(r.res_norm < 1e-10 for r in recs)
        assert recs[-1].lam >= 6.0
        out[reuse] = (sum(r.factorisations for r in recs), xs)
    assert out["contraction"][0] < out["reference"][0]
    # chord iterations converge to the same points as Newton: branch agreement
    # limited by the linear interpolation between the reference points
    assert _branch_dev(out["reference"][1], out["contraction"][1]) < 1e-3


def test_newton_krylov_corrections_stay_on_the_branch():
    """Newton-Krylov corrections in place of factorisations (GMRES on the
    Jacobian at the iterate, preconditioned by the older factorisation):
    every point converged to ||R|| < 1e-10 on the branch of the chord-only
    run, GMRES used, and no more factorisations than the chord-only run."""
    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    out = {}
    for krylov in (0, 10):
        cont, TL, EU = _driver(max_steps=400)
        cont.cfg = C.ArclengthSettings(dArN=0.01, max_steps=400, lam_max=6.0,
                                       reuse="contraction", theta_max=0.6, factor_cost=30.0,
                                       krylov=krylov)
        pred = LP.LearnedPredictor(n_modes=32, start=20, device="cpu", net=object(),
                                   use_net=False)
        recs, xs = cont.run(TL, EU, predictor=pred)
        assert all(r.res_norm < 1e-10 for r in recs)
        assert recs[-1].lam >= 6.0
        out[krylov] = (sum(r.factorisations for r in recs), xs, cont.krylov_iterations)
    assert out[10][2] > 0 and out[0][2] == 0
    assert out[10][0] <= out[0][0]
    assert _branch_dev(out[0][1], out[10][1]) < 1e-3


def test_contraction_reuse_far_start_takes_newton_steps():
    """From the far initial state the chord policy takes full Newton steps
    while the correction is above MNR_eps, as the reference does, and
    converges the first point without an emergency restart."""
    cont, TL, EU = _driver(max_steps=1)
    cont.cfg = C.ArclengthSettings(dArN=0.01, max_steps=1, reuse="contraction", theta_max=0.6,
                                   factor_cost=30.0)
    recs, xs = cont.run(TL, EU)
    ref, TL, EU = _driver(max_steps=1)
    r0, x0 = ref.run(TL, EU)
    assert recs[0].emergencies == 0 and recs[0].res_norm < 1e-10
    assert np.max(np.abs(xs[0] - x0[0])) <= 1e-8 * np.max(np.abs(x0[0]))


def test_unknown_reuse_policy_is_rejected():
    cont, TL, EU = _driver(max_steps=1)
    with pytest.raises(ValueError, match="reuse policy"):
        C.ArclengthContinuation(cont.asm, cont.mesh, cont.phys, "fd64",
                                C.ArclengthSettings(reuse="sometimes"), assembly=cont.dev)


def test_step_cutback_predicts_again_at_half_the_step():
    """With cutbacks enabled a failed arclength solve halves dS and predicts
    again from the last converged point (no relaxation); the step converges
    on the arclength plane of the halved step."""
    cont, TL, EU = _driver(max_steps=5)
    cont.cfg = C.ArclengthSettings(dArN=0.01, max_steps=5, reuse="contraction", theta_max=0.6,
                                   factor_cost=30.0, cutbacks=2)
    orig = cont._newton
    calls = {"n": 0, "x0": []}

    def newton(x0, *a, **kw):
        calls["n"] += 1
        calls["x0"].append(x0.copy())
        if calls["n"] == 4:                  # the first solve of increment 4
            return x0, 1, 0, 1.0, None, False
        return orig(x0, *a, **kw)

    cont._newton = newton
    recs, xs = cont.run(TL, EU)
    r4 = recs[3]
    assert r4.cutbacks == 1 and r4.emergencies == 0 and r4.res_norm < 1e-10
    # the plain predictions x_o + t dS: the second lies half as far from the
    # last converged point, along the same unit tangent
    x3 = xs[2]
    d1 = np.linalg.norm(calls["x0"][3] - x3)
    d2 = np.linalg.norm(calls["x0"][4] - x3)
    assert d2 == pytest.approx(0.5 * d1, rel=1e-12)
    assert r4.dS == pytest.approx(d2, rel=1e-12)
    # the converged point lies on the halved step's arclength plane
    t = (calls["x0"][4] - x3) / d2
    assert abs(np.dot(t, xs[3] - x3) - r4.dS) <= 1e-8 * r4.dS


class _GarbagePredictor:
    """A predictor whose candidates are garbage: one not finite, one far off."""

    def __init__(self):
        self.calls = 0

    def observe(self, k, x, wi):
        pass

    def candidates(self, k, x_o, t, dS, x_plain):
        self.calls += 1
        bad = x_plain.copy()
        bad[::7] = np.nan
        far = x_plain + 10.0
        return [("learned", bad), ("extrapolation", far)]


def test_garbage_predictions_are_rejected_by_the_residual_judge():
    """Newton judges the candidates by residual norm: garbage from the
    predictor (NaN entries, a far-off state) is never taken, and the run
    equals the one without a predictor bit for bit."""
    ref, TL, EU = _driver(max_steps=6)
    r0, x0 = ref.run(TL, EU)
    cont, TL, EU = _driver(max_steps=6)
    pred = _GarbagePredictor()
    r1, x1 = cont.run(TL, EU, predictor=pred)
    assert pred.calls == 4                              # increments 3..6
    assert all(r.predictor == "plain" for r in r1)
    assert len(r0) == len(r1)
    for a, b in zip(x0, x1):
        assert np.array_equal(a, b)


def test_natural_continuation_extrapolation_is_lagrange_in_wi():
    """The start of the next natural-continuation point: exact for states
    that are polynomials of degree <= 2 in Wi, from the last three points."""
    rng = np.random.default_rng(0)
    a, b, c = (rng.standard_normal((6, 5)) for _ in range(3))
    f = lambda w: a + b * w + c * w * w                           # noqa: E731
    ws = [0.1, 0.2, 0.3, 0.4]
    X = [f(w) for w in ws]
    assert np.allclose(N.extrapolate(ws, X, 0.55), f(0.55), rtol=0, atol=1e-12)
    # two points: the secant
    assert np.allclose(N.extrapolate(ws[:2], X[:2], 0.3), 2 * X[1] - X[0], atol=1e-12)


def test_emergency_restarts_are_bounded():
    """emergencyNewtonRaphson halves the relaxation until xF < 1e-2; with
    max_restarts the caller bounds the number of restarts."""
    class Diverging:
        def __init__(self):
            self.calls = []

        def solve(self, TL, EU, xF=1.0, log=None, **kw):
            self.calls.append(xF)
            return N.NewtonResult(TL, EU, False, 1, [], 0.0, 0.0)

    nr = Diverging()
    res = N.emergency_solve(nr, np.zeros((6, 2)), np.zeros(0))
    assert not res.converged and nr.calls == [1.0, 0.5, 0.25, 0.125, 0.0625, 0.03125, 0.015625]
    nr = Diverging()
    N.emergency_solve(nr, np.zeros((6, 2)), np.zeros(0), max_restarts=1)
    assert nr.calls == [1.0, 0.5]
    nr = Diverging()
    N.emergency_solve(nr, np.zeros((6, 2)), np.zeros(0), max_restarts=0)
    assert nr.calls == [1.0]
