"""CPU pins of the network oracle (oracle/mlp_ref.py) and of the learned
predictor's host logic (POD basis, samples, prediction) with the oracle
network standing in for the GPU one."""
import numpy as np
import pytest

from oracle.mlp_ref import MLPRef, bf16_round


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.1415926], np.float32)
    r = bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert r[4] == np.float32(3.140625)


def _loss64(ref, p, X, T):
    a = np.asarray(X, np.float64)
    L, o = [], 0
    for i, n in ref.layers:
        W = bf16_round(p[o:o + i * n].astype(np.float32)).astype(np.float64).reshape(n, i)
        o += i * n
        L.append((W, p[o:o + n]))
        o += n
    for k, (W, b) in enumerate(L):
        z = a @ W.T + b
        a = ref.gelu(z) if k + 1 < len(L) else z
    return float(np.mean((a - T) ** 2))


def test_gradient_is_derivative_of_loss():
    """Analytic bias gradients against central differences of the loss in
    float64; biases are not rounded to BF16, so the difference is smooth."""
    ref = MLPRef(6, 3, width=8, hidden=2)
    ref.init_params(11)
    X = np.random.default_rng(2).standard_normal((5, 6))
    T = np.ones((5, 3))
    _, g = ref.loss_grad(X, T)
    o = 0
    h = 1e-4
    for i, n in ref.layers:
        o += i * n
        for k in range(n):
            pp = ref.params.astype(np.float64)
            pm = pp.copy()
            pp[o + k] += h
            pm[o + k] -= h
            fd = (_loss64(ref, pp, X, T) - _loss64(ref, pm, X, T)) / (2 * h)
            assert abs(fd - g[o + k]) <= 1e-7 * max(1.0, abs(g[o + k]))
        o += n


def test_gelu_derivative():
    z = np.linspace(-4, 4, 81)
    h = 1e-6
    fd = (MLPRef.gelu(z + h) - MLPRef.gelu(z - h)) / (2 * h)
    assert np.max(np.abs(fd - MLPRef.gelu_prime(z))) < 1e-8


def test_init_is_deterministic_and_bounded():
    a = MLPRef(10, 4, width=16, hidden=2)
    b = MLPRef(10, 4, width=16, hidden=2)
    assert np.array_equal(a.init_params(3), b.init_params(3))
    assert not np.array_equal(a.params, b.init_params(4))
    W0, b0 = a.unpack()[0]
    assert np.all(np.abs(W0) <= np.sqrt(1 / 10)) and np.all(b0 == 0)


def test_adam_reduces_loss():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((40, 12))
    T = np.sin(X[:, :3])
    ref = MLPRef(12, 3, width=32, hidden=2)
    ref.init_params(0)
    l0 = ref.loss_grad(X, T)[0]
    l1 = ref.train(X, T, 300, 3e-3)
    assert l1 < 0.05 * l0


class _Curve:
    """A smooth synthetic solution branch x(s) in R^n with a scalar parameter."""

    def __init__(self, n=400, seed=0):
        rng = np.random.default_rng(seed)
        self.B = np.linalg.qr(rng.standard_normal((n, 6)))[0]
        self.c = rng.standard_normal(n)

    def __call__(self, s):
        f = np.array([s, 0.3 * s ** 2, np.sin(s), 0.1 * np.cos(2 * s), 0.05 * s ** 3, np.exp(-s)])
        return self.c + self.B @ f


def _feed(pred, curve, ss):
    for k, s in enumerate(ss, start=1):
        pred.observe(k, curve(s), 0.1 + 0.05 * s)


def test_pod_basis_and_coefficients():
    pytest.importorskip("torch")
    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    curve = _Curve()
    ref = MLPRef(2 + 3 * 8, 8, width=16, hidden=1)
    ref.init_params(0)
    pred = LP.LearnedPredictor(n_modes=8, start=10, net=ref, device="cpu", iters=5)
    _feed(pred, curve, np.linspace(0, 1.2, 12))
    mean, Phi = pred.basis
    Phi = Phi.numpy()
    assert Phi.shape[1] <= 6 + 1
    assert np.allclose(Phi.T @ Phi, np.eye(Phi.shape[1]), atol=1e-10)
    X = np.stack([x.numpy() for x in pred.X], axis=1)
    rec = mean.numpy()[:, None] + Phi @ pred.coef[:, :Phi.shape[1]].T
    assert np.allclose(rec, X, atol=1e-9 * np.abs(X).max())
    assert pred.trainings == 3


def test_learned_prediction_beats_tangent_on_smooth_branch():
    """Trained on the branch so far, the learned prediction of the next point
    is closer to the corrected point (the point of the branch on the
    arclength plane t . (x - x_o) = dS) than the tangent step it replaces."""
    pytest.importorskip("torch")
    from scipy.optimize import brentq

    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    curve = _Curve()
    ref = MLPRef(2 + 3 * 8, 8, width=64, hidden=3)
    ref.init_params(0)
    pred = LP.LearnedPredictor(n_modes=8, start=20, net=ref, device="cpu", iters=300, lr=1e-3)
    h = 0.08
    ss = np.cumsum(np.full(24, h))
    _feed(pred, curve, ss)
    x1, x0 = curve(ss[-1]), curve(ss[-2])
    dS = np.linalg.norm(x1 - x0)
    t = (x1 - x0) / dS
    x_plain = x1 + t * dS
    s_star = brentq(lambda s: t @ (curve(s) - x1) - dS, ss[-1], ss[-1] + 5 * h)
    truth = curve(s_star)
    cand = pred.predict(25, x1, t, dS, x_plain)
    assert pred.trainings == 5
    assert np.linalg.norm(cand - truth) < 0.2 * np.linalg.norm(x_plain - truth)


def test_trained_network_gains_over_extrapolation_alone():
    """What the network adds: on a smooth branch walked with the arclength
    plane, predictions of the next six points by the cubic extrapolation in
    the POD space with the trained network's correction are on average
    closer to the corrected points than the extrapolation alone (both
    candidates of the same predictor, the network retrained after each
    point)."""
    pytest.importorskip("torch")
    from scipy.optimize import brentq

    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    for h in (0.08, 0.12):
        curve = _Curve()
        ref = MLPRef(2 + 3 * 8, 8, width=64, hidden=3)
        ref.init_params(0)
        pred = LP.LearnedPredictor(n_modes=8, start=20, net=ref, device="cpu", iters=300,
                                   lr=1e-3, order=3)
        ss = list(np.cumsum(np.full(22, h)))
        _feed(pred, curve, ss)
        err = {"learned": [], "extrapolation": []}
        for k in range(23, 29):
            x1, x0 = curve(ss[-1]), curve(ss[-2])
            dS = np.linalg.norm(x1 - x0)
            t = (x1 - x0) / dS
            s_star = brentq(lambda s: t @ (curve(s) - x1) - dS, ss[-1], ss[-1] + 5 * h)
            truth = curve(s_star)
            cands = dict(pred.candidates(k, x1, t, dS, x1 + t * dS))
            assert set(cands) == {"learned", "extrapolation"}
            for name, x in cands.items():
                err[name].append(np.linalg.norm(x - truth) / np.linalg.norm(truth))
            ss.append(s_star)
            pred.observe(k, truth, 0.1 + 0.05 * s_star)
        assert np.mean(err["learned"]) < 0.7 * np.mean(err["extrapolation"]), (h, err)


def test_warm_up_leaves_the_predictor_unchanged():
    """warm_up runs the predictor's code path on synthetic snapshots and
    restores its state: the predictions after it equal those of a predictor
    that was never warmed up, bit for bit."""
    pytest.importorskip("torch")
    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    curve = _Curve()
    out = []
    for warm in (False, True):
        ref = MLPRef(2 + 3 * 8, 8, width=16, hidden=1)
        ref.init_params(0)
        pred = LP.LearnedPredictor(n_modes=8, start=10, net=ref, device="cpu", iters=5)
        if warm:
            pred.warm_up(400)
            assert pred.X == [] and pred.basis is None and pred.trainings == 0
            assert pred.use_net and pred.timers == {"pod": 0.0, "train": 0.0, "predict": 0.0}
        ss = list(np.linspace(0, 1.2, 12))
        _feed(pred, curve, ss)
        x1, x0 = curve(ss[-1]), curve(ss[-2])
        t = (x1 - x0) / np.linalg.norm(x1 - x0)
        out.append(pred.candidates(13, x1, t, 0.1, x1 + 0.1 * t))
    assert [n for n, _ in out[0]] == [n for n, _ in out[1]] == ["learned", "extrapolation"]
    for (_, a), (_, b) in zip(out[0], out[1]):
        assert np.array_equal(a, b)
