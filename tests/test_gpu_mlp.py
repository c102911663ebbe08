"""The learned predictor's network kernels against the numpy oracle.

The network (vefem_mlp_*) is checked piece by piece: its initial parameters
bit for bit, the forward pass, the gradient from the backward kernels and a
run of Adam iterations, against oracle/mlp_ref.py.  The GPU accumulates in
FP32 and the oracle in FP64 over the same BF16-rounded weights; tolerances are
relative to the largest entry and written per check.
"""
import numpy as np
import pytest

from oracle.mlp_ref import MLPRef
from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu

IN, OUT, WIDTH, HIDDEN = 98, 32, 256, 3


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, IN)).astype(np.float32)
    A = rng.standard_normal((IN, OUT)) / np.sqrt(IN)
    T = (np.tanh(X @ A) + 0.1 * rng.standard_normal((n, OUT))).astype(np.float32)
    return X, T


def _pair(seed=3):
    net = V.MLP(IN, OUT, width=WIDTH, hidden=HIDDEN, seed=seed)
    ref = MLPRef(IN, OUT, width=WIDTH, hidden=HIDDEN)
    ref.init_params(seed)
    return net, ref


def test_init_identical():
    net, ref = _pair()
    assert net.n_params == ref.n_params == 98 * 256 + 256 + 2 * (256 * 256 + 256) + 256 * 32 + 32
    assert np.array_equal(net.get_params(), ref.params)
    net.close()


def test_forward_matches_oracle():
    net, ref = _pair()
    X, _ = _problem(200, 0)
    y = net.forward(X)
    yr = ref.forward(X)
    # FP32 accumulation of 256-term products against FP64: 1e-5 of the largest output
    assert np.max(np.abs(y - yr)) <= 1e-5 * np.max(np.abs(yr))
    net.close()


def test_loss_and_gradient_reproducible():
    """The loss is reduced in a fixed order (no atomics): two evaluations on
    the same data give the same bits, loss and gradient."""
    net, _ = _pair(11)
    X, T = _problem(300, 2)
    l1, g1 = net.loss_grad(X, T)
    l2, g2 = net.loss_grad(X, T)
    assert l1 == l2
    assert np.array_equal(g1, g2)
    net.close()


def test_gradient_matches_oracle():
    net, ref = _pair(7)
    X, T = _problem(150, 1)
    loss, g = net.loss_grad(X, T)
    lr_, gr = ref.loss_grad(X, T)
    assert abs(loss - lr_) <= 1e-5 * lr_
    # per layer, gradient error below 1e-4 of that layer's largest gradient entry
    o = 0
    for i, n in ref.layers:
        for size in (i * n, n):
            a, b = g[o:o + size], gr[o:o + size]
            assert np.max(np.abs(a - b)) <= 1e-4 * np.max(np.abs(b)), (i, n, size)
            o += size
    net.close()


def test_adam_training_tracks_oracle():
    net, ref = _pair(5)
    X, T = _problem(120, 4)
    l0 = float(np.mean((ref.forward(X) - T) ** 2))
    # one iteration: identical update up to FP32 rounding of g, m and v
    net.train(X, T, 1, 1e-3)
    ref.train(X, T, 1, 1e-3)
    d = np.abs(net.get_params() - ref.params)
    _, g = ref.loss_grad(X, T)
    assert np.median(d) <= 1e-6
    assert np.max(d) <= 2.1e-3
    # 20 more iterations: the losses agree within 1 %
    lg = net.train(X, T, 20, 1e-3)
    lr_ = ref.train(X, T, 20, 1e-3)
    assert abs(lg - lr_) <= 0.01 * lr_
    # 200 more: both fitted (the trajectories are not compared this deep into
    # the fit, where FP32 and FP64 rounding steer them apart)
    lg = net.train(X, T, 200, 1e-3)
    lr_ = ref.train(X, T, 200, 1e-3)
    assert lg < 0.01 * l0 and lr_ < 0.01 * l0
    net.close()


def test_set_params_roundtrip_and_reset():
    net, ref = _pair(1)
    p = np.random.default_rng(0).standard_normal(net.n_params).astype(np.float32) * 0.05
    net.set_params(p)
    assert np.array_equal(net.get_params(), p)
    ref.set_params(p)
    X, _ = _problem(10, 9)
    assert np.max(np.abs(net.forward(X) - ref.forward(X))) <= 1e-5 * np.max(np.abs(ref.forward(X)))
    net.reset_optimizer()
    net.close()


def test_bad_arguments_are_errors():
    with pytest.raises(V.VefemError):
        V.MLP(0, 4)
    net = V.MLP(4, 2, width=8, hidden=1)
    with pytest.raises(ValueError):
        net.set_params(np.zeros(3, np.float32))
    with pytest.raises(ValueError):
        net.forward(np.zeros((2, 5), np.float32))
    net.close()
