"""Algodiff registration of the conv/pool ops, checked on the CPU oracle in
float64: every registered op against central finite differences, a small
CNN end to end, the custom-op builders, and determinism.

FD error model: with eps = 1e-6 the central difference has truncation error
O(eps^2) and rounding error about 1e-16 * |f| / eps, so analytic and numeric
derivatives agree to about 1e-8 relative; the bound used is 1e-6."""

import numpy as np
import pytest

from owl_gb300.algodiff import (Algodiff, build_piso, check_grad, loss_and_grads, make_reverse,
                                primal, reverse_prop)

SAME, VALID = "SAME", "VALID"
EPS = 1e-6
TOL = 1e-6


@pytest.fixture(scope="module")
def ad(oracle_nn):
    return Algodiff(oracle_nn)


def _fd_check_op(fn, arrays, rng, n_idx=6):
    """Gradient of sum(fn(*arrays) * r) w.r.t. each array against FD."""
    out = primal(fn(*arrays))
    r = rng.standard_normal(out.shape)

    def loss(p):
        return float((primal(fn(*[p[k] for k in sorted(p)])) * r).sum())

    params = {i: a for i, a in enumerate(arrays)}
    nodes = {i: make_reverse(a) for i, a in params.items()}
    y = fn(*[nodes[k] for k in sorted(nodes)])
    reverse_prop(r, y)
    grads = {i: n.adj for i, n in nodes.items()}
    for i, a in params.items():
        idx = rng.choice(a.size, size=min(n_idx, a.size), replace=False)
        err, _ = check_grad(loss, params, grads, i, idx, EPS)
        assert err <= TOL, (i, err)


CONV_CASES = [
    ("conv1d", (2, 9, 3), (3, 3, 4), lambda N: lambda x, w: N.conv1d(x, w, [2], SAME)),
    ("conv2d", (2, 7, 6, 3), (3, 2, 3, 4), lambda N: lambda x, w: N.conv2d(x, w, [1, 2], SAME)),
    ("conv2d_valid", (2, 7, 6, 3), (3, 3, 3, 2),
     lambda N: lambda x, w: N.conv2d(x, w, [2, 1], VALID)),
    ("conv3d", (1, 5, 4, 5, 2), (2, 3, 2, 2, 3),
     lambda N: lambda x, w: N.conv3d(x, w, [1, 1, 2], SAME)),
    ("dilated_conv1d", (2, 11, 2), (3, 2, 3),
     lambda N: lambda x, w: N.dilated_conv1d(x, w, [1], [1, 2], SAME)),
    ("dilated_conv2d", (2, 8, 7, 2), (3, 3, 2, 3),
     lambda N: lambda x, w: N.dilated_conv2d(x, w, [1, 1], [2, 2], SAME)),
    ("dilated_conv3d", (1, 6, 5, 6, 2), (2, 2, 2, 2, 2),
     lambda N: lambda x, w: N.dilated_conv3d(x, w, [1, 1, 1], [2, 1, 2], VALID)),
    ("transpose_conv1d", (2, 5, 3), (3, 3, 2),
     lambda N: lambda x, w: N.transpose_conv1d(x, w, [2], SAME)),
    ("transpose_conv2d", (2, 4, 5, 3), (3, 3, 3, 2),
     lambda N: lambda x, w: N.transpose_conv2d(x, w, [2, 2], VALID)),
    ("transpose_conv3d", (1, 3, 4, 3, 2), (2, 2, 2, 2, 3),
     lambda N: lambda x, w: N.transpose_conv3d(x, w, [2, 2, 2], SAME)),
]


@pytest.mark.parametrize("case", CONV_CASES, ids=[c[0] for c in CONV_CASES])
def test_conv_ops_match_finite_differences(ad, case):
    _, xs, ws, make = case
    rng = np.random.default_rng(31)
    x = rng.uniform(-1, 1, xs)
    w = rng.uniform(-1, 1, ws)
    _fd_check_op(make(ad.NN), [x, w], rng)


POOL_CASES = [
    ("max_pool1d", (2, 9, 3), lambda N: lambda x: N.max_pool1d(SAME, x, [3], [2])),
    ("avg_pool1d", (2, 9, 3), lambda N: lambda x: N.avg_pool1d(VALID, x, [2], [2])),
    ("max_pool2d", (2, 7, 6, 3), lambda N: lambda x: N.max_pool2d(SAME, x, [3, 2], [2, 2])),
    ("avg_pool2d", (2, 7, 6, 3), lambda N: lambda x: N.avg_pool2d(SAME, x, [3, 3], [2, 1])),
    ("max_pool3d", (1, 5, 4, 6, 2), lambda N: lambda x: N.max_pool3d(VALID, x, [2, 2, 2],
                                                                     [2, 2, 2])),
    ("avg_pool3d", (1, 5, 4, 6, 2), lambda N: lambda x: N.avg_pool3d(SAME, x, [2, 3, 2],
                                                                     [1, 2, 2])),
    ("upsampling2d", (2, 3, 4, 3), lambda N: lambda x: N.upsampling2d(x, [2, 3])),
]


@pytest.mark.parametrize("case", POOL_CASES, ids=[c[0] for c in POOL_CASES])
def test_pool_ops_match_finite_differences(ad, case):
    _, xs, make = case
    rng = np.random.default_rng(32)
    x = rng.uniform(-1, 1, xs)  # distinct values: no ties within eps
    _fd_check_op(make(ad.NN), [x], rng)


def test_pool_forward_mode_fails_like_owl(ad):
    from owl_gb300.algodiff import _Siso

    with pytest.raises(NotImplementedError, match="max_pool2d:df"):
        _Siso("max_pool2d", None, None).df(None, None, None)


def _small_cnn(ad, p, x, onehot):
    M, N = ad.Maths, ad.NN
    h = M.relu(M.add(N.conv2d(x, p["w1"], [1, 1], SAME), p["b1"]))
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = M.relu(M.add(N.conv2d(h, p["w2"], [1, 1], SAME), p["b2"]))
    h = N.avg_pool2d(VALID, h, [2, 2], [2, 2])
    h = M.reshape(h, (primal(h).shape[0], 3 * 3 * 6))
    z = M.add(M.dot(h, p["w3"]), p["b3"])
    return M.softmax_cross_entropy(z, onehot)


def _small_params(rng):
    shapes = {"w1": (3, 3, 1, 4), "b1": (4,), "w2": (3, 3, 4, 6), "b2": (6,),
              "w3": (54, 10), "b3": (10,)}
    return {k: rng.standard_normal(s) * (0.5 if k.startswith("w") else 0.1)
            for k, s in shapes.items()}


def test_small_cnn_gradients_match_finite_differences(ad):
    rng = np.random.default_rng(33)
    params = _small_params(rng)
    x = rng.uniform(0, 1, (4, 12, 12, 1))
    onehot = np.eye(10)[rng.integers(0, 10, 4)]
    _, grads = loss_and_grads(ad, params, x, onehot, model=_small_cnn)

    def loss(p):
        return _small_cnn(ad, p, x, onehot)

    for name in params:
        idx = rng.choice(params[name].size, size=min(8, params[name].size), replace=False)
        err, _ = check_grad(loss, params, grads, name, idx, EPS)
        assert err <= TOL, (name, err)


def test_gradients_are_deterministic(ad):
    rng = np.random.default_rng(34)
    params = _small_params(rng)
    x = rng.uniform(0, 1, (3, 12, 12, 1))
    onehot = np.eye(10)[rng.integers(0, 10, 3)]
    _, g1 = loss_and_grads(ad, params, x, onehot, model=_small_cnn)
    _, g2 = loss_and_grads(ad, params, x, onehot, model=_small_cnn)
    for k in g1:
        assert np.array_equal(g1[k], g2[k])


def test_custom_piso_registration():
    """A user op registered with build_piso, like Owl's
    examples/custom_algodiff_op.ml: f(a, b) = a * b elementwise."""

    class Mul:
        label = "mul"

        @staticmethod
        def ff_bb(a, b):
            return a * b

        @staticmethod
        def dr_ab(a, b, cp, ca):
            return ca * b, ca * a

        @staticmethod
        def dr_a(a, b, cp, ca):
            return ca * b

        @staticmethod
        def dr_b(a, b, cp, ca):
            return ca * a

    mul = build_piso(Mul)
    a, b = np.array([1.0, 2.0, 3.0]), np.array([4.0, 5.0, 6.0])
    na, nb = make_reverse(a), make_reverse(b)
    reverse_prop(np.ones(3), mul(na, nb))
    assert np.array_equal(na.adj, b) and np.array_equal(nb.adj, a)
    nb2 = make_reverse(b)
    reverse_prop(np.ones(3), mul(a, nb2))
    assert np.array_equal(nb2.adj, a)
    assert np.array_equal(mul(a, b), a * b)  # untracked: a plain value


def test_fan_in_adjoints_add(ad):
    x = np.random.default_rng(35).uniform(-1, 1, (1, 4, 4, 2))
    w = np.random.default_rng(36).uniform(-1, 1, (2, 2, 2, 2))
    nx = make_reverse(x)
    y = ad.Maths.add(ad.NN.conv2d(nx, w, [1, 1], SAME), ad.NN.conv2d(nx, w, [1, 1], SAME))
    reverse_prop(np.ones(primal(y).shape), y)
    one = ad.nn.conv2d_backward_input(x, w, [1, 1], np.ones(primal(y).shape))
    assert np.allclose(nx.adj, 2 * one, rtol=0, atol=1e-12)


# ---- the fused layers (owl_gb300.layers) as tape ops ------------------------


def _small_cnn_fused(ad, p, x, onehot):
    """_small_cnn with each conv + bias + ReLU, the dense layer and the loss
    as the library's fused ops."""
    M, N = ad.Maths, ad.NN
    h = N.conv2d_bias_act(x, p["w1"], p["b1"], [1, 1], SAME, 1)
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = N.conv2d_bias_act(h, p["w2"], p["b2"], [1, 1], SAME, 1)
    h = N.avg_pool2d(VALID, h, [2, 2], [2, 2])
    h = M.reshape(h, (primal(h).shape[0], 3 * 3 * 6))
    z = N.fully_connected(h, p["w3"], p["b3"], 0)
    return N.softmax_cross_entropy(z, onehot)


def test_fused_layers_equal_owls_composition(ad):
    """conv2d_bias_act / fully_connected / softmax_cross_entropy give the
    loss and gradients of Owl's separate operations (conv2d, add, relu, dot,
    softmax, cross_entropy) to float64 rounding."""
    rng = np.random.default_rng(37)
    params = _small_params(rng)
    x = rng.uniform(0, 1, (4, 12, 12, 1))
    onehot = np.eye(10)[rng.integers(0, 10, 4)]
    la, ga = loss_and_grads(ad, params, x, onehot, model=_small_cnn_fused)
    lb, gb = loss_and_grads(ad, params, x, onehot, model=_small_cnn)
    assert abs(float(la) - float(lb)) <= 1e-13 * abs(float(lb))
    for k in ga:
        assert np.max(np.abs(ga[k] - gb[k])) <= 1e-12 * max(np.max(np.abs(gb[k])), 1e-300), k


def test_fused_layers_match_finite_differences(ad):
    rng = np.random.default_rng(38)
    params = _small_params(rng)
    x = rng.uniform(0, 1, (3, 12, 12, 1))
    onehot = np.eye(10)[rng.integers(0, 10, 3)]
    _, grads = loss_and_grads(ad, params, x, onehot, model=_small_cnn_fused)

    def loss(p):
        return _small_cnn_fused(ad, p, x, onehot)

    for name in params:
        idx = rng.choice(params[name].size, size=min(8, params[name].size), replace=False)
        err, _ = check_grad(loss, params, grads, name, idx, EPS)
        assert err <= TOL, (name, err)


def test_fully_connected_with_relu_and_untracked_inputs(ad):
    """A ReLU dense layer with only some inputs tracked: the adjoints of the
    tracked ones, against FD."""
    rng = np.random.default_rng(39)
    a = rng.standard_normal((5, 7))
    w = rng.standard_normal((7, 4))
    b = rng.standard_normal(4)
    for tracked in ("a", "w", "b"):
        _fd_check_op(lambda *t: ad.NN.fully_connected(
            t[0] if tracked == "a" else a, t[0] if tracked == "w" else w,
            t[0] if tracked == "b" else b, 1), [{"a": a, "w": w, "b": b}[tracked]], rng)
