"""The C restatement against Owl's own compiled stubs on seeded random
inputs: every conv/pool entry point, float32 and float64, odd shapes,
strides, dilations and both paddings.  Pooling must match bit for bit."""

import numpy as np
import pytest

SAME, VALID = "SAME", "VALID"

CONV2D = [((2, 7, 9, 5), (3, 2, 5, 4), (1, 1), (1, 1), SAME),
          ((2, 8, 8, 3), (3, 3, 3, 6), (2, 2), (1, 1), VALID),
          ((1, 5, 6, 4), (2, 3, 4, 2), (2, 1), (2, 1), SAME),
          ((3, 9, 7, 2), (3, 3, 2, 3), (1, 2), (2, 3), VALID),
          ((1, 1, 1, 1), (1, 1, 1, 1), (1, 1), (1, 1), SAME),
          ((2, 3, 4, 3), (5, 5, 3, 2), (1, 1), (1, 1), SAME)]
CONV3D = [((2, 5, 4, 6, 3), (3, 2, 3, 3, 4), (1, 1, 1), (1, 1, 1), SAME),
          ((1, 6, 6, 5, 2), (2, 3, 2, 2, 3), (2, 1, 2), (1, 2, 1), VALID),
          ((1, 4, 5, 6, 2), (2, 2, 3, 2, 2), (1, 2, 1), (2, 1, 2), SAME)]
POOL2D = [((2, 7, 9, 5), (2, 3), (1, 2), SAME), ((2, 8, 8, 4), (2, 2), (2, 2), VALID),
          ((1, 5, 6, 3), (3, 3), (2, 2), SAME), ((1, 4, 4, 1), (4, 4), (1, 1), SAME)]
POOL3D = [((2, 5, 4, 6, 3), (2, 2, 3), (1, 2, 1), SAME), ((1, 6, 6, 4, 2), (2, 2, 2), (2, 2, 2), VALID),
          ((1, 5, 5, 5, 4), (3, 2, 2), (2, 1, 2), SAME)]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", CONV2D)
def test_conv2d_family(oracle_nn, ref_nn, dt, case):
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, xs).astype(dt)
    w = rng.uniform(-1, 1, ks).astype(dt)
    tol = 1e-5 if dt == np.float32 else 1e-12
    for O, R in [(oracle_nn, ref_nn)]:
        y = O.conv2d(x, w, list(st), pad)
        assert rel(y, R.conv2d(x, w, list(st), pad)) < tol
        dy = rng.standard_normal(y.shape).astype(dt)
        assert rel(O.conv2d_backward_input(x, w, list(st), dy),
                   R.conv2d_backward_input(x, w, list(st), dy)) < tol
        assert rel(O.conv2d_backward_kernel(x, w, list(st), dy),
                   R.conv2d_backward_kernel(x, w, list(st), dy)) < tol
        y = O.dilated_conv2d(x, w, list(st), list(rate), pad)
        assert rel(y, R.dilated_conv2d(x, w, list(st), list(rate), pad)) < tol
        dy = rng.standard_normal(y.shape).astype(dt)
        assert rel(O.dilated_conv2d_backward_input(x, w, list(st), list(rate), dy),
                   R.dilated_conv2d_backward_input(x, w, list(st), list(rate), dy)) < tol
        assert rel(O.dilated_conv2d_backward_kernel(x, w, list(st), list(rate), dy),
                   R.dilated_conv2d_backward_kernel(x, w, list(st), list(rate), dy)) < tol
        t = O.transpose_conv2d(x, w, list(st), pad)
        assert rel(t, R.transpose_conv2d(x, w, list(st), pad)) < tol


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", CONV3D)
def test_conv3d_family(oracle_nn, ref_nn, dt, case):
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, xs).astype(dt)
    w = rng.uniform(-1, 1, ks).astype(dt)
    tol = 1e-5 if dt == np.float32 else 1e-12
    O, R = oracle_nn, ref_nn
    y = O.conv3d(x, w, list(st), pad)
    assert rel(y, R.conv3d(x, w, list(st), pad)) < tol
    dy = rng.standard_normal(y.shape).astype(dt)
    assert rel(O.conv3d_backward_input(x, w, list(st), dy), R.conv3d_backward_input(x, w, list(st), dy)) < tol
    assert rel(O.conv3d_backward_kernel(x, w, list(st), dy), R.conv3d_backward_kernel(x, w, list(st), dy)) < tol
    y = O.dilated_conv3d(x, w, list(st), list(rate), pad)
    assert rel(y, R.dilated_conv3d(x, w, list(st), list(rate), pad)) < tol
    dy = rng.standard_normal(y.shape).astype(dt)
    assert rel(O.dilated_conv3d_backward_input(x, w, list(st), list(rate), dy),
               R.dilated_conv3d_backward_input(x, w, list(st), list(rate), dy)) < tol
    assert rel(O.dilated_conv3d_backward_kernel(x, w, list(st), list(rate), dy),
               R.dilated_conv3d_backward_kernel(x, w, list(st), list(rate), dy)) < tol


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", POOL2D)
def test_pool2d_bit_exact(oracle_nn, ref_nn, dt, case):
    xs, k, st, pad = case
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, xs).astype(dt)
    x.reshape(-1)[::7] = x.reshape(-1)[3]  # plant ties
    O, R = oracle_nn, ref_nn
    for f in ("max_pool2d", "avg_pool2d"):
        a, b = getattr(O, f)(x, list(k), list(st), pad), getattr(R, f)(x, list(k), list(st), pad)
        assert np.array_equal(a, b, equal_nan=True)
        g = rng.standard_normal(a.shape).astype(dt)
        assert np.array_equal(getattr(O, f + "_backward")(pad, x, list(k), list(st), g),
                              getattr(R, f + "_backward")(pad, x, list(k), list(st), g))
    a1, i1 = O.max_pool2d_argmax(x, list(k), list(st), pad)
    a2, i2 = R.max_pool2d_argmax(x, list(k), list(st), pad)
    assert np.array_equal(a1, a2) and np.array_equal(i1, i2)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", POOL3D)
def test_pool3d_bit_exact(oracle_nn, ref_nn, dt, case):
    xs, k, st, pad = case
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, xs).astype(dt)
    O, R = oracle_nn, ref_nn
    for f in ("max_pool3d", "avg_pool3d"):
        a, b = getattr(O, f)(x, list(k), list(st), pad), getattr(R, f)(x, list(k), list(st), pad)
        assert np.array_equal(a, b)
        g = rng.standard_normal(a.shape).astype(dt)
        assert np.array_equal(getattr(O, f + "_backward")(pad, x, list(k), list(st), g),
                              getattr(R, f + "_backward")(pad, x, list(k), list(st), g))


def test_degenerate_max_windows_route_to_element_zero(oracle_nn, ref_nn):
    """Owl's max-pool backward starts max_idx at 0 (owl_ndarray_pool_impl.h:167):
    windows with no value above -inf send their gradient to flat element 0."""
    x = np.full((1, 4, 4, 2), -np.inf, dtype=np.float32)
    x[0, 0, 0, 0] = 1.0
    x[0, 3, 3, 1] = np.nan
    g = np.arange(1, 9, dtype=np.float32).reshape(1, 2, 2, 2)
    a = oracle_nn.max_pool2d_backward("VALID", x, [2, 2], [2, 2], g)
    b = ref_nn.max_pool2d_backward("VALID", x, [2, 2], [2, 2], g)
    assert np.array_equal(a, b)
    assert a.reshape(-1)[0] == g.sum()
