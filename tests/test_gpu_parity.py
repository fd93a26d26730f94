"""CUDA library against the CPU oracle on seeded inputs.

Tolerances (error = max|gpu - oracle| / max|oracle|):
  float32 FP32 kernels   <= 1e-4   (the plain FP32 kernel vs Owl's S path)
  float64 kernels        <= 1e-11
  pooling, argmax        bit-exact (values and int64 indices)
"""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu
SAME, VALID = "SAME", "VALID"
TOL = {np.float32: 1e-4, np.float64: 1e-11}


@pytest.fixture(scope="module")
def gpu_nn(gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend("fp32"))


CONV2D = [((2, 7, 9, 5), (3, 2, 5, 4), (1, 1), (1, 1), SAME),
          ((2, 8, 8, 3), (3, 3, 3, 6), (2, 2), (1, 1), VALID),
          ((1, 5, 6, 4), (2, 3, 4, 2), (2, 1), (2, 1), SAME),
          ((3, 9, 7, 2), (3, 3, 2, 3), (1, 2), (2, 3), VALID),
          ((1, 1, 1, 1), (1, 1, 1, 1), (1, 1), (1, 1), SAME),
          ((2, 3, 4, 3), (5, 5, 3, 2), (1, 1), (1, 1), SAME),
          ((4, 17, 13, 37), (3, 3, 37, 70), (1, 1), (1, 1), SAME),
          ((2, 15, 15, 64), (3, 3, 64, 128), (2, 2), (1, 1), VALID),
          ((2, 14, 14, 33), (1, 1, 33, 129), (1, 1), (1, 1), SAME)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", CONV2D)
@pytest.mark.parametrize("where", ["host", "device"])
def test_conv2d_family(gpu_nn, oracle_nn, dt, case, where):
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, xs).astype(dt)
    w = rng.uniform(-1, 1, ks).astype(dt)
    put, get = (to_dev, from_dev) if where == "device" else ((lambda a: a), np.asarray)
    G, O = gpu_nn, oracle_nn
    xd, wd = put(x), put(w)
    y = O.conv2d(x, w, list(st), pad)
    assert rel(get(G.conv2d(xd, wd, list(st), pad)), y) <= TOL[dt]
    dy = rng.standard_normal(y.shape).astype(dt)
    dyd = put(dy)
    assert rel(get(G.conv2d_backward_input(xd, wd, list(st), dyd)),
               O.conv2d_backward_input(x, w, list(st), dy)) <= TOL[dt]
    assert rel(get(G.conv2d_backward_kernel(xd, wd, list(st), dyd)),
               O.conv2d_backward_kernel(x, w, list(st), dy)) <= TOL[dt]
    y = O.dilated_conv2d(x, w, list(st), list(rate), pad)
    assert rel(get(G.dilated_conv2d(xd, wd, list(st), list(rate), pad)), y) <= TOL[dt]
    dy = rng.standard_normal(y.shape).astype(dt)
    dyd = put(dy)
    assert rel(get(G.dilated_conv2d_backward_input(xd, wd, list(st), list(rate), dyd)),
               O.dilated_conv2d_backward_input(x, w, list(st), list(rate), dy)) <= TOL[dt]
    assert rel(get(G.dilated_conv2d_backward_kernel(xd, wd, list(st), list(rate), dyd)),
               O.dilated_conv2d_backward_kernel(x, w, list(st), list(rate), dy)) <= TOL[dt]
    if ks[2] == ks[3] or True:
        t = O.transpose_conv2d(x, w, list(st), pad)
        assert rel(get(G.transpose_conv2d(xd, wd, list(st), pad)), t) <= TOL[dt]


CONV3D = [((2, 5, 4, 6, 3), (3, 2, 3, 3, 4), (1, 1, 1), (1, 1, 1), SAME),
          ((1, 6, 6, 5, 2), (2, 3, 2, 2, 3), (2, 1, 2), (1, 2, 1), VALID),
          ((1, 4, 5, 6, 2), (2, 2, 3, 2, 2), (1, 2, 1), (2, 1, 2), SAME),
          ((2, 8, 8, 8, 32), (3, 3, 3, 32, 64), (1, 1, 1), (1, 1, 1), SAME)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", CONV3D)
def test_conv3d_family(gpu_nn, oracle_nn, dt, case):
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(12)
    x = rng.uniform(-1, 1, xs).astype(dt)
    w = rng.uniform(-1, 1, ks).astype(dt)
    G, O = gpu_nn, oracle_nn
    xd, wd = to_dev(x), to_dev(w)
    y = O.conv3d(x, w, list(st), pad)
    assert rel(from_dev(G.conv3d(xd, wd, list(st), pad)), y) <= TOL[dt]
    dy = rng.standard_normal(y.shape).astype(dt)
    dyd = to_dev(dy)
    assert rel(from_dev(G.conv3d_backward_input(xd, wd, list(st), dyd)),
               O.conv3d_backward_input(x, w, list(st), dy)) <= TOL[dt]
    assert rel(from_dev(G.conv3d_backward_kernel(xd, wd, list(st), dyd)),
               O.conv3d_backward_kernel(x, w, list(st), dy)) <= TOL[dt]
    y = O.dilated_conv3d(x, w, list(st), list(rate), pad)
    assert rel(from_dev(G.dilated_conv3d(xd, wd, list(st), list(rate), pad)), y) <= TOL[dt]
    dy = rng.standard_normal(y.shape).astype(dt)
    dyd = to_dev(dy)
    assert rel(from_dev(G.dilated_conv3d_backward_input(xd, wd, list(st), list(rate), dyd)),
               O.dilated_conv3d_backward_input(x, w, list(st), list(rate), dy)) <= TOL[dt]
    assert rel(from_dev(G.dilated_conv3d_backward_kernel(xd, wd, list(st), list(rate), dyd)),
               O.dilated_conv3d_backward_kernel(x, w, list(st), list(rate), dy)) <= TOL[dt]
    if ks[3] == ks[4]:
        pass
    t = O.transpose_conv3d(x[..., :ks[3]], w, list(st), pad)
    assert rel(from_dev(G.transpose_conv3d(to_dev(x[..., :ks[3]].copy()), wd, list(st), pad)),
               t) <= TOL[dt]


POOL2D = [((2, 7, 9, 5), (2, 3), (1, 2), SAME), ((2, 8, 8, 4), (2, 2), (2, 2), VALID),
          ((1, 5, 6, 3), (3, 3), (2, 2), SAME), ((1, 4, 4, 1), (4, 4), (1, 1), SAME),
          ((3, 16, 12, 64), (3, 3), (1, 1), SAME), ((2, 9, 11, 6), (3, 2), (2, 3), VALID),
          # non-overlapping windows: cells wider than windows, padded first
          # cell, ragged tail, 16-byte channel vectors
          ((2, 9, 10, 5), (2, 2), (3, 3), VALID), ((1, 4, 7, 3), (3, 3), (3, 3), SAME),
          ((2, 10, 10, 64), (2, 2), (2, 2), SAME), ((1, 11, 5, 8), (1, 2), (3, 2), SAME),
          # interior windows of the fixed-size kernels (2x2, 3x3), overlapping
          # and not
          ((2, 9, 11, 8), (3, 3), (2, 2), VALID), ((2, 7, 6, 12), (2, 2), (1, 1), VALID),
          ((1, 12, 10, 16), (3, 3), (3, 3), VALID)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", POOL2D)
def test_pool2d_bit_exact(gpu_nn, oracle_nn, dt, case):
    xs, k, st, pad = case
    rng = np.random.default_rng(13)
    x = rng.uniform(-1, 1, xs).astype(dt)
    x.reshape(-1)[::7] = x.reshape(-1)[3]  # ties: the first maximum must win
    G, O = gpu_nn, oracle_nn
    xd = to_dev(x)
    for f in ("max_pool2d", "avg_pool2d"):
        a = O.__getattribute__(f)(x, list(k), list(st), pad)
        assert np.array_equal(from_dev(getattr(G, f)(xd, list(k), list(st), pad)), a)
        g = rng.standard_normal(a.shape).astype(dt)
        assert np.array_equal(
            from_dev(getattr(G, f + "_backward")(pad, xd, list(k), list(st), to_dev(g))),
            getattr(O, f + "_backward")(pad, x, list(k), list(st), g))
    a1, i1 = O.max_pool2d_argmax(x, list(k), list(st), pad)
    a2, i2 = G.max_pool2d_argmax(xd, list(k), list(st), pad)
    assert np.array_equal(from_dev(a2), a1) and np.array_equal(from_dev(i2), i1)


POOL3D = [((2, 5, 4, 6, 3), (2, 2, 3), (1, 2, 1), SAME), ((1, 6, 6, 4, 2), (2, 2, 2), (2, 2, 2), VALID),
          ((1, 5, 5, 5, 4), (3, 2, 2), (2, 1, 2), SAME), ((2, 8, 8, 8, 64), (2, 2, 2), (2, 2, 2), SAME),
          ((1, 7, 5, 9, 6), (2, 2, 3), (3, 2, 3), VALID), ((1, 4, 7, 5, 2), (3, 3, 2), (3, 3, 2), SAME)]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("case", POOL3D)
def test_pool3d_bit_exact(gpu_nn, oracle_nn, dt, case):
    xs, k, st, pad = case
    rng = np.random.default_rng(14)
    x = rng.uniform(-1, 1, xs).astype(dt)
    G, O = gpu_nn, oracle_nn
    xd = to_dev(x)
    for f in ("max_pool3d", "avg_pool3d"):
        a = getattr(O, f)(x, list(k), list(st), pad)
        assert np.array_equal(from_dev(getattr(G, f)(xd, list(k), list(st), pad)), a)
        g = rng.standard_normal(a.shape).astype(dt)
        assert np.array_equal(
            from_dev(getattr(G, f + "_backward")(pad, xd, list(k), list(st), to_dev(g))),
            getattr(O, f + "_backward")(pad, x, list(k), list(st), g))


def test_config1_full_size(gpu_nn, oracle_nn):
    """The plain float32 conv2d of [8;32;32;16] * [3;3;16;32] SAME (within
    1e-4 of the oracle) followed by max_pool2d 2x2/2 with argmax, bit-exact."""
    rng = np.random.default_rng(2024)
    x = rng.uniform(-1, 1, (8, 32, 32, 16)).astype(np.float32)
    w = rng.uniform(-1, 1, (3, 3, 16, 32)).astype(np.float32)
    y_o = oracle_nn.conv2d(x, w, [1, 1], SAME)
    y_g = gpu_nn.conv2d(x, w, [1, 1], SAME)
    assert rel(y_g, y_o) <= 1e-4
    # pool on the GPU's own conv output, compared with the oracle on the same
    p_o, i_o = oracle_nn.max_pool2d_argmax(y_g, [2, 2], [2, 2], SAME)
    p_g, i_g = gpu_nn.max_pool2d_argmax(y_g, [2, 2], [2, 2], SAME)
    assert np.array_equal(p_g, p_o) and np.array_equal(i_g, i_o)


@pytest.mark.parametrize("ch", [2, 4])
def test_degenerate_windows_match_owl(gpu_nn, oracle_nn, ch):
    x = np.full((1, 4, 4, ch), -np.inf, dtype=np.float32)
    x[0, 0, 0, 0] = 1.0
    x[0, 3, 3, 1] = np.nan
    g = np.arange(1, 4 * ch + 1, dtype=np.float32).reshape(1, 2, 2, ch)
    a = oracle_nn.max_pool2d_backward("VALID", x, [2, 2], [2, 2], g)
    b = from_dev(gpu_nn.max_pool2d_backward("VALID", to_dev(x), [2, 2], [2, 2], to_dev(g)))
    assert np.array_equal(a, b)
    pa, ia = oracle_nn.max_pool2d_argmax(x, [2, 2], [2, 2], "VALID")
    pb, ib = gpu_nn.max_pool2d_argmax(x, [2, 2], [2, 2], "VALID")
    assert np.array_equal(pa, pb) and np.array_equal(ia, ib)


@pytest.mark.parametrize("k,st", [((2, 2), (2, 2)), ((3, 3), (1, 1)), ((3, 2), (2, 3))])
def test_degenerate_windows_ordered(gpu_nn, oracle_nn, k, st):
    """Many windows that select nothing (all -inf or NaN), spread over the
    tensor, in both backward forms: their gradients are summed into element
    0 in Owl's window order."""
    rng = np.random.default_rng(17)
    x = rng.uniform(-1, 1, (2, 9, 8, 6)).astype(np.float32)
    x[:, 2:7, 1:6, :] = -np.inf
    x[1, 4:8, 3:5, 2:4] = np.nan
    y = oracle_nn.max_pool2d(x, list(k), list(st), SAME)
    g = rng.standard_normal(y.shape).astype(np.float32)
    a = oracle_nn.max_pool2d_backward(SAME, x, list(k), list(st), g)
    b = from_dev(gpu_nn.max_pool2d_backward(SAME, to_dev(x), list(k), list(st), to_dev(g)))
    assert np.array_equal(a, b)
    for c3 in (3, 4):
        x3 = np.full((1, 4, 4, 4, c3), -np.inf, dtype=np.float64)
        x3[0, 1, 2, 3, 1] = 0.5
        g3 = np.arange(1, 8 * c3 + 1, dtype=np.float64).reshape(1, 2, 2, 2, c3)
        a3 = oracle_nn.max_pool3d_backward("VALID", x3, [2, 2, 2], [2, 2, 2], g3)
        b3 = from_dev(gpu_nn.max_pool3d_backward("VALID", to_dev(x3), [2, 2, 2], [2, 2, 2],
                                                 to_dev(g3)))
        assert np.array_equal(a3, b3)


def test_repeat_calls_are_deterministic(gpu_nn):
    rng = np.random.default_rng(5)
    x = to_dev(rng.uniform(-1, 1, (4, 20, 20, 32)).astype(np.float32))
    w = to_dev(rng.uniform(-1, 1, (3, 3, 32, 48)).astype(np.float32))
    dy = to_dev(rng.standard_normal((4, 20, 20, 48)).astype(np.float32))
    a = from_dev(gpu_nn.conv2d_backward_kernel(x, w, [1, 1], dy))
    b = from_dev(gpu_nn.conv2d_backward_kernel(x, w, [1, 1], dy))
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_1d_family(gpu_nn, oracle_nn, dt):
    """conv1d / dilated_conv1d / transpose_conv1d and pool1d, forward and
    backward: Owl runs them as 2-D calls on [B;1;W;C] views (G:3402,
    G:4967, G:6483, G:7027, G:7840)."""
    rng = np.random.default_rng(15)
    G, O = gpu_nn, oracle_nn
    x = rng.uniform(-1, 1, (3, 17, 5)).astype(dt)
    w = rng.uniform(-1, 1, (3, 5, 4)).astype(dt)
    xd, wd = to_dev(x), to_dev(w)
    for pad in (SAME, VALID):
        y = O.conv1d(x, w, [2], pad)
        assert rel(from_dev(G.conv1d(xd, wd, [2], pad)), y) <= TOL[dt]
        dy = rng.standard_normal(y.shape).astype(dt)
        assert rel(from_dev(G.conv1d_backward_input(xd, wd, [2], to_dev(dy))),
                   O.conv1d_backward_input(x, w, [2], dy)) <= TOL[dt]
        assert rel(from_dev(G.conv1d_backward_kernel(xd, wd, [2], to_dev(dy))),
                   O.conv1d_backward_kernel(x, w, [2], dy)) <= TOL[dt]
        y = O.dilated_conv1d(x, w, [1], [1, 2], pad)
        assert rel(from_dev(G.dilated_conv1d(xd, wd, [1], [1, 2], pad)), y) <= TOL[dt]
        dy = rng.standard_normal(y.shape).astype(dt)
        assert rel(from_dev(G.dilated_conv1d_backward_input(xd, wd, [1], [1, 2], to_dev(dy))),
                   O.dilated_conv1d_backward_input(x, w, [1], [1, 2], dy)) <= TOL[dt]
        assert rel(from_dev(G.dilated_conv1d_backward_kernel(xd, wd, [1], [1, 2], to_dev(dy))),
                   O.dilated_conv1d_backward_kernel(x, w, [1], [1, 2], dy)) <= TOL[dt]
        wt = rng.uniform(-1, 1, (3, 5, 2)).astype(dt)
        y = O.transpose_conv1d(x, wt, [2], pad)
        assert rel(from_dev(G.transpose_conv1d(xd, to_dev(wt), [2], pad)), y) <= TOL[dt]
        dy = rng.standard_normal(y.shape).astype(dt)
        assert rel(from_dev(G.transpose_conv1d_backward_input(xd, to_dev(wt), [2], to_dev(dy))),
                   O.transpose_conv1d_backward_input(x, wt, [2], dy)) <= TOL[dt]
        assert rel(from_dev(G.transpose_conv1d_backward_kernel(xd, to_dev(wt), [2],
                                                               to_dev(dy))),
                   O.transpose_conv1d_backward_kernel(x, wt, [2], dy)) <= TOL[dt]
        for f in ("max_pool1d", "avg_pool1d"):
            a = getattr(O, f)(x, [3], [2], pad)
            assert np.array_equal(from_dev(getattr(G, f)(xd, [3], [2], pad)), a)
            g = rng.standard_normal(a.shape).astype(dt)
            assert np.array_equal(
                from_dev(getattr(G, f + "_backward")(pad, xd, [3], [2], to_dev(g))),
                getattr(O, f + "_backward")(pad, x, [3], [2], g))
