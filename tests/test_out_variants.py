"""Owl's `_ ~out` variants (G:2402 conv2d_ and the like): every conv/pool
function writes into a caller-provided array when `out` is given, with the
same values as the allocating call, and rejects an `out` of the wrong
shape.  Run on the oracle."""

import numpy as np
import pytest

from owl_gb300.dense import InvalidArgument

SAME = "SAME"


def _cases(rng):
    x2 = rng.uniform(-1, 1, (2, 7, 6, 3))
    w2 = rng.uniform(-1, 1, (3, 3, 3, 4))
    x3 = rng.uniform(-1, 1, (1, 5, 4, 5, 2))
    w3 = rng.uniform(-1, 1, (2, 2, 2, 2, 3))
    x1 = rng.uniform(-1, 1, (2, 9, 3))
    w1 = rng.uniform(-1, 1, (3, 3, 4))
    return [
        ("conv2d", (x2, w2, [1, 1], SAME)),
        ("dilated_conv2d", (x2, w2, [1, 1], [2, 2], SAME)),
        ("transpose_conv2d", (x2, w2, [2, 2], SAME)),
        ("conv3d", (x3, w3, [1, 1, 1], SAME)),
        ("transpose_conv3d", (x3, w3, [2, 2, 2], SAME)),
        ("conv1d", (x1, w1, [2], SAME)),
        ("dilated_conv1d", (x1, w1, [1], [1, 2], SAME)),
        ("max_pool2d", (x2, [2, 2], [2, 2], SAME)),
        ("avg_pool3d", (x3, [2, 2, 2], [2, 2, 2], SAME)),
        ("max_pool1d", (x1, [3], [2], SAME)),
    ]


def test_forward_out_variants(oracle_nn):
    rng = np.random.default_rng(50)
    for name, args in _cases(rng):
        f = getattr(oracle_nn, name)
        ref = f(*args)
        out = np.full_like(ref, np.nan)
        got = f(*args, out=out)
        assert got is out or np.shares_memory(got, out), name
        assert np.array_equal(out, ref), name
        with pytest.raises(InvalidArgument):
            f(*args, out=np.empty(ref.shape[:-1] + (ref.shape[-1] + 1,)))


def test_backward_out_variants(oracle_nn):
    rng = np.random.default_rng(51)
    x = rng.uniform(-1, 1, (2, 7, 6, 3))
    w = rng.uniform(-1, 1, (3, 3, 3, 4))
    dy = rng.standard_normal((2, 7, 6, 4))
    for name, like in (("conv2d_backward_input", x), ("conv2d_backward_kernel", w)):
        f = getattr(oracle_nn, name)
        ref = f(x, w, [1, 1], dy)
        out = np.full_like(like, np.nan)
        f(x, w, [1, 1], dy, out=out)
        assert np.array_equal(out, ref), name
    g = rng.standard_normal((2, 4, 3, 3))
    for name in ("max_pool2d_backward", "avg_pool2d_backward"):
        f = getattr(oracle_nn, name)
        ref = f(SAME, x, [2, 2], [2, 2], g)
        out = np.full_like(x, np.nan)
        f(SAME, x, [2, 2], [2, 2], g, out=out)
        assert np.array_equal(out, ref), name
    v, i = oracle_nn.max_pool2d_argmax(x, [2, 2], [2, 2], SAME)
    ov, oi = np.empty_like(v), np.empty_like(i)
    oracle_nn.max_pool2d_argmax(x, [2, 2], [2, 2], SAME, out=ov, out_argmax=oi)
    assert np.array_equal(ov, v) and np.array_equal(oi, i)
