"""The layers around the convolutions (include/owlgpu.h "Extensions"): the
dense layer's GEMM, the conv forward with bias and ReLU in its epilogue, the
bias + activation backward, softmax cross-entropy and the SGD update, each
through the C ABI on the GPU against a float64 numpy reference of Owl's
composition of ndarray operations.

Bars (error = max|gpu - ref| / max|ref|): float64 1e-12, FP32 1e-5 (GEMM,
CUDA cores), BF16 1e-2, split-BF16 1e-5 -- the precision ladder of the
convolutions.  For the GEMM the denominator is max over outputs of
sum_k |op(a)[m][k] op(b)[k][n]|, the scale its rounding errors are relative
to (equal to max|ref| up to a constant for large sums, but not for the
ragged few-term products, whose sums may cancel).  Elementwise results (the
ReLU mask, SGD) are bit-exact.
"""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "bf16": 1e-2, "bf16x3": 1e-5}


def _layers(prec="fp32"):
    from owl_gb300.dense import NN, GpuBackend
    from owl_gb300.layers import Layers

    return Layers(NN(GpuBackend(prec)))


def _path_status():
    from owl_gb300 import _lib

    assert _lib.lib().owlgpu_device_status() == 0, _lib.last_error()


# m, n, k: the config-4 dense layers (batch 256, 3136 -> 1024 -> 10) and
# ragged shapes (single rows, sizes off every tile and chunk multiple)
GEMM_SHAPES = [(256, 1024, 3136), (256, 10, 1024), (1, 7, 5), (130, 33, 70), (300, 257, 129)]


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
@pytest.mark.parametrize("shape", GEMM_SHAPES)
@pytest.mark.parametrize("orient", ["nn", "nt", "tn"])
def test_dot(gpu_lib, prec, shape, orient):
    m, n, k = shape
    rng = np.random.default_rng(51)
    ta, tb = orient[0] == "t", orient[1] == "t"
    a = rng.uniform(-1, 1, (k, m) if ta else (m, k)).astype(np.float32)
    b = (rng.standard_normal((n, k) if tb else (k, n)) / np.sqrt(k)).astype(np.float32)
    bias = rng.standard_normal(n).astype(np.float32) * 0.1 if orient == "nn" else None
    act = 1 if orient == "nn" else 0
    L = _layers(prec)
    c = from_dev(L.dot(to_dev(a), to_dev(b), ta, tb, None if bias is None else to_dev(bias), act))
    _path_status()
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    ref = (a64.T if ta else a64) @ (b64.T if tb else b64)
    if bias is not None:
        ref = ref + bias
    if act:
        ref = np.maximum(ref, 0)
    assert c.shape == (m, n)
    scale = np.max(np.abs(a64.T if ta else a64) @ np.abs(b64.T if tb else b64))
    err = np.max(np.abs(c - ref)) / scale
    assert err <= TOL[prec], err


def test_dot_float64_and_determinism(gpu_lib):
    rng = np.random.default_rng(52)
    a = rng.standard_normal((256, 300))
    b = rng.standard_normal((300, 70))
    L = _layers()
    c = from_dev(L.dot(to_dev(a), to_dev(b)))
    assert rel(c, a @ b) <= 1e-12
    a32, b32 = to_dev(a.astype(np.float32)), to_dev(b.astype(np.float32))
    L16 = _layers("bf16")
    x = from_dev(L16.dot(a32, b32))  # split-K over several CTAs
    y = from_dev(L16.dot(a32, b32))
    assert np.array_equal(x, y)


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
@pytest.mark.parametrize("act", [0, 1])
@pytest.mark.parametrize("with_bias", [True, False])
def test_conv2d_bias_act(gpu_lib, oracle_nn, prec, act, with_bias):
    """act(conv2d + bias) in the convolution's epilogue against the oracle's
    conv2d (float64) plus the bias and ReLU; the ReLU result is exactly
    zero where the reference is negative beyond the error bar."""
    from owl_gb300 import _lib

    rng = np.random.default_rng(53)
    x = rng.uniform(-1, 1, (4, 14, 14, 32)).astype(np.float32)
    w = (rng.standard_normal((5, 5, 32, 64)) * np.sqrt(2 / 800)).astype(np.float32)
    b = (rng.standard_normal(64) * 0.2).astype(np.float32) if with_bias else None
    L = _layers(prec)
    y = from_dev(L.conv2d_bias_act(to_dev(x), to_dev(w), None if b is None else to_dev(b),
                                   [1, 1], "SAME", act))
    assert _lib.lib().owlgpu_last_conv_path() == (0 if prec == "fp32" else 1)
    _path_status()
    ref = oracle_nn.conv2d(x.astype(np.float64), w.astype(np.float64), [1, 1], "SAME")
    if b is not None:
        ref = ref + b
    if act:
        ref = np.maximum(ref, 0)
    assert rel(y, ref) <= TOL[prec] * 3
    if act:
        assert (y >= 0).all()


def test_conv_cuboid_bias_act(gpu_lib, oracle_nn):
    from owl_gb300 import _lib

    rng = np.random.default_rng(54)
    x = rng.uniform(-1, 1, (2, 8, 8, 8, 16)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 3, 16, 32)) * 0.05).astype(np.float32)
    b = (rng.standard_normal(32) * 0.2).astype(np.float32)
    y = to_dev(np.zeros((2, 8, 8, 8, 32), np.float32))
    import torch

    xd, wd, bd = to_dev(x), to_dev(w), to_dev(b)  # held until the call has run
    _lib.call("owlgpu_float32_ndarray_conv_cuboid_bias_act", xd.data_ptr(), wd.data_ptr(),
              y.data_ptr(), 2, 8, 8, 8, 16, 3, 3, 3, 8, 8, 8, 32, 1, 1, 1, 0, bd.data_ptr(), 1,
              _lib.PREC["bf16"], torch.cuda.current_stream().cuda_stream)
    ref = np.maximum(oracle_nn.conv3d(x.astype(np.float64), w.astype(np.float64), [1, 1, 1],
                                      "SAME") + b, 0)
    assert rel(from_dev(y), ref) <= 1e-2


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_bias_act_backward(gpu_lib, dtype):
    rng = np.random.default_rng(55)
    y = np.maximum(rng.standard_normal((37, 13, 11, 64)), 0).astype(dtype)
    y[0, 0, 0, :5] = 0.0  # exact zeros: the mask is y > 0
    dy = rng.standard_normal(y.shape).astype(dtype)
    L = _layers()
    dz, db = L.bias_act_backward(to_dev(y), to_dev(dy), 1)
    dz, db = from_dev(dz), from_dev(db)
    assert np.array_equal(dz, dy * (y > 0))
    ref = (dy * (y > 0)).astype(np.float64).reshape(-1, 64).sum(axis=0)
    assert rel(db, ref) <= (1e-5 if dtype == np.float32 else 1e-12)
    dz2, db2 = L.bias_act_backward(to_dev(y), to_dev(dy), 1)
    assert np.array_equal(from_dev(db2), db)  # fixed summation order
    dz0, db0 = L.bias_act_backward(to_dev(y), to_dev(dy), 0)
    assert np.array_equal(from_dev(dz0), dy)
    assert rel(from_dev(db0), dy.astype(np.float64).reshape(-1, 64).sum(axis=0)) <= (
        1e-5 if dtype == np.float32 else 1e-12)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(256, 10), (3, 1), (1000, 77)])
def test_softmax_cross_entropy(gpu_lib, dtype, shape):
    import torch

    rows, classes = shape
    rng = np.random.default_rng(56)
    z = (rng.standard_normal(shape) * 4).astype(dtype)
    lab = np.eye(classes, dtype=dtype)[rng.integers(0, classes, rows)]
    L = _layers()
    dloss = to_dev(np.array(0.5, dtype))
    loss, g = L.softmax_cross_entropy(to_dev(z), to_dev(lab), dloss=dloss, want_grad=True)
    z64 = z.astype(np.float64)
    m = z64.max(axis=1, keepdims=True)
    sm = np.exp(z64 - m) / np.exp(z64 - m).sum(axis=1, keepdims=True)
    ref_loss = -(lab * np.log(sm)).sum() / rows  # Owl: cross_entropy of softmax, batch mean
    ref_g = (sm - lab) * 0.5 / rows
    tol = 1e-5 if dtype == np.float32 else 1e-12
    assert abs(float(loss.item()) - ref_loss) <= tol * abs(ref_loss)
    assert rel(from_dev(g), ref_g) <= tol
    loss2, _ = L.softmax_cross_entropy(to_dev(z), to_dev(lab))
    assert float(loss2.item()) == float(loss.item())


def test_sgd_update(gpu_lib):
    rng = np.random.default_rng(57)
    w = rng.standard_normal(100003).astype(np.float32)
    g = rng.standard_normal(100003).astype(np.float32)
    wd = to_dev(w)
    _layers().sgd_update(wd, to_dev(g), 0.01)
    assert np.array_equal(from_dev(wd), w - np.float32(0.01) * g)


def test_bias_act_backward_ragged_channels(gpu_lib):
    """Channel counts off the 32-channel tile and few pixels (one chunk)."""
    rng = np.random.default_rng(59)
    for shape in [(3, 70), (1000, 33), (5, 1)]:
        y = np.maximum(rng.standard_normal(shape), 0).astype(np.float32)
        dy = rng.standard_normal(shape).astype(np.float32)
        dz, db = _layers().bias_act_backward(to_dev(y), to_dev(dy), 1)
        assert np.array_equal(from_dev(dz), dy * (y > 0))
        ref = (dy * (y > 0)).astype(np.float64).sum(axis=0)
        assert np.max(np.abs(from_dev(db) - ref)) <= 1e-5 * max(np.max(np.abs(ref)), 1.0)
