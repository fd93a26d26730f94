"""The measured workloads' own layers, at their own spatial and channel sizes
(batch sliced), through every precision, against the float64 oracle (Owl's D
path restated).

Config 2 (conv2d, owl_ndarray_conv_impl.h:246 forward, :465 backward_input,
:675 backward_kernel):
  L1  [B;56;56;128] * [3;3;128;128], stride 1, SAME
  L2  [B;28;28;256] * [3;3;256;256], stride 2, VALID
  D   L1 with rate 2 (dilated_conv2d, G:3797 / :3960 / :4151)
Config 3 (conv3d, im2col stubs :1211 / :1456 / :1331):
  conv3d           [B;32;32;32;32] * [3;3;3;32;64], stride 1, SAME
  transpose_conv3d [B;32;32;32;64] * [2;2;2;64;32], stride 2, SAME (G:5915,
                   backward_input G:6072, backward_kernel G:6277)

Inputs follow the workloads' distributions: uniform[-1,1] activations,
N(0, 2/fan_in) kernels, N(0,1) output gradients.  Bars (error = max|gpu -
f64| / max|f64|): FP32 plain 1e-4, TF32 5e-3, BF16 1e-2, split-BF16 1e-5.
Every tensor-core call also asserts that the tcgen05 kernel ran.
"""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-4, "tf32": 5e-3, "bf16": 1e-2, "bf16x3": 1e-5}
PRECS = ["fp32", "tf32", "bf16", "bf16x3"]

# name: input shape (batch 2), kernel, stride, rate (None = plain), padding
CONFIG2 = {
    "L1": ((2, 56, 56, 128), (3, 3, 128, 128), [1, 1], None, "SAME"),
    "L2": ((2, 28, 28, 256), (3, 3, 256, 256), [2, 2], None, "VALID"),
    "D": ((2, 56, 56, 128), (3, 3, 128, 128), [1, 1], [2, 2], "SAME"),
}


def _nn(prec):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend(prec))


def _check_path(prec):
    from owl_gb300 import _lib

    L = _lib.lib()
    assert L.owlgpu_device_status() == 0, _lib.last_error()
    want = 0 if prec == "fp32" else 1  # 0: CUDA-core kernel, 1: tcgen05
    assert L.owlgpu_last_conv_path() == want


def _inputs(xs, ks, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * np.sqrt(2.0 / np.prod(ks[:-1]))).astype(np.float32)
    return rng, x, w


@pytest.fixture(scope="module")
def config2_f64(oracle_nn):
    """Float64 oracle results of each config-2 layer (computed once)."""
    out = {}
    for name, (xs, ks, st, rate, pad) in CONFIG2.items():
        rng, x, w = _inputs(xs, ks, 31)
        x64, w64 = x.astype(np.float64), w.astype(np.float64)
        if rate:
            y64 = oracle_nn.dilated_conv2d(x64, w64, st, rate, pad)
        else:
            y64 = oracle_nn.conv2d(x64, w64, st, pad)
        dy = rng.standard_normal(y64.shape).astype(np.float32)
        dy64 = dy.astype(np.float64)
        if rate:
            dx64 = oracle_nn.dilated_conv2d_backward_input(x64, w64, st, rate, dy64)
            dw64 = oracle_nn.dilated_conv2d_backward_kernel(x64, w64, st, rate, dy64)
        else:
            dx64 = oracle_nn.conv2d_backward_input(x64, w64, st, dy64)
            dw64 = oracle_nn.conv2d_backward_kernel(x64, w64, st, dy64)
        out[name] = (x, w, dy, y64, dx64, dw64)
    return out


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("layer", list(CONFIG2))
def test_config2_layer(gpu_lib, config2_f64, layer, prec):
    _, _, st, rate, pad = CONFIG2[layer]
    x, w, dy, y64, dx64, dw64 = config2_f64[layer]
    G = _nn(prec)
    xd, wd, dyd = to_dev(x), to_dev(w), to_dev(dy)
    if rate:
        y = from_dev(G.dilated_conv2d(xd, wd, st, rate, pad))
        _check_path(prec)
        dx = from_dev(G.dilated_conv2d_backward_input(xd, wd, st, rate, dyd))
        _check_path(prec)
        dw = from_dev(G.dilated_conv2d_backward_kernel(xd, wd, st, rate, dyd))
    else:
        y = from_dev(G.conv2d(xd, wd, st, pad))
        _check_path(prec)
        dx = from_dev(G.conv2d_backward_input(xd, wd, st, dyd))
        _check_path(prec)
        dw = from_dev(G.conv2d_backward_kernel(xd, wd, st, dyd))
    _check_path(prec)
    errs = (rel(y, y64), rel(dx, dx64), rel(dw, dw64))
    print(f"{layer} {prec}: fwd {errs[0]:.2e} bwd_input {errs[1]:.2e} bwd_kernel {errs[2]:.2e}")
    assert max(errs) <= TOL[prec], errs


def test_config2_fp32_matches_float32_oracle(gpu_lib, oracle_nn, config2_f64):
    """The plain FP32 kernel within 1e-4 of Owl's float32 S path (restated)."""
    _, _, st, _, pad = CONFIG2["L2"]
    x, w, dy, _, _, _ = config2_f64["L2"]
    G = _nn("fp32")
    y = from_dev(G.conv2d(to_dev(x), to_dev(w), st, pad))
    assert rel(y, oracle_nn.conv2d(x, w, st, pad)) <= 1e-4
    dx = from_dev(G.conv2d_backward_input(to_dev(x), to_dev(w), st, to_dev(dy)))
    assert rel(dx, oracle_nn.conv2d_backward_input(x, w, st, dy)) <= 1e-4
    dw = from_dev(G.conv2d_backward_kernel(to_dev(x), to_dev(w), st, to_dev(dy)))
    assert rel(dw, oracle_nn.conv2d_backward_kernel(x, w, st, dy)) <= 1e-4


@pytest.fixture(scope="module")
def config3_f64(oracle_nn):
    """Float64 oracle results of the config-3 conv3d and transpose_conv3d
    (batch 1)."""
    rng, x, w = _inputs((1, 32, 32, 32, 32), (3, 3, 3, 32, 64), 41)
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    st = [1, 1, 1]
    y64 = oracle_nn.conv3d(x64, w64, st, "SAME")
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    conv = (x, w, dy, y64,
            oracle_nn.conv3d_backward_input(x64, w64, st, dy.astype(np.float64)),
            oracle_nn.conv3d_backward_kernel(x64, w64, st, dy.astype(np.float64)))
    # the transpose convolution reads the conv3d output's shape
    rng, xt, wt = _inputs((1, 32, 32, 32, 64), (2, 2, 2, 64, 32), 42)
    xt64, wt64 = xt.astype(np.float64), wt.astype(np.float64)
    s2 = [2, 2, 2]
    yt64 = oracle_nn.transpose_conv3d(xt64, wt64, s2, "SAME")
    dyt = rng.standard_normal(yt64.shape).astype(np.float32)
    tconv = (xt, wt, dyt, yt64,
             oracle_nn.transpose_conv3d_backward_input(xt64, wt64, s2, dyt.astype(np.float64)),
             oracle_nn.transpose_conv3d_backward_kernel(xt64, wt64, s2, dyt.astype(np.float64)))
    return {"conv3d": conv, "transpose_conv3d": tconv}


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("op", ["conv3d", "transpose_conv3d"])
def test_config3(gpu_lib, config3_f64, op, prec):
    x, w, dy, y64, dx64, dw64 = config3_f64[op]
    G = _nn(prec)
    st = [1, 1, 1] if op == "conv3d" else [2, 2, 2]
    xd, wd, dyd = to_dev(x), to_dev(w), to_dev(dy)
    y = from_dev(getattr(G, op)(xd, wd, st, "SAME"))
    _check_path(prec)
    dx = from_dev(getattr(G, op + "_backward_input")(xd, wd, st, dyd))
    _check_path(prec)
    dw = from_dev(getattr(G, op + "_backward_kernel")(xd, wd, st, dyd))
    _check_path(prec)
    errs = (rel(y, y64), rel(dx, dx64), rel(dw, dw64))
    print(f"{op} {prec}: fwd {errs[0]:.2e} bwd_input {errs[1]:.2e} bwd_kernel {errs[2]:.2e}")
    assert max(errs) <= TOL[prec], errs
