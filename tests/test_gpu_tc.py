"""Tensor-core (tcgen05) convolutions: BF16, TF32 and split-BF16 precision
against the float64 oracle (Owl's D path restated).

Tolerances (error = max|gpu - f64| / max|f64|), written here as the
acceptance bar for each precision:
  BF16   <= 1e-2    TF32 <= 5e-3    BF16X3 (hi*hi + hi*lo + lo*hi) <= 1e-5
BF16X3 represents each operand as hi + lo with 8 + 8 significant bits; what
that drops is about 2^-17 relative per product, 4e-6 of max|y| with exact
sums.  The tensor core rounds its FP32 accumulator toward zero after every
MMA, so the cross terms accumulate apart from the hi*hi sums (measured on
GB300: 6.7e-6 at K = 4608, against 1.8e-5 with all three MMAs in one
accumulator).
Every case also asserts that the tensor-core kernel (not the CUDA-core
fallback) ran, through owlgpu_last_conv_path(), and that no tensor-core
kernel abandoned a pipeline wait (owlgpu_device_status).  A TF32 request for
backward_kernel runs the split-BF16 kernel (MN-major operands).
"""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu
TOL = {"bf16": 1e-2, "tf32": 5e-3, "bf16x3": 1e-5}
SAME, VALID = "SAME", "VALID"

CASES2D = [
    # input, kernel, rate (None = plain), padding
    ((2, 12, 10, 16), (3, 3, 16, 32), None, SAME),
    ((2, 20, 20, 32), (3, 3, 32, 48), None, SAME),
    ((1, 9, 11, 5), (3, 2, 5, 7), None, VALID),
    ((2, 17, 19, 40), (3, 3, 40, 24), (2, 2), SAME),
    ((1, 33, 18, 64), (5, 5, 64, 130), None, SAME),
    ((3, 14, 14, 33), (1, 1, 33, 129), None, SAME),
    ((2, 16, 24, 128), (3, 3, 128, 128), None, SAME),
    ((1, 23, 21, 200), (3, 3, 200, 72), (1, 3), SAME),
    # short outputs (128-pixel tiles) with several 128-channel output tiles:
    # two co tiles per CTA tile, the last group holding one
    ((2, 13, 11, 64), (3, 3, 64, 384), None, SAME),
    ((1, 7, 7, 256), (3, 3, 256, 512), None, SAME),
    # outputs taller than 32 rows split into equal tiles of an even height
    # (MMA N = 8 x rows): 2 x 20, 2 x 26 (last 24), 2 x 28 (the config-2
    # L1 height), 3 x 22 with dilation
    ((1, 40, 9, 32), (3, 3, 32, 64), None, SAME),
    ((1, 50, 8, 16), (3, 3, 16, 128), None, SAME),
    ((1, 56, 16, 128), (3, 3, 128, 128), None, SAME),
    ((1, 66, 10, 8), (3, 3, 8, 16), (2, 2), SAME),
]
CASES3D = [
    ((2, 6, 7, 9, 8), (3, 3, 3, 8, 16), None, SAME),
    ((1, 8, 8, 8, 32), (3, 3, 3, 32, 64), None, SAME),
    ((1, 5, 6, 7, 3), (2, 3, 2, 3, 5), (2, 1, 2), SAME),
]


@pytest.fixture(scope="module")
def f64_nn(oracle_nn):
    return oracle_nn


def _nn(prec):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend(prec))


def _path():
    from owl_gb300 import _lib

    L = _lib.lib()
    assert L.owlgpu_device_status() == 0, _lib.last_error()
    return L.owlgpu_last_conv_path()


@pytest.mark.parametrize("prec", ["bf16", "tf32", "bf16x3"])
@pytest.mark.parametrize("case", CASES2D)
def test_conv2d_tc(gpu_lib, f64_nn, prec, case):
    xs, ks, rate, pad = case
    rng = np.random.default_rng(21)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * np.sqrt(2.0 / np.prod(ks[:3]))).astype(np.float32)
    G = _nn(prec)
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    xd, wd = to_dev(x), to_dev(w)
    if rate:
        y = from_dev(G.dilated_conv2d(xd, wd, [1, 1], list(rate), pad))
        assert _path() == 1
        y64 = f64_nn.dilated_conv2d(x64, w64, [1, 1], list(rate), pad)
    else:
        y = from_dev(G.conv2d(xd, wd, [1, 1], pad))
        assert _path() == 1
        y64 = f64_nn.conv2d(x64, w64, [1, 1], pad)
    assert rel(y, y64) <= TOL[prec]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dyd = to_dev(dy)
    if rate:
        dx = from_dev(G.dilated_conv2d_backward_input(xd, wd, [1, 1], list(rate), dyd))
        assert _path() == 1
        dx64 = f64_nn.dilated_conv2d_backward_input(x64, w64, [1, 1], list(rate), dy.astype(np.float64))
    else:
        dx = from_dev(G.conv2d_backward_input(xd, wd, [1, 1], dyd))
        assert _path() == 1
        dx64 = f64_nn.conv2d_backward_input(x64, w64, [1, 1], dy.astype(np.float64))
    assert rel(dx, dx64) <= TOL[prec]
    if rate:
        dw = from_dev(G.dilated_conv2d_backward_kernel(xd, wd, [1, 1], list(rate), dyd))
        assert _path() == 1
        dw64 = f64_nn.dilated_conv2d_backward_kernel(x64, w64, [1, 1], list(rate), dy.astype(np.float64))
    else:
        dw = from_dev(G.conv2d_backward_kernel(xd, wd, [1, 1], dyd))
        assert _path() == 1
        dw64 = f64_nn.conv2d_backward_kernel(x64, w64, [1, 1], dy.astype(np.float64))
    assert rel(dw, dw64) <= TOL[prec]


@pytest.mark.parametrize("prec", ["bf16", "tf32", "bf16x3"])
@pytest.mark.parametrize("case", CASES3D)
def test_conv3d_tc(gpu_lib, f64_nn, prec, case):
    xs, ks, rate, pad = case
    rng = np.random.default_rng(22)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * np.sqrt(2.0 / np.prod(ks[:4]))).astype(np.float32)
    G = _nn(prec)
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    xd, wd = to_dev(x), to_dev(w)
    st = [1, 1, 1]
    if rate:
        y = from_dev(G.dilated_conv3d(xd, wd, st, list(rate), pad))
        y64 = f64_nn.dilated_conv3d(x64, w64, st, list(rate), pad)
    else:
        y = from_dev(G.conv3d(xd, wd, st, pad))
        y64 = f64_nn.conv3d(x64, w64, st, pad)
    assert _path() == 1
    assert rel(y, y64) <= TOL[prec]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    if rate:
        dx = from_dev(G.dilated_conv3d_backward_input(xd, wd, st, list(rate), to_dev(dy)))
        dx64 = f64_nn.dilated_conv3d_backward_input(x64, w64, st, list(rate), dy.astype(np.float64))
    else:
        dx = from_dev(G.conv3d_backward_input(xd, wd, st, to_dev(dy)))
        dx64 = f64_nn.conv3d_backward_input(x64, w64, st, dy.astype(np.float64))
    assert rel(dx, dx64) <= TOL[prec]
    if rate:
        dw = from_dev(G.dilated_conv3d_backward_kernel(xd, wd, st, list(rate), to_dev(dy)))
        dw64 = f64_nn.dilated_conv3d_backward_kernel(x64, w64, st, list(rate), dy.astype(np.float64))
    else:
        dw = from_dev(G.conv3d_backward_kernel(xd, wd, st, to_dev(dy)))
        dw64 = f64_nn.conv3d_backward_kernel(x64, w64, st, dy.astype(np.float64))
    assert _path() == 1
    assert rel(dw, dw64) <= TOL[prec]


def test_tc_repeatable_and_host_dropin(gpu_lib, f64_nn):
    """Same inputs twice give bit-identical results; the host drop-in path
    with OWLGPU precision bf16 matches the device path."""
    rng = np.random.default_rng(23)
    x = rng.uniform(-1, 1, (4, 30, 26, 64)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 64, 96)) * 0.06).astype(np.float32)
    G = _nn("bf16")
    a = from_dev(G.conv2d(to_dev(x), to_dev(w), [1, 1], SAME))
    b = from_dev(G.conv2d(to_dev(x), to_dev(w), [1, 1], SAME))
    assert np.array_equal(a, b)
    h = G.conv2d(x, w, [1, 1], SAME)  # numpy arrays: host drop-in entry point
    assert np.array_equal(a, h)


STRIDED = [
    # input, kernel, stride, rate, padding
    ((2, 15, 15, 16), (3, 3, 16, 8), (2, 2), (1, 1), VALID),
    ((2, 28, 28, 64), (3, 3, 64, 128), (2, 2), (1, 1), VALID),
    ((2, 17, 13, 24), (3, 2, 24, 40), (2, 3), (1, 2), SAME),
    ((1, 20, 22, 32), (5, 5, 32, 48), (3, 2), (2, 1), SAME),
    ((2, 16, 16, 64), (1, 1, 64, 128), (2, 2), (1, 1), SAME),
    # stride and dilation sharing a factor (residue classes with dilation d/g)
    ((1, 14, 12, 16), (3, 3, 16, 32), (2, 2), (2, 2), SAME),
    ((2, 13, 13, 32), (3, 3, 32, 64), (2, 2), (1, 1), VALID),
]


@pytest.mark.parametrize("prec", ["bf16", "tf32", "bf16x3"])
@pytest.mark.parametrize("case", STRIDED)
def test_strided_conv2d_tc(gpu_lib, f64_nn, prec, case):
    """Strided geometries: forward stages the halo in stride residue classes,
    backward_input runs as one stride-1 correlation per residue class of dX
    (the 1x1 case has classes no tap reaches, which stay zero),
    backward_kernel stages X in residue classes -- all on tcgen05."""
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(25)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * np.sqrt(2.0 / np.prod(ks[:3]))).astype(np.float32)
    G = _nn(prec)
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    xd, wd = to_dev(x), to_dev(w)
    st, rate = list(st), list(rate)
    y = from_dev(G.dilated_conv2d(xd, wd, st, rate, pad))
    assert _path() == 1
    y64 = f64_nn.dilated_conv2d(x64, w64, st, rate, pad)
    assert rel(y, y64) <= TOL[prec]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dx = from_dev(G.dilated_conv2d_backward_input(xd, wd, st, rate, to_dev(dy)))
    assert _path() == 1
    assert rel(dx, f64_nn.dilated_conv2d_backward_input(x64, w64, st, rate,
                                                        dy.astype(np.float64))) <= TOL[prec]
    dw = from_dev(G.dilated_conv2d_backward_kernel(xd, wd, st, rate, to_dev(dy)))
    assert _path() == 1
    assert rel(dw, f64_nn.dilated_conv2d_backward_kernel(x64, w64, st, rate,
                                                         dy.astype(np.float64))) <= TOL[prec]


def test_strided_conv3d_tc(gpu_lib, f64_nn):
    rng = np.random.default_rng(26)
    x = rng.uniform(-1, 1, (2, 9, 9, 8, 16)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 3, 16, 32)) * 0.07).astype(np.float32)
    G = _nn("bf16")
    st = [2, 2, 2]
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    y = from_dev(G.conv3d(to_dev(x), to_dev(w), st, SAME))
    assert _path() == 1
    y64 = f64_nn.conv3d(x64, w64, st, SAME)
    assert rel(y, y64) <= TOL["bf16"]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dx = from_dev(G.conv3d_backward_input(to_dev(x), to_dev(w), st, to_dev(dy)))
    assert _path() == 1
    assert rel(dx, f64_nn.conv3d_backward_input(x64, w64, st, dy.astype(np.float64))) <= 1e-2
    dw = from_dev(G.conv3d_backward_kernel(to_dev(x), to_dev(w), st, to_dev(dy)))
    assert _path() == 1
    assert rel(dw, f64_nn.conv3d_backward_kernel(x64, w64, st, dy.astype(np.float64))) <= 1e-2


# transpose convolutions whose kernel is not larger than the stride: every
# residue class of the output receives one tap (or none), so the classes run
# as one 1x1 convolution with a depth-to-space epilogue
TCONV = [
    ((2, 7, 9, 48), (2, 2, 48, 40), (2, 2), SAME),
    ((1, 6, 5, 24), (2, 2, 24, 16), (3, 3), SAME),
    ((2, 5, 6, 32), (3, 3, 32, 8), (3, 3), VALID),
    ((1, 4, 5, 6, 64), (2, 2, 2, 64, 32), (2, 2, 2), SAME),
]


# transpose convolutions whose kernel is larger than the stride (several
# taps per output residue class)
TCONV_WIDE = [
    ((2, 7, 9, 48), (3, 3, 48, 40), (2, 2), SAME),
    ((1, 6, 5, 24), (5, 4, 24, 16), (2, 3), VALID),
    ((1, 4, 5, 6, 32), (3, 3, 3, 32, 16), (2, 2, 2), SAME),
]


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
@pytest.mark.parametrize("case", TCONV + TCONV_WIDE)
def test_transpose_conv_tc(gpu_lib, f64_nn, prec, case):
    """Transpose convolution forward (strided backward_input by residue
    classes), backward_input (a strided forward convolution of dY) and
    backward_kernel (the weight gradient with the roles swapped), all on
    tcgen05, against the float64 oracle."""
    xs, ks, st, pad = case
    rng = np.random.default_rng(27)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.2).astype(np.float32)
    G = _nn(prec)
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    f = "transpose_conv3d" if len(xs) == 5 else "transpose_conv2d"
    y = from_dev(getattr(G, f)(to_dev(x), to_dev(w), list(st), pad))
    assert _path() == 1
    y64 = getattr(f64_nn, f)(x64, w64, list(st), pad)
    assert rel(y, y64) <= TOL[prec]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dx = from_dev(getattr(G, f + "_backward_input")(to_dev(x), to_dev(w), list(st), to_dev(dy)))
    assert _path() == 1
    dx64 = getattr(f64_nn, f + "_backward_input")(x64, w64, list(st), dy.astype(np.float64))
    assert rel(dx, dx64) <= TOL[prec]
    dw = from_dev(getattr(G, f + "_backward_kernel")(to_dev(x), to_dev(w), list(st), to_dev(dy)))
    assert _path() == 1
    dw64 = getattr(f64_nn, f + "_backward_kernel")(x64, w64, list(st), dy.astype(np.float64))
    assert rel(dw, dw64) <= TOL[prec]


# convolutions whose kernel equals their stride (non-overlapping windows,
# the backward passes of a kernel = stride transpose convolution): forward
# and backward_kernel run as a tcgen05 GEMM over the windows
PATCH = [
    ((2, 16, 16, 32), (4, 4, 32, 64), (4, 4), VALID),
    ((3, 12, 10, 16), (2, 2, 16, 40), (2, 2), SAME),
    ((1, 8, 6, 4, 24), (2, 2, 2, 24, 16), (2, 2, 2), VALID),
]


@pytest.mark.parametrize("prec", ["bf16", "tf32", "bf16x3"])
@pytest.mark.parametrize("case", PATCH)
def test_kernel_equals_stride_tc(gpu_lib, f64_nn, prec, case):
    xs, ks, st, pad = case
    rng = np.random.default_rng(28)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.1).astype(np.float32)
    G = _nn(prec)
    f = "conv3d" if len(xs) == 5 else "conv2d"
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    y64 = getattr(f64_nn, f)(x64, w64, list(st), pad)
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dw = from_dev(getattr(G, f + "_backward_kernel")(to_dev(x), to_dev(w), list(st), to_dev(dy)))
    assert _path() == 1
    assert rel(dw, getattr(f64_nn, f + "_backward_kernel")(x64, w64, list(st),
                                                            dy.astype(np.float64))) <= TOL[prec]
    if prec == "tf32":
        return  # a TF32 forward runs the convolution kernel (kind::tf32), tested above
    y = from_dev(getattr(G, f)(to_dev(x), to_dev(w), list(st), pad))
    assert _path() == 1
    assert rel(y, y64) <= TOL[prec]


def test_kernel_equals_stride_with_channels_off_the_chunk_runs_the_conv_kernel(gpu_lib, f64_nn):
    """Channels that are not a multiple of 8 cannot be gathered window by
    window in whole chunks: the convolution kernel runs instead, still on
    the tensor cores, with the same results."""
    rng = np.random.default_rng(29)
    x = rng.uniform(-1, 1, (3, 8, 8, 12)).astype(np.float32)
    w = (rng.standard_normal((2, 2, 12, 20)) * 0.2).astype(np.float32)
    G = _nn("bf16")
    y = from_dev(G.conv2d(to_dev(x), to_dev(w), [2, 2], VALID))
    assert _path() == 1
    assert rel(y, f64_nn.conv2d(x.astype(np.float64), w.astype(np.float64), [2, 2],
                                VALID)) <= TOL["bf16"]


@pytest.mark.parametrize("rows", [1, 3, 5, 7, 9, 15, 17, 29, 33, 56])
def test_tile_heights(gpu_lib, f64_nn, rows):
    """Output heights that select every kind of tile the planner may choose
    (one tile of the output's even height, the fewest tiles of up to 32
    rows, partial last tiles, two co tiles under 128 pixels), forward and
    backward_input, BF16, against the float64 oracle."""
    rng = np.random.default_rng(77)
    x = rng.uniform(-1, 1, (2, rows, 11, 64)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 64, 160)) * 0.06).astype(np.float32)
    G = _nn("bf16")
    y = from_dev(G.conv2d(to_dev(x), to_dev(w), [1, 1], SAME))
    assert _path() == 1
    y64 = f64_nn.conv2d(x.astype(np.float64), w.astype(np.float64), [1, 1], SAME)
    assert rel(y, y64) <= TOL["bf16"]
    dy = rng.standard_normal(y64.shape).astype(np.float32)
    dx = from_dev(G.conv2d_backward_input(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    assert _path() == 1
    ref = f64_nn.conv2d_backward_input(x.astype(np.float64), w.astype(np.float64), [1, 1],
                                       dy.astype(np.float64))
    assert rel(dx, ref) <= TOL["bf16"]
