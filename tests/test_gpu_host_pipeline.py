"""The host drop-in stages batch-independent calls in batch chunks on three
streams (copy in, compute, copy out).  Chunked results must equal the
device-resident call on the same data bit for bit: every sample is computed
independently and a convolution's accumulation order does not depend on
the batch.  Calls large enough to be split (>= 48 MB of batched traffic)."""

import numpy as np
import pytest

from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_chunked_conv_equals_device_call(gpu_lib, precision):
    import torch

    from owl_gb300.dense import NN, GpuBackend

    nn = NN(GpuBackend(precision))
    rng = np.random.default_rng(60)
    x = rng.uniform(-1, 1, (24, 40, 40, 64)).astype(np.float32)      # 9.8 MB
    w = (rng.standard_normal((3, 3, 64, 64)) * 0.05).astype(np.float32)
    dy = rng.standard_normal((24, 40, 40, 64)).astype(np.float32)
    xb = np.concatenate([x] * 4)                                      # 39 MB: 2+ chunks
    dyb = np.concatenate([dy] * 4)
    y_host = nn.conv2d(xb, w, [1, 1], "SAME")
    y_dev = from_dev(nn.conv2d(to_dev(xb), to_dev(w), [1, 1], "SAME"))
    assert np.array_equal(y_host, y_dev)
    dx_host = nn.conv2d_backward_input(xb, w, [1, 1], dyb)
    dx_dev = from_dev(nn.conv2d_backward_input(to_dev(xb), to_dev(w), [1, 1], to_dev(dyb)))
    assert np.array_equal(dx_host, dx_dev)
    out = np.empty_like(y_host)
    nn.conv2d(xb, w, [1, 1], "SAME", out=out)
    assert np.array_equal(out, y_dev)


def test_chunked_pooling_equals_device_call(gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    nn = NN(GpuBackend("fp32"))
    rng = np.random.default_rng(61)
    x = rng.uniform(-1, 1, (16, 32, 32, 16, 32)).astype(np.float32)   # 67 MB
    k, s = [2, 2, 2], [2, 2, 2]
    a = nn.avg_pool3d(x, k, s, "SAME")
    assert np.array_equal(a, from_dev(nn.avg_pool3d(to_dev(x), k, s, "SAME")))
    m = nn.max_pool3d(x, k, s, "SAME")
    assert np.array_equal(m, from_dev(nn.max_pool3d(to_dev(x), k, s, "SAME")))
    g = rng.standard_normal(a.shape).astype(np.float32)
    da = nn.avg_pool3d_backward("SAME", x, k, s, g)
    assert np.array_equal(da, from_dev(nn.avg_pool3d_backward("SAME", to_dev(x), k, s,
                                                               to_dev(g))))


def _pinned(a):
    import torch

    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
    t.numpy()[...] = a
    return t.numpy()


CASES_IN_PLACE = [
    # input, kernel, stride, rate, padding
    ((6, 20, 18, 64), (3, 3, 64, 128), (1, 1), (1, 1), "SAME"),
    ((4, 28, 28, 64), (3, 3, 64, 128), (2, 2), (1, 1), "VALID"),
    ((3, 16, 16, 32), (1, 1, 32, 64), (2, 2), (1, 1), "SAME"),   # residue classes with no tap
    ((2, 17, 19, 40), (3, 3, 40, 24), (1, 1), (2, 2), "SAME"),
]


@pytest.mark.parametrize("precision", ["bf16", "bf16x3"])
@pytest.mark.parametrize("case", CASES_IN_PLACE)
def test_page_locked_conv_equals_device_call(gpu_lib, precision, case):
    """Tensor-core convolutions through the host drop-in from page-locked
    arrays (staged in batch chunks on the copy streams) into page-locked
    `~out` arrays: the result is the device call's, bit for bit, for forward,
    backward_input (strided, including zero-filled residue classes) and
    backward_kernel."""
    from owl_gb300 import _lib
    from owl_gb300.dense import NN, GpuBackend

    nn = NN(GpuBackend(precision))
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(62)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.05).astype(np.float32)
    st, rate = list(st), list(rate)
    y_dev = from_dev(nn.dilated_conv2d(to_dev(x), to_dev(w), st, rate, pad))
    dy = rng.standard_normal(y_dev.shape).astype(np.float32)
    dx_dev = from_dev(nn.dilated_conv2d_backward_input(to_dev(x), to_dev(w), st, rate, to_dev(dy)))
    dw_dev = from_dev(nn.dilated_conv2d_backward_kernel(to_dev(x), to_dev(w), st, rate, to_dev(dy)))
    px, pw, pdy = _pinned(x), _pinned(w), _pinned(dy)
    oy = _pinned(np.full(y_dev.shape, np.nan, np.float32))
    odx = _pinned(np.full(x.shape, np.nan, np.float32))
    odw = _pinned(np.full(w.shape, np.nan, np.float32))
    nn.dilated_conv2d(px, pw, st, rate, pad, out=oy)
    assert _lib.lib().owlgpu_last_conv_path() == 1
    nn.dilated_conv2d_backward_input(px, pw, st, rate, pdy, out=odx)
    nn.dilated_conv2d_backward_kernel(px, pw, st, rate, pdy, out=odw)
    assert np.array_equal(oy, y_dev)
    assert np.array_equal(odx, dx_dev)
    assert np.array_equal(odw, dw_dev)
    assert _lib.lib().owlgpu_device_status() == 0


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_chunked_backward_kernel(gpu_lib, precision):
    """A float32 backward_kernel from page-locked arrays large enough to be
    staged in batch chunks (51 MB of X and dY): each chunk's weight gradient
    goes to its own partial and the partials are summed in chunk order.  The
    products are the device call's; only the grouping of the float32 sums
    differs, so the result agrees with the device call to float32 rounding
    (1e-5 relative) and is bit-identical from one call to the next."""
    from owl_gb300.dense import NN, GpuBackend

    nn = NN(GpuBackend(precision))
    rng = np.random.default_rng(63)
    x = rng.uniform(-1, 1, (32, 56, 56, 64)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 64, 64)) * 0.05).astype(np.float32)
    dy = rng.standard_normal((32, 56, 56, 64)).astype(np.float32)
    dw_dev = from_dev(nn.conv2d_backward_kernel(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    px, pw, pdy = _pinned(x), _pinned(w), _pinned(dy)
    a = _pinned(np.zeros(w.shape, np.float32))
    b = _pinned(np.zeros(w.shape, np.float32))
    nn.conv2d_backward_kernel(px, pw, [1, 1], pdy, out=a)
    nn.conv2d_backward_kernel(px, pw, [1, 1], pdy, out=b)
    assert np.array_equal(a, b)
    err = float(np.max(np.abs(a.astype(np.float64) - dw_dev)) / np.max(np.abs(dw_dev)))
    assert err <= 1e-5, err
