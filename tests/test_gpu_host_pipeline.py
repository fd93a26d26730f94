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
