"""The tensor-core kernels' bounded pipeline waits, exercised without any GPU
fault.  With the wait limit cut to 2000 cycles (about 1 us) the first
barrier waits of a BF16 convolution run out long before their stage lands:
every CTA unwinds (waits for its own copies and MMAs, frees tensor memory,
returns) and the call reports the timeout -- through the device status word
for the device entry points, as OWLGPU_ERR_TIMEOUT from the host drop-in.
With the limit restored the context is intact and the same calls are
correct again."""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu


def test_short_wait_limit_times_out_and_context_recovers(gpu_lib, oracle_nn):
    import torch

    from owl_gb300._lib import OwlGpuError
    from owl_gb300.dense import NN, GpuBackend

    L = gpu_lib
    G = NN(GpuBackend("bf16"))
    rng = np.random.default_rng(41)
    x = rng.uniform(-1, 1, (2, 40, 40, 64)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 64, 64)) * 0.06).astype(np.float32)
    dy = rng.standard_normal((2, 40, 40, 64)).astype(np.float32)
    xd, wd, dyd = to_dev(x), to_dev(w), to_dev(dy)
    assert L.owlgpu_device_status() == 0

    prev = L.owlgpu_set_wait_limit(2000)
    try:
        # device entry points: the status word reports the unwound launches
        G.conv2d(xd, wd, [1, 1], "SAME")
        torch.cuda.synchronize()
        assert L.owlgpu_device_status() == -5  # OWLGPU_ERR_TIMEOUT, word cleared
        G.conv2d_backward_kernel(xd, wd, [1, 1], dyd)
        torch.cuda.synchronize()
        assert L.owlgpu_device_status() == -5
        # host drop-in: the call itself returns the timeout
        with pytest.raises(OwlGpuError) as e:
            G.conv2d(x, w, [1, 1], "SAME")
        assert e.value.status == -5
    finally:
        L.owlgpu_set_wait_limit(0)
    assert prev == 4000000000
    assert L.owlgpu_device_status() == 0

    # recovered: the same calls are correct
    x64, w64 = x.astype(np.float64), w.astype(np.float64)
    y = from_dev(G.conv2d(xd, wd, [1, 1], "SAME"))
    assert rel(y, oracle_nn.conv2d(x64, w64, [1, 1], "SAME")) <= 1e-2
    dw = from_dev(G.conv2d_backward_kernel(xd, wd, [1, 1], dyd))
    assert rel(dw, oracle_nn.conv2d_backward_kernel(x64, w64, [1, 1],
                                                    dy.astype(np.float64))) <= 1e-2
    assert np.allclose(G.conv2d(x, w, [1, 1], "SAME"), y, rtol=0, atol=0)
    assert L.owlgpu_device_status() == 0
