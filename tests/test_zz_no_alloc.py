"""The allocation-free backward-kernel entry point.

owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc serves callers
that cannot let a library allocate GPU memory during a call (their HBM is
owned by another allocator's arena, or their latency/memory budget forbids
driver allocations): its split-K scratch is a fixed device array inside the
library.  This test calls it through the C ABI, on device buffers that the
test itself allocates, and checks it against the allocating entry point
(owlgpu_float32_ndarray_conv_spatial_backward_kernel at FP32) within the
float32 tolerance used by the other parity tests (1e-4 relative), on two
calls in a row -- the second call sees the scratch the first one left.

The file name sorts last so that a `-x` run has executed every other test
before this one; it passes alone in a fresh process as well.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4  # float32 FP32-kernel tolerance, as in test_gpu_parity.py


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _args(x, dy, w_shape, stride):
    B, IC, IR, Ci = x.shape
    KC, KR, _, Co = w_shape
    _, OC, OR, _ = dy.shape
    return [B, IC, IR, Ci, KC, KR, OC, OR, Co, stride[1], stride[0], 1, 1]


@pytest.mark.parametrize("shape", [
    ((4, 20, 20, 32), (3, 3, 32, 48), (1, 1)),
    ((2, 15, 15, 64), (3, 3, 64, 128), (2, 2)),
    # a wide kernel over few pixels: the split count the pixels would allow
    # (4) is cut to the 3 partials of 1,179,648 elements that fit the scratch
    ((1, 16, 16, 256), (3, 3, 256, 512), (1, 1)),
    # exactly the element limit: one split, written straight into dW
    ((1, 8, 8, 512), (4, 4, 512, 512), (1, 1)),
])
def test_noalloc_matches_allocating_entry_point(gpu_lib, shape):
    import torch

    from owl_gb300 import _lib

    xs, ws, stride = shape
    rng = np.random.default_rng(31)
    B, IC, IR, Ci = xs
    KC, KR, _, Co = ws
    from owl_gb300.dense import calc_conv2d_output_shape

    pad = "SAME" if stride == (1, 1) else "VALID"
    OC, OR = calc_conv2d_output_shape(pad, IC, IR, KC, KR, stride[1], stride[0])
    x = torch.from_numpy(rng.uniform(-1, 1, xs).astype(np.float32)).cuda()
    dy = torch.from_numpy(rng.standard_normal((B, OC, OR, Co)).astype(np.float32)).cuda()
    ref = torch.empty(ws, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    a = _args(x, dy, ws, stride)
    _lib.call("owlgpu_float32_ndarray_conv_spatial_backward_kernel", x.data_ptr(),
              ref.data_ptr(), dy.data_ptr(), *a, 0, stream)
    torch.cuda.synchronize()
    expect = ref.cpu().numpy()
    for _ in range(2):  # two calls in a row share the device scratch
        out = torch.full(ws, float("nan"), dtype=torch.float32, device="cuda")
        _lib.call("owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc", x.data_ptr(),
                  out.data_ptr(), dy.data_ptr(), *a, stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert _rel(got, expect) <= TOL


def test_noalloc_rejects_kernels_beyond_its_scratch(gpu_lib):
    import torch

    from owl_gb300 import _lib

    L = _lib.lib()
    x = torch.zeros(16, device="cuda")
    # 3 x 3 x 1024 x 1024 = 9.4M elements > the 4,194,304-element limit
    rc = L.owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc(
        x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 4, 4, 1024, 3, 3, 4, 4, 1024, 1, 1, 1, 1,
        torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert "16 MiB" in _lib.last_error()
