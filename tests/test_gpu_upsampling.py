"""upsampling2d on the GPU against the oracle: Owl's known-answer tests
through the host drop-in (float32) and the device entry points (float64),
and bit-exact parity on random data for the vector (16-byte) and scalar
paths, the stub's clamp of extra output cols/rows, and `out=`."""

import numpy as np
import pytest

from gpu_util import from_dev, to_dev
from upsampling_cases import UP_CASES, run_up_case, up_id

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_nn(gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend("fp32"))


@pytest.mark.parametrize("c", UP_CASES, ids=[up_id(c) for c in UP_CASES])
def test_golden_host_float32(gpu_nn, c):
    got, expected = run_up_case(gpu_nn, c, np.float32)
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("c", UP_CASES, ids=[up_id(c) for c in UP_CASES])
def test_golden_device_float64(gpu_nn, c):
    got, expected = run_up_case(gpu_nn, c, np.float64, conv=to_dev, back=from_dev)
    assert np.array_equal(got, expected)


# (shape, size): channels % 4 == 0 take the float4 path (float64: % 2, double2)
CASES = [((2, 5, 7, 4), (2, 3)), ((3, 4, 3, 5), (3, 2)), ((2, 6, 6, 64), (2, 2)),
         ((1, 3, 9, 3), (1, 4)), ((4, 7, 5, 8), (1, 1)), ((2, 16, 16, 32), (3, 3))]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape,size", CASES)
def test_bit_exact_vs_oracle(gpu_nn, oracle_nn, dt, shape, size):
    rng = np.random.default_rng(23)
    x = rng.uniform(-1, 1, shape).astype(dt)
    oshape = (shape[0], shape[1] * size[0], shape[2] * size[1], shape[3])
    dy = rng.standard_normal(oshape).astype(dt)
    y_ref = oracle_nn.upsampling2d(x, list(size))
    dx_ref = oracle_nn.upsampling2d_backward(x, list(size), dy)
    assert np.array_equal(from_dev(gpu_nn.upsampling2d(to_dev(x), list(size))), y_ref)
    assert np.array_equal(
        from_dev(gpu_nn.upsampling2d_backward(to_dev(x), list(size), to_dev(dy))), dx_ref)
    # host drop-in
    assert np.array_equal(gpu_nn.upsampling2d(x, list(size)), y_ref)
    assert np.array_equal(gpu_nn.upsampling2d_backward(x, list(size), dy), dx_ref)


@pytest.mark.parametrize("oc,or_", [(9, 5), (5, 9), (2, 3)])
def test_stub_clamp_vs_oracle(gpu_lib, oracle_nn, oc, or_):
    """The C entry point with output extents other than input * scale
    (the stub clamps into the last input col/row): IC = 3, IR = 2, 2 x 2."""
    import torch

    rng = np.random.default_rng(5)
    dy = rng.standard_normal((2, oc, or_, 3)).astype(np.float32)
    ref = np.empty((2, 3, 2, 3), dtype=np.float32)
    oracle_nn.b.stub("float32", "upsampling_spatial_backward", ref, dy, 2, 3, 2, 3, oc, or_, 2, 2)
    host = np.full((2, 3, 2, 3), np.nan, dtype=np.float32)
    rc = gpu_lib.owl_float32_ndarray_upsampling_spatial_backward(
        host.ctypes.data, dy.ctypes.data, 2, 3, 2, 3, oc, or_, 2, 2)
    assert rc == 0 and np.array_equal(host, ref)
    ddy = to_dev(dy)
    ddx = torch.full((2, 3, 2, 3), float("nan"), device="cuda")
    rc = gpu_lib.owlgpu_float32_ndarray_upsampling_spatial_backward(
        ddx.data_ptr(), ddy.data_ptr(), 2, 3, 2, 3, oc, or_, 2, 2, 0,
        torch.cuda.current_stream().cuda_stream)
    assert rc == 0 and np.array_equal(from_dev(ddx), ref)


def test_forward_rejects_mismatched_output(gpu_lib):
    x = np.zeros((1, 2, 2, 4), dtype=np.float32)
    y = np.zeros((1, 5, 4, 4), dtype=np.float32)
    rc = gpu_lib.owl_float32_ndarray_upsampling_spatial(x.ctypes.data, y.ctypes.data,
                                                        1, 2, 2, 4, 5, 4, 2, 2)
    assert rc < 0


def test_out_variant_device(gpu_nn):
    import torch

    x = to_dev(np.arange(16, dtype=np.float32).reshape(1, 2, 2, 4))
    out = torch.full((1, 4, 6, 4), 9.0, device="cuda")
    r = gpu_nn.upsampling2d(x, [2, 3], out=out)
    assert r.data_ptr() == out.data_ptr()
    assert np.array_equal(from_dev(out), from_dev(x).repeat(2, axis=1).repeat(3, axis=2))
