"""The Python mirror's argument checks (owl_dense_ndarray_generic.ml's
`INVALID_ARGUMENT` cases, restated in owl_gb300/dense.py): each rejects a bad
call with Owl's message before any stub runs.  The messages are built only
when a check fails, so these tests pin that they still are."""

import numpy as np
import pytest

from owl_gb300.dense import InvalidArgument, _kind


def test_conv2d_dimension_message(oracle_nn):
    x = np.zeros((2, 8, 8), np.float32)
    w = np.zeros((3, 3, 8, 4), np.float32)
    with pytest.raises(InvalidArgument, match=r"conv2d: input dimension = 3 \(should be 4\)"):
        oracle_nn.conv2d(x, w, [1, 1], "SAME")


def test_conv2d_channel_message(oracle_nn):
    x = np.zeros((2, 8, 8, 5), np.float32)
    w = np.zeros((3, 3, 4, 4), np.float32)
    with pytest.raises(InvalidArgument, match="the 4th dimension of input shape should be equal"):
        oracle_nn.conv2d(x, w, [1, 1], "SAME")


def test_out_shape_message(oracle_nn):
    x = np.zeros((2, 8, 8, 4), np.float32)
    w = np.zeros((3, 3, 4, 6), np.float32)
    out = np.zeros((2, 8, 8, 5), np.float32)
    with pytest.raises(InvalidArgument, match=r"out: shape \[2, 8, 8, 5\] should be \[2, 8, 8, 6\]"):
        oracle_nn.conv2d(x, w, [1, 1], "SAME", out=out)


def test_padding_message(oracle_nn):
    x = np.zeros((1, 4, 4, 2), np.float32)
    w = np.zeros((2, 2, 2, 2), np.float32)
    with pytest.raises(InvalidArgument, match="padding must be SAME or VALID"):
        oracle_nn.conv2d(x, w, [1, 1], "FULL")


def test_backward_shape_message(oracle_nn):
    x = np.zeros((2, 8, 8, 4), np.float32)
    w = np.zeros((3, 3, 4, 6), np.float32)
    dy = np.zeros((2, 8, 8, 7), np.float32)
    with pytest.raises(InvalidArgument, match="does not match input/kernel"):
        oracle_nn.conv2d_backward_input(x, w, [1, 1], dy)


def test_element_kinds():
    assert _kind(np.zeros(1, np.float32)) == "float32"
    assert _kind(np.zeros(1, np.float64)) == "float64"
    assert _kind(np.zeros(1, np.complex64)) == "complex32"
    assert _kind(np.zeros(1, np.complex128)) == "complex64"
    assert _kind(np.zeros(2, np.float32)) == "float32"  # cached kind, same answer
    with pytest.raises(InvalidArgument, match="unsupported element kind int32"):
        _kind(np.zeros(1, np.int32))


def test_mixed_host_and_device_arrays_rejected():
    """A stub call gets either device tensors or host arrays: a host pointer
    handed to a device entry point would be dereferenced on the GPU."""
    torch = pytest.importorskip("torch")
    from owl_gb300.dense import NN, GpuBackend

    nn = NN(GpuBackend("fp32"))
    x = np.zeros((1, 4, 4, 2), np.float32)
    w = torch.zeros((2, 2, 2, 2))
    with pytest.raises(InvalidArgument):
        nn.conv2d(x, w, [1, 1], "SAME")
