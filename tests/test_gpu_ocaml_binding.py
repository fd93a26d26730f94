"""The generated OCaml stubs on the GPU: a conv2d and a complex average pool
called the way OCaml calls them (Bigarray descriptors, tagged ints) give the
host drop-in's results, which the oracle checks."""

import ctypes

import numpy as np
import pytest

from test_ocaml_binding import _CamlBa, _tag, build_stubs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stubs(gpu_lib, tmp_path_factory):
    L = ctypes.CDLL(str(build_stubs(tmp_path_factory.mktemp("ocaml_gpu"))))
    L.shim_last_failure.restype = ctypes.c_char_p
    return L


def _ba(a, keep):
    b = _CamlBa(a.ctypes.data, a.ndim, 0, None)
    for i, d in enumerate(a.shape):
        b.dim[i] = d
    keep.append(b)
    return ctypes.cast(ctypes.pointer(b), ctypes.c_void_p)


def test_conv2d_through_the_ocaml_stub(stubs, oracle_nn):
    rng = np.random.default_rng(31)
    x = rng.uniform(-1, 1, (2, 9, 8, 5)).astype(np.float32)
    w = rng.uniform(-1, 1, (3, 3, 5, 7)).astype(np.float32)
    y = np.full((2, 9, 8, 7), np.nan, np.float32)
    keep = []
    # batches, cols, rows, in_ch, 3x3 kernel, 9x8 output, out_ch, strides 1, SAME, in-strides
    ints = [2, 9, 8, 5, 3, 3, 9, 8, 7, 1, 1, 0, 1, 1]
    stubs.shim_reset()
    stubs.owlgpu_stub_float32_ndarray_conv_spatial_native(
        _ba(x, keep), _ba(w, keep), _ba(y, keep), *map(_tag, ints))
    assert stubs.shim_last_failure() == b""
    assert stubs.shim_entered() == 1 and stubs.shim_left() == 1
    ref = oracle_nn.conv2d(x, w, [1, 1], "SAME")
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 1e-4


def test_complex_avg_pool_through_the_ocaml_stub(stubs, oracle_nn):
    rng = np.random.default_rng(32)
    x = (rng.uniform(-1, 1, (2, 6, 6, 3)) + 1j * rng.uniform(-1, 1, (2, 6, 6, 3))).astype(
        np.complex64)
    y = np.zeros((2, 3, 3, 3), np.complex64)
    keep = []
    # batches, cols, rows, channels, 2x2 window, 3x3 output, strides 2, VALID, in-strides
    ints = [2, 6, 6, 3, 2, 2, 3, 3, 2, 2, 1, 1, 1]
    stubs.shim_reset()
    stubs.owlgpu_stub_complex32_ndarray_avgpool_spatial_native(_ba(x, keep), _ba(y, keep),
                                                               *map(_tag, ints))
    assert stubs.shim_last_failure() == b""
    assert np.array_equal(y, oracle_nn.avg_pool2d(x, [2, 2], [2, 2], "VALID"))


def _fn(stubs, name):
    f = getattr(stubs, name)
    f.restype = ctypes.c_void_p
    return f


def test_device_resident_arrays_through_the_ocaml_stubs(stubs, oracle_nn):
    """Owl arrays kept on the GPU between calls, as OCaml would hold them:
    a stream and device buffers in custom blocks, Bigarray upload, a conv2d
    and a ReLU dense layer (its bias passed as `Some buf`) on device
    buffers, download; then the collector's finalisers release them."""
    rng = np.random.default_rng(33)
    x = rng.uniform(-1, 1, (2, 9, 8, 5)).astype(np.float32)
    w = rng.uniform(-1, 1, (3, 3, 5, 7)).astype(np.float32)
    a = rng.uniform(-1, 1, (6, 20)).astype(np.float32)
    b = rng.uniform(-1, 1, (20, 4)).astype(np.float32)
    bias = rng.uniform(-1, 1, 4).astype(np.float32)
    keep = []
    V = ctypes.c_void_p
    stubs.shim_reset()
    s = V(_fn(stubs, "owlgpu_dstub_stream_create")(_tag(0)))
    bufs = {}
    for k, arr in (("x", x), ("w", w), ("y", np.zeros((2, 9, 8, 7), np.float32)), ("a", a),
                   ("b", b), ("bias", bias), ("c", np.zeros((6, 4), np.float32))):
        bufs[k] = V(_fn(stubs, "owlgpu_dstub_buf_create")(_tag(arr.nbytes), s))
        assert _fn(stubs, "owlgpu_dstub_buf_bytes")(bufs[k]) == (arr.nbytes << 1) | 1
        if k in ("x", "w", "a", "b", "bias"):
            stubs.owlgpu_dstub_buf_upload(bufs[k], _ba(arr, keep), s)
    assert stubs.shim_last_failure() == b""
    ints = [2, 9, 8, 5, 3, 3, 9, 8, 7, 1, 1, 0, 1, 1]
    stubs.owlgpu_dstub_float32_ndarray_conv_spatial_native(
        bufs["x"], bufs["w"], bufs["y"], *map(_tag, ints), _tag(0), s)
    some_bias = (ctypes.c_void_p * 1)(bufs["bias"].value)  # the block of `Some bias`
    stubs.owlgpu_dstub_float32_dot_native(
        bufs["a"], bufs["b"], bufs["c"], _tag(6), _tag(4), _tag(20), _tag(0), _tag(0),
        ctypes.cast(some_bias, V), _tag(1), _tag(0), s)
    stubs.owlgpu_dstub_stream_sync(s)
    y = np.full((2, 9, 8, 7), np.nan, np.float32)
    c = np.full((6, 4), np.nan, np.float32)
    stubs.owlgpu_dstub_buf_download(bufs["y"], _ba(y, keep), s)
    stubs.owlgpu_dstub_buf_download(bufs["c"], _ba(c, keep), s)
    assert stubs.shim_last_failure() == b""
    ref = oracle_nn.conv2d(x, w, [1, 1], "SAME")
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 1e-4
    ref_c = np.maximum(a.astype(np.float64) @ b + bias, 0)
    assert np.max(np.abs(c - ref_c)) <= 1e-5 * np.max(np.abs(a) @ np.abs(b))
    # the collector: finalisers free the device memory and the stream
    for v in bufs.values():
        stubs.shim_finalize(v)
        assert _fn(stubs, "owlgpu_dstub_buf_bytes")(v) == 1  # Val_long(0)
    stubs.shim_finalize(s)
    from owl_gb300 import _lib

    assert _lib.lib().owlgpu_device_status() == 0
