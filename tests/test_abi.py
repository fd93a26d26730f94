"""The C ABI library: loads, exports every symbol include/owlgpu.h declares,
and rejects malformed arguments with a status (no GPU work is issued)."""

import ctypes
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_header_declares_every_owl_stub_in_scope():
    from owl_gb300._lib import parse_header

    names = set(parse_header())
    ops = ["conv_spatial", "conv_spatial_backward_input", "conv_spatial_backward_kernel",
           "conv_cuboid_im2col", "conv_cuboid_backward_input_im2col",
           "conv_cuboid_backward_kernel_im2col", "conv_dilated_spatial_im2col",
           "conv_dilated_spatial_backward_input_im2col",
           "conv_dilated_spatial_backward_kernel_im2col", "conv_dilated_cuboid_im2col",
           "conv_dilated_cuboid_backward_input_im2col",
           "conv_dilated_cuboid_backward_kernel_im2col", "maxpool_spatial", "avgpool_spatial",
           "maxpool_spatial_backward", "avgpool_spatial_backward", "maxpool_argmax_spatial",
           "maxpool_cuboid", "avgpool_cuboid", "maxpool_cuboid_backward",
           "avgpool_cuboid_backward"]
    for kind in ("float32", "float64"):
        for op in ops:
            assert f"owl_{kind}_ndarray_{op}" in names
            assert f"owlgpu_{kind}_ndarray_{op}" in names


def test_library_exports_every_declared_symbol():
    from owl_gb300 import _lib

    L = _lib.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIBPATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in _lib.PROTOS if n not in exported]
    assert not missing, missing
    for n in _lib.PROTOS:
        assert getattr(L, n) is not None


def test_argument_counts_match_owl_stubs():
    from owl_gb300._lib import PROTOS

    # Owl stub arities (owl_ndarray_conv_impl.h / owl_ndarray_pool_impl.h).
    arity = {"conv_spatial": 17, "conv_spatial_backward_input": 16,
             "conv_spatial_backward_kernel": 16, "conv_cuboid_im2col": 19,
             "conv_cuboid_backward_input_im2col": 18, "conv_cuboid_backward_kernel_im2col": 18,
             "conv_dilated_spatial_im2col": 17, "conv_dilated_cuboid_im2col": 22,
             "conv_dilated_cuboid_backward_input_im2col": 21, "maxpool_spatial": 15,
             "maxpool_spatial_backward": 15, "maxpool_argmax_spatial": 15,
             "maxpool_cuboid": 17, "maxpool_cuboid_backward": 18}
    for op, n in arity.items():
        assert len(PROTOS[f"owl_float32_ndarray_{op}"][1]) == n, op
        assert len(PROTOS[f"owlgpu_float32_ndarray_{op}"][1]) == n + 2, op


def test_invalid_arguments_return_status_without_gpu():
    from owl_gb300 import _lib

    L = _lib.lib()
    buf = (ctypes.c_float * 16)()
    # negative stride: rejected while checking arguments, before any CUDA call
    rc = L.owl_float32_ndarray_conv_spatial(buf, buf, buf, 1, 2, 2, 1, 1, 1, 2, 2, 1, -1, 1,
                                            0, 1, 1)
    assert rc == -1
    assert "stride" in _lib.last_error()
    rc = L.owl_float32_ndarray_maxpool_cuboid(buf, buf, 1, 2, 2, 2, 1, 1, 1, 1, -2, 2, 2, 1, 1,
                                              1, 0)
    assert rc == -1
    rc = L.owl_float32_ndarray_conv_spatial(buf, buf, buf, 1, 2, 2, 1, 1, 1, 2, 2, 1, 1, 1,
                                            7, 1, 1)
    assert rc == -1 and "padding" in _lib.last_error()
    assert L.owlgpu_set_precision(9) == -1


def test_python_layer_raises_like_owl(oracle_nn):
    import numpy as np
    from owl_gb300.dense import InvalidArgument

    x = np.zeros((1, 4, 4, 3), np.float32)
    w = np.zeros((3, 3, 2, 4), np.float32)
    with pytest.raises(InvalidArgument):
        oracle_nn.conv2d(x, w, [1, 1])
    with pytest.raises(InvalidArgument):
        oracle_nn.conv2d(x, np.zeros((3, 3, 3), np.float32), [1, 1])
    with pytest.raises(InvalidArgument):
        oracle_nn.max_pool2d(x, [2, 2], [2])



def _probe_args(params, buf, value):
    """Arguments for an entry point: every array the same small buffer, every
    integer value(name)."""
    import ctypes

    return [ctypes.cast(buf, ctypes.c_void_p) if "*" in t else value(a) for t, a in params]


def _is_stride(a):
    return (a.endswith("stride") and "in_stride" not in a) or a.endswith("scale")


def test_every_host_entry_point_rejects_bad_arguments_without_gpu():
    """Every host drop-in (all kinds, all spellings) checks its arguments
    before touching CUDA: a stride or scale below 1, and a padding flag other
    than 0 (SAME) or 1 (VALID), return OWLGPU_ERR_INVALID with a message."""
    import ctypes

    from owl_gb300 import _lib

    L = _lib.lib()
    buf = (ctypes.c_double * 64)()
    hosts = {n: p for n, (_, p) in _lib.PROTOS.items() if n.startswith("owl_")}
    assert len(hosts) == 152
    for name, params in hosts.items():
        assert any(_is_stride(a) for _, a in params), name
        args = _probe_args(params, buf, lambda a: -1 if _is_stride(a) else 1)
        assert getattr(L, name)(*args) == -1, name
        assert _lib.last_error(), name
        if any(a == "padding" for _, a in params):
            args = _probe_args(params, buf, lambda a: 7 if a == "padding" else 1)
            assert getattr(L, name)(*args) == -1, name
            assert "padding" in _lib.last_error(), name


def test_noalloc_entry_point_checks_like_the_regular_one_without_gpu():
    """The allocation-free backward_kernel applies the regular entry point's
    argument checks (strides 1..2^20, dimensions 0..2^30) and rejects kernels
    beyond its fixed scratch, all before touching CUDA -- including kernels
    whose element count would overflow a 64-bit product."""
    import ctypes

    from owl_gb300 import _lib

    L = _lib.lib()
    buf = (ctypes.c_float * 16)()
    f = L.owlgpu_float32_ndarray_conv_spatial_backward_kernel_noalloc
    # x, dW, dY, B, IC, IR, Ci, KC, KR, OC, OR, Co, row_s, col_s, row_in, col_in, stream
    ok = [buf, buf, buf, 1, 2, 2, 1, 1, 1, 2, 2, 1, 1, 1, 1, 1, None]
    for i, v in [(12, 0), (13, -1), (12, (1 << 20) + 1), (13, 1 << 40), (4, 1 << 31), (6, -2)]:
        args = list(ok)
        args[i] = v
        assert f(*args) == -1, (i, v)
        assert _lib.last_error()
    big = list(ok)
    big[6:9] = [1 << 30, 1 << 30, 1 << 30]  # Ci, KC, KR: 2^90 kernel elements
    big[11] = 1 << 30
    assert f(*big) == -1
    assert "16 MiB" in _lib.last_error()
