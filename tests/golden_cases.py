"""Replay Owl's own conv/pool unit tests (tests/golden/owl_golden.json,
extracted by tests/golden/make_golden.py) through ``owl_gb300.dense.NN``
with any stub provider."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = json.loads((Path(__file__).parent / "golden" / "owl_golden.json").read_text())
CASES = GOLDEN["cases"]
HELPERS = GOLDEN["helpers"]
TOL = GOLDEN["tolerance_sum_abs"]  # Owl: close a b = sum |a - b| < 5e-4


def case_id(c) -> str:
    return f"{c['file'].replace('.ml', '')}:{c['module']}.{c['fun']}"


def _make(recipe, shape, seq, dtype):
    n = int(np.prod(shape))
    if recipe == "seq1":
        return np.arange(1, n + 1, dtype=np.float64).reshape(shape).astype(dtype)
    if recipe == "seq0":
        return np.arange(0, n, dtype=np.float64).reshape(shape).astype(dtype)
    if recipe == "seq1n":
        return (np.arange(1, n + 1, dtype=dtype) / dtype(n)).reshape(shape)
    if recipe == "ones":
        return np.ones(shape, dtype=dtype)
    if recipe == "seqk":
        return _make("seq1" if seq else "ones", shape, seq, dtype)
    raise ValueError(recipe)


def run_case(nn, c, dtype=np.float32, to_dev=None, from_dev=None):
    """Compute one golden case with ``nn``; returns the result as numpy.
    ``to_dev``/``from_dev`` move arrays to and from a device backend."""
    to_dev = to_dev or (lambda a: a)
    from_dev = from_dev or (lambda a: np.asarray(a))
    if c["helper"] == "test_forward":
        ishape, kshape, stride = c["args"]
        x = to_dev(np.ones(ishape, dtype=dtype))
        w = to_dev(np.ones(kshape, dtype=dtype))
        return from_dev(nn.transpose_conv2d(x, w, stride, c["pad"]))
    fn, rx, rw, rdy = HELPERS[c["helper"]]
    seq = c["labels"].get("seq") == "true"
    a = c["args"]
    pad = c["pad"]
    if fn.startswith(("max_pool", "avg_pool")):
        ishape, kernel, stride = a
        x = _make(rx, ishape, seq, dtype)
        xd = to_dev(x)
        fwd = getattr(nn, fn.replace("_backward", ""))
        y = fwd(xd, kernel, stride, pad)
        if rdy is None:
            return from_dev(y)
        dy = to_dev(_make(rdy, tuple(np.asarray(from_dev(y)).shape), seq, dtype))
        return from_dev(getattr(nn, fn)(pad, xd, kernel, stride, dy))
    ishape, kshape = a[0], a[1]
    x = to_dev(_make(rx, ishape, seq, dtype))
    w = to_dev(_make(rw, kshape, seq, dtype))
    dilated = fn.startswith("dilated")
    if dilated:
        rate = a[2]
        stride = [int(v) for v in c["labels"].get("stride", [1] * len(rate))]
    else:
        stride = a[2]
    base = fn.split("_backward")[0]
    if dilated:
        y = getattr(nn, base)(x, w, stride, rate, pad)
    else:
        y = getattr(nn, base)(x, w, stride, pad)
    if rdy is None:
        return from_dev(y)
    dy = to_dev(_make(rdy, tuple(np.asarray(from_dev(y)).shape), seq, dtype))
    if dilated:
        return from_dev(getattr(nn, fn)(x, w, stride, rate, dy))
    return from_dev(getattr(nn, fn)(x, w, stride, dy))


def check_forward_closed_form(result, c) -> bool:
    """Restatement of test/unit_transpose_conv2d.ml:51-88 (test_forward):
    the expected transposed-conv output of all-ones inputs is built from three
    'magic' numbers and compared with exact equality."""
    ishape, kshape, stride = c["args"]
    m = c["magic"]
    pad = c["pad"]
    s = result.shape
    ph = 0 if pad == "SAME" else stride[0] - 1
    pw = 0 if pad == "SAME" else stride[1] - 1
    exp = np.zeros(s, dtype=result.dtype)
    for n in range(s[0]):
        for k in range(s[3]):
            for w in range(pw, s[2] - pw):
                for h in range(ph, s[1] - ph):
                    h_in = h % stride[0] == 0 and ph < h < s[1] - 1 - ph
                    w_in = w % stride[1] == 0 and pw < w < s[2] - 1 - pw
                    add = m[1] if (h_in and w_in) else (m[2] if (h_in or w_in) else 0.0)
                    exp[n, h, w, k] = m[0] + add
            if pad == "VALID":
                exp[n, :, 0, k] = exp[n, :, 1, k]
                exp[n, :, -1, k] = exp[n, :, -2, k]
                exp[n, 0, :, k] = exp[n, 1, :, k]
                exp[n, -1, :, k] = exp[n, -2, :, k]
    return bool(np.array_equal(result, exp))


def matches(result, c) -> tuple[bool, float]:
    if c["helper"] == "test_forward":
        return check_forward_closed_form(result, c), 0.0
    exp = np.asarray(c["expected"], dtype=np.float64)
    r = np.asarray(result, dtype=np.float64).reshape(-1)
    if r.size != exp.size:
        return False, float("inf")
    err = float(np.abs(r - exp).sum())
    return err < TOL, err


# Owl's MEC and naive conv stubs take the im2col / GEBP stubs' arguments
# (owl_ndarray_conv_impl.h:1570-3086); Owl's unit_conv_mec_naive.ml runs the
# conv2d and conv3d suites on them.
MEC = {"conv_spatial": "conv_spatial_mec",
       "conv_spatial_backward_input": "conv_spatial_backward_input_mec",
       "conv_spatial_backward_kernel": "conv_spatial_backward_kernel_mec",
       "conv_cuboid_im2col": "conv_cuboid_mec",
       "conv_cuboid_backward_input_im2col": "conv_cuboid_backward_input_mec",
       "conv_cuboid_backward_kernel_im2col": "conv_cuboid_backward_kernel_mec"}
NAIVE = {k: v.replace("_mec", "_naive") for k, v in MEC.items()}
MEC_NAIVE_FILES = ("unit_conv2d_generic.ml", "unit_conv3d_generic.ml")


class Spelling:
    """A stub provider that sends the conv stubs to another spelling (MEC or
    naive) of the same function; everything else goes through unchanged."""

    def __init__(self, inner, names):
        self.inner, self.names = inner, names
        self.name = f"{inner.name}+{next(iter(names.values())).rsplit('_', 1)[1]}"

    def stub(self, kind, op, *args):
        self.inner.stub(kind, self.names.get(op, op), *args)

    def empty(self, like, shape, dtype=None):
        return self.inner.empty(like, shape, dtype)

    def shape(self, a):
        return self.inner.shape(a)

    def reshape(self, a, shape):
        return self.inner.reshape(a, shape)
