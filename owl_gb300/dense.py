"""Host-side mirror of Owl's dense-ndarray NN functions over libowlgpu.

Owl's OCaml layer (src/owl/dense/owl_dense_ndarray_generic.ml, "G") checks
shapes, infers output shapes (src/base/misc/owl_utils_infer_shape.ml, "IS"),
allocates the output and calls a C stub.  That layer stays OCaml in a real
integration and only its externals change; it cannot be compiled here, so this
module restates it in Python with the same function names, argument meaning
and errors, parameterised by the stub provider:

    NN(backend).conv2d(x, w, [1, 1], padding=SAME)

mirrors ``Owl.Dense.Ndarray.S.conv2d ~padding x w [|1;1|]`` with the stubs
of ``backend``.  This is the same trick as Owl's functorised tests
(test/unit_conv2d_generic.ml:7): the product backend (GpuBackend) calls the
CUDA library, the test backends call the CPU oracle or Owl's own compiled
stubs, and the golden-vector tests run unchanged against each.

Arrays are numpy arrays (host drop-in path) or torch CUDA tensors (device
resident path) for the GPU backend.
"""

from __future__ import annotations

import math
from typing import Any, Sequence

import numpy as np

SAME = "SAME"
VALID = "VALID"


class InvalidArgument(ValueError):
    """Mirror of Owl_exception.INVALID_ARGUMENT (raised before any stub call)."""


def _verify(cond: bool, msg) -> None:
    """Raise InvalidArgument(msg) unless cond; msg may be a function that
    builds the message (formatted only on failure: these checks run on
    every call)."""
    if not cond:
        raise InvalidArgument(msg() if callable(msg) else msg)


# ---- IS: shape and padding math (owl_utils_infer_shape.ml) ----------------

def calc_conv2d_output_shape(padding, input_cols, input_rows, kernel_cols, kernel_rows,
                             row_stride, col_stride):
    """IS:19-45.  Computed in float with ceil, as Owl does."""
    if padding == SAME:
        oc = math.ceil(float(input_cols) / float(col_stride))
        orr = math.ceil(float(input_rows) / float(row_stride))
    else:
        oc = math.ceil((float(input_cols) - float(kernel_cols) + 1.0) / float(col_stride))
        orr = math.ceil((float(input_rows) - float(kernel_rows) + 1.0) / float(row_stride))
    return int(oc), int(orr)


def calc_conv3d_output_shape(padding, input_cols, input_rows, input_dpts, kernel_cols,
                             kernel_rows, kernel_dpts, row_stride, col_stride, dpt_stride):
    """IS:127-164."""
    oc, orr = calc_conv2d_output_shape(padding, input_cols, input_rows, kernel_cols,
                                       kernel_rows, row_stride, col_stride)
    if padding == SAME:
        od = math.ceil(float(input_dpts) / float(dpt_stride))
    else:
        od = math.ceil((float(input_dpts) - float(kernel_dpts) + 1.0) / float(dpt_stride))
    return oc, orr, int(od)


def calc_transpose_conv2d_output_shape(padding, input_cols, input_rows, kernel_cols,
                                       kernel_rows, row_stride, col_stride):
    """IS:48-68."""
    if padding == SAME:
        return input_cols * col_stride, input_rows * row_stride
    return (input_cols * col_stride + max(kernel_cols - col_stride, 0),
            input_rows * row_stride + max(kernel_rows - row_stride, 0))


def calc_transpose_conv3d_output_shape(padding, input_cols, input_rows, input_dpts,
                                       kernel_cols, kernel_rows, kernel_dpts, row_stride,
                                       col_stride, dpt_stride):
    """IS:167-195."""
    oc, orr = calc_transpose_conv2d_output_shape(padding, input_cols, input_rows, kernel_cols,
                                                 kernel_rows, row_stride, col_stride)
    if padding == SAME:
        od = input_dpts * dpt_stride
    else:
        od = input_dpts * dpt_stride + max(kernel_dpts - dpt_stride, 0)
    return oc, orr, od


def calc_conv2d_padding(input_cols, input_rows, kernel_cols, kernel_rows, output_cols,
                        output_rows, row_stride, col_stride):
    """IS:71-92: (pad_top, pad_left, pad_bottom, pad_right)."""
    ph = max((output_rows - 1) * row_stride + kernel_rows - input_rows, 0)
    pw = max((output_cols - 1) * col_stride + kernel_cols - input_cols, 0)
    return ph // 2, pw // 2, ph - ph // 2, pw - pw // 2


def _pad_typ(padding) -> int:
    _verify(padding in (SAME, VALID), lambda: f"padding must be SAME or VALID, got {padding!r}")
    return 0 if padding == SAME else 1


# ---- stub name mapping -------------------------------------------------------

_KIND_OF: dict = {}  # element type -> kind name, filled as types are met


def _kind(a) -> str:
    """Owl's kind name of an array's element type: float32 / float64 (S, D)
    and complex32 / complex64 (C, Z), the latter numpy's / torch's complex64
    and complex128."""
    dtype = getattr(a, "dtype", None)
    k = _KIND_OF.get(dtype)
    if k is not None:
        return k
    dt = str(dtype if dtype is not None else "")
    for name, kind in (("float32", "float32"), ("float64", "float64"),
                       ("complex64", "complex32"), ("complex128", "complex64")):
        if name in dt:
            _KIND_OF[dtype] = kind
            return kind
    raise InvalidArgument(f"unsupported element kind {dt} (float32, float64, complex64 and "
                          "complex128 only)")


class Backend:
    """Stub provider.  `stub(kind, op, *args)` runs the C stub
    `<kind>_ndarray_<op>` with Owl's argument order; `empty(like, shape,
    dtype)` allocates an uninitialised array where `like` lives."""

    name = "abstract"

    def empty(self, like, shape, dtype=None):
        raise NotImplementedError

    def stub(self, kind: str, op: str, *args) -> None:
        raise NotImplementedError

    def shape(self, a) -> tuple:
        return tuple(a.shape)

    def reshape(self, a, shape):
        return a.reshape(shape)


class GpuBackend(Backend):
    """The product path: libowlgpu through its C ABI.  numpy arrays go to
    the host drop-in entry points (`owl_*`), torch CUDA tensors to the
    device-resident ones (`owlgpu_*`) on torch's current stream."""

    name = "gpu"

    def __init__(self, precision: str | int = "fp32"):
        from . import _lib

        self._lib = _lib
        self.precision = _lib.PREC[precision] if isinstance(precision, str) else int(precision)

    @staticmethod
    def _is_torch(a) -> bool:
        return type(a).__module__.startswith("torch")

    def empty(self, like, shape, dtype=None):
        if self._is_torch(like):
            import torch

            return torch.empty(tuple(shape), dtype=dtype or like.dtype, device=like.device)
        return np.empty(tuple(shape), dtype=dtype or like.dtype)

    def stub(self, kind, op, *args):
        conv = []
        dev = host = False
        for a in args:
            if isinstance(a, (int, np.integer)):
                conv.append(int(a))
            elif self._is_torch(a):
                if not a.is_cuda or not a.is_contiguous():
                    raise InvalidArgument("device arrays must be contiguous CUDA tensors")
                conv.append(a.data_ptr())
                dev = True
            else:
                if not (isinstance(a, np.ndarray) and a.flags.c_contiguous):
                    raise InvalidArgument("host arrays must be C-contiguous numpy arrays")
                conv.append(a.ctypes.data)
                host = True
        if dev and host:
            raise InvalidArgument("a call takes either CUDA tensors or numpy arrays, not both")
        if dev:
            import torch

            stream = torch.cuda.current_stream().cuda_stream
            self._lib.call(f"owlgpu_{kind}_ndarray_{op}", *conv, self.precision, stream)
        else:
            prev = self._lib.set_precision(self.precision)
            try:
                self._lib.call(f"owl_{kind}_ndarray_{op}", *conv)
            finally:
                if prev != self.precision:
                    self._lib.set_precision(prev)


# ---- the NN function set (G) -------------------------------------------------

class NN:
    """Owl's conv/pool ndarray functions over one stub provider."""

    def __init__(self, backend: Backend):
        self.b = backend

    # -- helpers
    def _shape(self, a):
        return self.b.shape(a)

    def _dims(self, a):
        return len(self._shape(a))

    def _out(self, out, like, shape, dtype=None):
        """The `~out` argument of Owl's `_` variants (e.g. `conv2d_ ~out`,
        G:2402): write into `out` when given (its shape must be the result's),
        else allocate where `like` lives."""
        if out is None:
            return self.b.empty(like, shape, dtype)
        _verify(tuple(self._shape(out)) == tuple(shape),
                lambda: f"out: shape {list(self._shape(out))} should be {list(shape)}")
        return out

    def _ob(self, out):
        """A 1-D result [B;W;C] seen as the 2-D [B;1;W;C] it is computed as."""
        if out is None:
            return None
        sh = tuple(self._shape(out))
        return self.b.reshape(out, (sh[0], 1) + sh[1:])

    def _ok(self, out):
        """A 1-D kernel [K;Ci;Co] seen as the 2-D [1;K;Ci;Co]."""
        return None if out is None else self.b.reshape(out, (1,) + tuple(self._shape(out)))

    # ======================= conv2d (G:2324-2850) =======================

    def conv2d(self, input, kernel, stride: Sequence[int], padding=SAME, out=None):
        """G:2324 conv2d."""
        _verify(self._dims(input) == 4 and self._dims(kernel) == 4 and len(stride) == 2,
                lambda: f"conv2d: input dimension = {self._dims(input)} (should be 4); kernel "
                f"dimension = {self._dims(kernel)} (should be 4); stride dimension = "
                f"{len(stride)} (should be 2).")
        B, IC, IR, Ci = self._shape(input)
        KC, KR, kci, Co = self._shape(kernel)
        _verify(Ci == kci, lambda: f"conv2d: input shape is {list(self._shape(input))}, kernel "
                f"shape is {list(self._shape(kernel))}, the 4th dimension of input shape should "
                f"be equal to the 3rd dimension of kernel shape.")
        cs, rs = stride
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        output = self._out(out, input, (B, OC, OR, Co))
        self.b.stub(_kind(input), "conv_spatial", input, kernel, output, B, IC, IR, Ci, KC, KR,
                    OC, OR, Co, rs, cs, _pad_typ(padding), 1, 1)
        return output

    def _conv2d_bwd_check(self, name, input, kernel, stride, output_):
        _verify(self._dims(input) == 4 and self._dims(kernel) == 4 and
                self._dims(output_) == 4 and len(stride) == 2, lambda: f"{name}: bad dimensions")
        B, IC, IR, Ci = self._shape(input)
        KC, KR, kci, Co = self._shape(kernel)
        _verify(Ci == kci, lambda: f"{name}: the 4th dimension of input shape should be equal to "
                f"the 3rd dimension of kernel shape")
        ob, OC, OR, oco = self._shape(output_)
        _verify(B == ob and Co == oco,
                lambda: f"{name}: output' shape {list(self._shape(output_))} does not match "
                f"input/kernel")
        return B, IC, IR, Ci, KC, KR, Co, OC, OR

    def conv2d_backward_input(self, input, kernel, stride, output_, out=None):
        """G:2479 conv2d_backward_input."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "conv2d_backward_input", input, kernel, stride, output_)
        cs, rs = stride
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_spatial_backward_input", input_, kernel, output_, B, IC,
                    IR, Ci, KC, KR, OC, OR, Co, rs, cs, 1, 1)
        return input_

    def conv2d_backward_kernel(self, input, kernel, stride, output_, out=None):
        """G:2660 conv2d_backward_kernel."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "conv2d_backward_kernel", input, kernel, stride, output_)
        cs, rs = stride
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_spatial_backward_kernel", input, kernel_, output_, B,
                    IC, IR, Ci, KC, KR, OC, OR, Co, rs, cs, 1, 1)
        return kernel_

    # ======================= conv1d (G:3402) =======================

    def conv1d(self, input, kernel, stride, padding=SAME, out=None):
        """G:3402 conv1d: reshape to conv2d [B;1;W;C] with stride [1;s]."""
        _verify(self._dims(input) == 3 and self._dims(kernel) == 3 and len(stride) == 1,
                "conv1d: bad dimensions")
        B, IC, Ci = self._shape(input)
        KC, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "conv1d: channel mismatch")
        x = self.b.reshape(input, (B, 1, IC, Ci))
        w = self.b.reshape(kernel, (1, KC, Ci, Co))
        y = self.conv2d(x, w, [1, stride[0]], padding, out=self._ob(out))
        return self.b.reshape(y, (B, self._shape(y)[2], Co))

    def conv1d_backward_input(self, input, kernel, stride, output_, out=None):
        B, IC, Ci = self._shape(input)
        KC, _, Co = self._shape(kernel)
        OC = self._shape(output_)[1]
        dx = self.conv2d_backward_input(self.b.reshape(input, (B, 1, IC, Ci)),
                                        self.b.reshape(kernel, (1, KC, Ci, Co)),
                                        [1, stride[0]], self.b.reshape(output_, (B, 1, OC, Co)),
                                        out=self._ob(out))
        return self.b.reshape(dx, (B, IC, Ci))

    def conv1d_backward_kernel(self, input, kernel, stride, output_, out=None):
        B, IC, Ci = self._shape(input)
        KC, _, Co = self._shape(kernel)
        OC = self._shape(output_)[1]
        dw = self.conv2d_backward_kernel(self.b.reshape(input, (B, 1, IC, Ci)),
                                         self.b.reshape(kernel, (1, KC, Ci, Co)),
                                         [1, stride[0]], self.b.reshape(output_, (B, 1, OC, Co)),
                                         out=self._ok(out))
        return self.b.reshape(dw, (KC, Ci, Co))

    # ======================= conv3d (G:2848-3400) =======================

    def conv3d(self, input, kernel, stride, padding=SAME, out=None):
        """G:2848 conv3d."""
        _verify(self._dims(input) == 5 and self._dims(kernel) == 5 and len(stride) == 3,
                "conv3d: bad dimensions")
        B, IC, IR, ID, Ci = self._shape(input)
        KC, KR, KD, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "conv3d: the 5th dimension of input shape should be equal to the "
                "4th dimension of kernel shape")
        cs, rs, ds = stride
        OC, OR, OD = calc_conv3d_output_shape(padding, IC, IR, ID, KC, KR, KD, rs, cs, ds)
        output = self._out(out, input, (B, OC, OR, OD, Co))
        self.b.stub(_kind(input), "conv_cuboid_im2col", input, kernel, output, B, IC, IR, ID, Ci,
                    KC, KR, KD, OC, OR, OD, Co, ds, rs, cs, _pad_typ(padding))
        return output

    def _conv3d_bwd_check(self, name, input, kernel, stride, output_):
        _verify(self._dims(input) == 5 and self._dims(kernel) == 5 and
                self._dims(output_) == 5 and len(stride) == 3, lambda: f"{name}: bad dimensions")
        B, IC, IR, ID, Ci = self._shape(input)
        KC, KR, KD, kci, Co = self._shape(kernel)
        _verify(Ci == kci, lambda: f"{name}: channel mismatch")
        ob, OC, OR, OD, oco = self._shape(output_)
        _verify(B == ob and Co == oco, lambda: f"{name}: output' shape mismatch")
        return B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD

    def conv3d_backward_input(self, input, kernel, stride, output_, out=None):
        """G:3017 conv3d_backward_input."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "conv3d_backward_input", input, kernel, stride, output_)
        cs, rs, ds = stride
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_cuboid_backward_input_im2col", input_, kernel, output_,
                    B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, ds, rs, cs)
        return input_

    def conv3d_backward_kernel(self, input, kernel, stride, output_, out=None):
        """G:3206 conv3d_backward_kernel."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "conv3d_backward_kernel", input, kernel, stride, output_)
        cs, rs, ds = stride
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_cuboid_backward_kernel_im2col", input, kernel_, output_,
                    B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, ds, rs, cs)
        return kernel_

    # ======================= dilated (G:3797-4900) =======================

    def dilated_conv2d(self, input, kernel, stride, rate, padding=SAME, out=None):
        """G:3797 dilated_conv2d: output shape from the dilated kernel extent."""
        _verify(self._dims(input) == 4 and self._dims(kernel) == 4 and len(stride) == 2 and
                len(rate) == 2, "dilated_conv2d: bad dimensions")
        B, IC, IR, Ci = self._shape(input)
        KC, KR, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "dilated_conv2d: channel mismatch")
        cs, rs = stride
        cr, rr = rate
        kcu, kru = KC + (KC - 1) * (cr - 1), KR + (KR - 1) * (rr - 1)
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, kcu, kru, rs, cs)
        output = self._out(out, input, (B, OC, OR, Co))
        self.b.stub(_kind(input), "conv_dilated_spatial_im2col", input, kernel, output, B, IC,
                    IR, Ci, KC, KR, OC, OR, Co, rs, cs, _pad_typ(padding), rr, cr)
        return output

    def dilated_conv2d_backward_input(self, input, kernel, stride, rate, output_, out=None):
        """G:3960."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "dilated_conv2d_backward_input", input, kernel, stride, output_)
        cs, rs = stride
        cr, rr = rate
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_dilated_spatial_backward_input_im2col", input_, kernel,
                    output_, B, IC, IR, Ci, KC, KR, OC, OR, Co, rs, cs, rr, cr)
        return input_

    def dilated_conv2d_backward_kernel(self, input, kernel, stride, rate, output_, out=None):
        """G:4151."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "dilated_conv2d_backward_kernel", input, kernel, stride, output_)
        cs, rs = stride
        cr, rr = rate
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_dilated_spatial_backward_kernel_im2col", input, kernel_,
                    output_, B, IC, IR, Ci, KC, KR, OC, OR, Co, rs, cs, rr, cr)
        return kernel_

    def dilated_conv3d(self, input, kernel, stride, rate, padding=SAME, out=None):
        """G:4348 dilated_conv3d."""
        _verify(self._dims(input) == 5 and self._dims(kernel) == 5 and len(stride) == 3 and
                len(rate) == 3, "dilated_conv3d: bad dimensions")
        B, IC, IR, ID, Ci = self._shape(input)
        KC, KR, KD, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "dilated_conv3d: channel mismatch")
        cs, rs, ds = stride
        cr, rr, dr = rate
        kcu = KC + (KC - 1) * (cr - 1)
        kru = KR + (KR - 1) * (rr - 1)
        kdu = KD + (KD - 1) * (dr - 1)
        OC, OR, OD = calc_conv3d_output_shape(padding, IC, IR, ID, kcu, kru, kdu, rs, cs, ds)
        output = self._out(out, input, (B, OC, OR, OD, Co))
        self.b.stub(_kind(input), "conv_dilated_cuboid_im2col", input, kernel, output, B, IC, IR,
                    ID, Ci, KC, KR, KD, OC, OR, OD, Co, ds, rs, cs, dr, rr, cr,
                    _pad_typ(padding))
        return output

    def dilated_conv3d_backward_input(self, input, kernel, stride, rate, output_, out=None):
        """G:4539."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "dilated_conv3d_backward_input", input, kernel, stride, output_)
        cs, rs, ds = stride
        cr, rr, dr = rate
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_dilated_cuboid_backward_input_im2col", input_, kernel,
                    output_, B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, ds, rs, cs, dr, rr, cr)
        return input_

    def dilated_conv3d_backward_kernel(self, input, kernel, stride, rate, output_, out=None):
        """G:4750."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "dilated_conv3d_backward_kernel", input, kernel, stride, output_)
        cs, rs, ds = stride
        cr, rr, dr = rate
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_dilated_cuboid_backward_kernel_im2col", input, kernel_,
                    output_, B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, ds, rs, cs, dr, rr, cr)
        return kernel_

    # ======================= transpose (G:5371-6480) =======================
    # Owl implements transposed convolution with the backward stubs and swapped
    # roles; the kernel buffer [KC;KR;Cin;Cout] is then read as
    # [KC][KR][Cout][Cin] (a reinterpretation, not a transpose), G:5422-5439.

    def transpose_conv2d(self, input, kernel, stride, padding=SAME, out=None):
        """G:5371 transpose_conv2d."""
        _verify(self._dims(input) == 4 and self._dims(kernel) == 4 and len(stride) == 2,
                "transpose_conv2d: bad dimensions")
        B, IC, IR, Ci = self._shape(input)
        KC, KR, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "transpose_conv2d: channel mismatch")
        cs, rs = stride
        OC, OR = calc_transpose_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        output = self._out(out, input, (B, OC, OR, Co))
        self.b.stub(_kind(input), "conv_spatial_backward_input", output, kernel, input, B, OC, OR,
                    Co, KC, KR, IC, IR, Ci, rs, cs, 1, 1)
        return output

    def transpose_conv2d_backward_input(self, input, kernel, stride, output_, out=None):
        """G:5713: a forward conv of output' with the SAME padding rule."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "transpose_conv2d_backward_input", input, kernel, stride, output_)
        cs, rs = stride
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_spatial", output_, kernel, input_, B, OC, OR, Co, KC, KR,
                    IC, IR, Ci, rs, cs, 0, 1, 1)
        return input_

    def transpose_conv2d_backward_kernel(self, input, kernel, stride, output_, out=None):
        """G:5514."""
        B, IC, IR, Ci, KC, KR, Co, OC, OR = self._conv2d_bwd_check(
            "transpose_conv2d_backward_kernel", input, kernel, stride, output_)
        cs, rs = stride
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_spatial_backward_kernel", output_, kernel_, input, B, OC,
                    OR, Co, KC, KR, IC, IR, Ci, rs, cs, 1, 1)
        return kernel_

    def transpose_conv1d(self, input, kernel, stride, padding=SAME, out=None):
        B, IC, Ci = self._shape(input)
        KC, _, Co = self._shape(kernel)
        y = self.transpose_conv2d(self.b.reshape(input, (B, 1, IC, Ci)),
                                  self.b.reshape(kernel, (1, KC, Ci, Co)), [1, stride[0]],
                                  padding, out=self._ob(out))
        return self.b.reshape(y, (B, self._shape(y)[2], Co))

    def _as2d(self, input, kernel, output_):
        """The [B;1;W;C] / [1;K;Ci;Co] views through which Owl runs 1-D
        convolutions as 2-D ones (G:3402-3440)."""
        _verify(self._dims(input) == 3 and self._dims(kernel) == 3 and
                (output_ is None or self._dims(output_) == 3), "1-D conv: bad dimensions")
        B, IC, Ci = self._shape(input)
        KC, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "1-D conv: the 3rd dimension of input shape should be equal to "
                "the 2nd dimension of kernel shape")
        x = self.b.reshape(input, (B, 1, IC, Ci))
        w = self.b.reshape(kernel, (1, KC, Ci, Co))
        dy = None
        if output_ is not None:
            ob, OC, oco = self._shape(output_)
            dy = self.b.reshape(output_, (ob, 1, OC, oco))
        return x, w, dy

    def transpose_conv1d_backward_input(self, input, kernel, stride, output_, out=None):
        """G:6570 transpose_conv1d_backward_input."""
        x, w, dy = self._as2d(input, kernel, output_)
        dx = self.transpose_conv2d_backward_input(x, w, [1, stride[0]], dy, out=self._ob(out))
        return self.b.reshape(dx, self._shape(input))

    def transpose_conv1d_backward_kernel(self, input, kernel, stride, output_, out=None):
        """G:6732 transpose_conv1d_backward_kernel."""
        x, w, dy = self._as2d(input, kernel, output_)
        dw = self.transpose_conv2d_backward_kernel(x, w, [1, stride[0]], dy, out=self._ok(out))
        return self.b.reshape(dw, self._shape(kernel))

    def dilated_conv1d(self, input, kernel, stride, rate, padding=SAME, out=None):
        """G:4967 dilated_conv1d: the 2-D view with stride [1; s]; `rate` is
        handed to dilated_conv2d unchanged, as Owl does (two entries)."""
        _verify(len(stride) == 1, "dilated_conv1d: stride dimension should be 1")
        x, w, _ = self._as2d(input, kernel, None)
        y = self.dilated_conv2d(x, w, [1, stride[0]], list(rate), padding, out=self._ob(out))
        B, _, OC, Co = self._shape(y)
        return self.b.reshape(y, (B, OC, Co))

    def dilated_conv1d_backward_input(self, input, kernel, stride, rate, output_, out=None):
        """G:5054 dilated_conv1d_backward_input."""
        x, w, dy = self._as2d(input, kernel, output_)
        dx = self.dilated_conv2d_backward_input(x, w, [1, stride[0]], list(rate), dy,
                                                out=self._ob(out))
        return self.b.reshape(dx, self._shape(input))

    def dilated_conv1d_backward_kernel(self, input, kernel, stride, rate, output_, out=None):
        """G:5210 dilated_conv1d_backward_kernel."""
        x, w, dy = self._as2d(input, kernel, output_)
        dw = self.dilated_conv2d_backward_kernel(x, w, [1, stride[0]], list(rate), dy,
                                                 out=self._ok(out))
        return self.b.reshape(dw, self._shape(kernel))

    def transpose_conv3d(self, input, kernel, stride, padding=SAME, out=None):
        """G:5915 transpose_conv3d."""
        _verify(self._dims(input) == 5 and self._dims(kernel) == 5 and len(stride) == 3,
                "transpose_conv3d: bad dimensions")
        B, IC, IR, ID, Ci = self._shape(input)
        KC, KR, KD, kci, Co = self._shape(kernel)
        _verify(Ci == kci, "transpose_conv3d: channel mismatch")
        cs, rs, ds = stride
        OC, OR, OD = calc_transpose_conv3d_output_shape(padding, IC, IR, ID, KC, KR, KD, rs, cs,
                                                        ds)
        output = self._out(out, input, (B, OC, OR, OD, Co))
        self.b.stub(_kind(input), "conv_cuboid_backward_input_im2col", output, kernel, input, B,
                    OC, OR, OD, Co, KC, KR, KD, IC, IR, ID, Ci, ds, rs, cs)
        return output

    def transpose_conv3d_backward_input(self, input, kernel, stride, output_, out=None):
        """G:6072."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "transpose_conv3d_backward_input", input, kernel, stride, output_)
        cs, rs, ds = stride
        input_ = self._out(out, input, self._shape(input))
        self.b.stub(_kind(input), "conv_cuboid_im2col", output_, kernel, input_, B, OC, OR, OD,
                    Co, KC, KR, KD, IC, IR, ID, Ci, ds, rs, cs, 0)
        return input_

    def transpose_conv3d_backward_kernel(self, input, kernel, stride, output_, out=None):
        """G:6277."""
        B, IC, IR, ID, Ci, KC, KR, KD, Co, OC, OR, OD = self._conv3d_bwd_check(
            "transpose_conv3d_backward_kernel", input, kernel, stride, output_)
        cs, rs, ds = stride
        kernel_ = self._out(out, kernel, self._shape(kernel))
        self.b.stub(_kind(input), "conv_cuboid_backward_kernel_im2col", output_, kernel_, input,
                    B, OC, OR, OD, Co, KC, KR, KD, IC, IR, ID, Ci, ds, rs, cs)
        return kernel_

    # ======================= pooling (G:6905-8200) =======================

    def _pool2d(self, which, padding, input, kernel, stride, out=None):
        _verify(self._dims(input) == 4 and len(kernel) == 2 and len(stride) == 2,
                lambda: f"{which}_pool2d: bad dimensions")
        B, IC, IR, C = self._shape(input)
        KC, KR = kernel
        cs, rs = stride
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        output = self._out(out, input, (B, OC, OR, C))
        self.b.stub(_kind(input), f"{which}pool_spatial", input, output, B, IC, IR, C, KC, KR, OC,
                    OR, rs, cs, _pad_typ(padding), 1, 1)
        return output

    def max_pool2d(self, input, kernel, stride, padding=SAME, out=None):
        """G:6905 max_pool2d ?padding input kernel stride."""
        return self._pool2d("max", padding, input, kernel, stride, out)

    def avg_pool2d(self, input, kernel, stride, padding=SAME, out=None):
        """G:7080 avg_pool2d."""
        return self._pool2d("avg", padding, input, kernel, stride, out)

    def max_pool2d_argmax(self, input, kernel, stride, padding=SAME, out=None, out_argmax=None):
        """G:7517 max_pool2d_argmax: (values, int64 flat indices)."""
        _verify(self._dims(input) == 4 and len(kernel) == 2 and len(stride) == 2,
                "max_pool2d_argmax: bad dimensions")
        B, IC, IR, C = self._shape(input)
        KC, KR = kernel
        cs, rs = stride
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        pt, pl, _, _ = calc_conv2d_padding(IC, IR, KC, KR, OC, OR, rs, cs)
        output = self._out(out, input, (B, OC, OR, C))
        argmax = self._out(out_argmax, input, (B, OC, OR, C), _int64_like(input))
        self.b.stub(_kind(input), "maxpool_argmax_spatial", input, output, argmax, B, IC, IR, C,
                    KC, KR, OC, OR, rs, cs, pt, pl)
        return output, argmax

    def _pool2d_backward(self, which, padding, input, kernel, stride, output_, out=None):
        _verify(self._dims(input) == 4 and len(kernel) == 2 and len(stride) == 2,
                lambda: f"{which}_pool2d_backward: bad dimensions")
        B, IC, IR, C = self._shape(input)
        KC, KR = kernel
        cs, rs = stride
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        pt, pl, _, _ = calc_conv2d_padding(IC, IR, KC, KR, OC, OR, rs, cs)
        input_ = self._out(out, input, self._shape(input))
        # avg: Owl's OCaml wrapper passes input' as the dummy first argument
        # (owl_ndarray_pool.ml:85-118); the stub never reads it.
        first = input if which == "max" else input_
        self.b.stub(_kind(input), f"{which}pool_spatial_backward", first, output_, input_, B, IC,
                    IR, C, KC, KR, OC, OR, rs, cs, pt, pl)
        return input_

    def max_pool2d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:7715 max_pool2d_backward padding input kernel stride output'."""
        return self._pool2d_backward("max", padding, input, kernel, stride, output_, out)

    def avg_pool2d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:8035 avg_pool2d_backward."""
        return self._pool2d_backward("avg", padding, input, kernel, stride, output_, out)

    def _pool3d(self, which, padding, input, kernel, stride, out=None):
        _verify(self._dims(input) == 5 and len(kernel) == 3 and len(stride) == 3,
                lambda: f"{which}_pool3d: bad dimensions")
        B, IC, IR, ID, C = self._shape(input)
        KC, KR, KD = kernel
        cs, rs, ds = stride
        OC, OR, OD = calc_conv3d_output_shape(padding, IC, IR, ID, KC, KR, KD, rs, cs, ds)
        output = self._out(out, input, (B, OC, OR, OD, C))
        self.b.stub(_kind(input), f"{which}pool_cuboid", input, output, B, IC, IR, ID, C, KC, KR,
                    KD, OC, OR, OD, ds, rs, cs, _pad_typ(padding))
        return output

    def max_pool3d(self, input, kernel, stride, padding=SAME, out=None):
        """G:7255 max_pool3d."""
        return self._pool3d("max", padding, input, kernel, stride, out)

    def avg_pool3d(self, input, kernel, stride, padding=SAME, out=None):
        """G:7386 avg_pool3d."""
        return self._pool3d("avg", padding, input, kernel, stride, out)

    def _pool3d_backward(self, which, padding, input, kernel, stride, output_, out=None):
        _verify(self._dims(input) == 5 and len(kernel) == 3 and len(stride) == 3,
                lambda: f"{which}_pool3d_backward: bad dimensions")
        B, IC, IR, ID, C = self._shape(input)
        KC, KR, KD = kernel
        cs, rs, ds = stride
        OC, OR, OD = calc_conv3d_output_shape(padding, IC, IR, ID, KC, KR, KD, rs, cs, ds)
        input_ = self._out(out, input, self._shape(input))
        first = input if which == "max" else input_
        # Stride order col, row, dpt (G:7627-7647, owl_ndarray_pool_impl.h:324-331).
        self.b.stub(_kind(input), f"{which}pool_cuboid_backward", first, output_, input_, B, IC,
                    IR, ID, C, KC, KR, KD, OC, OR, OD, cs, rs, ds, _pad_typ(padding))
        return input_

    def max_pool3d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:7584 max_pool3d_backward."""
        return self._pool3d_backward("max", padding, input, kernel, stride, output_, out)

    def avg_pool3d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:7906 avg_pool3d_backward."""
        return self._pool3d_backward("avg", padding, input, kernel, stride, output_, out)

    def max_pool1d(self, input, kernel, stride, padding=SAME, out=None):
        B, IC, C = self._shape(input)
        y = self.max_pool2d(self.b.reshape(input, (B, 1, IC, C)), [1, kernel[0]],
                            [1, stride[0]], padding, out=self._ob(out))
        return self.b.reshape(y, (B, self._shape(y)[2], C))

    def avg_pool1d(self, input, kernel, stride, padding=SAME, out=None):
        B, IC, C = self._shape(input)
        y = self.avg_pool2d(self.b.reshape(input, (B, 1, IC, C)), [1, kernel[0]],
                            [1, stride[0]], padding, out=self._ob(out))
        return self.b.reshape(y, (B, self._shape(y)[2], C))

    def _pool1d_backward(self, which, padding, input, kernel, stride, output_, out=None):
        _verify(self._dims(input) == 3 and len(kernel) == 1 and len(stride) == 1,
                lambda: f"{which}_pool1d_backward: bad dimensions")
        B, IC, C = self._shape(input)
        ob, OC, oc = self._shape(output_)
        dx = self._pool2d_backward(which, padding, self.b.reshape(input, (B, 1, IC, C)),
                                   [1, kernel[0]], [1, stride[0]],
                                   self.b.reshape(output_, (ob, 1, OC, oc)), self._ob(out))
        return self.b.reshape(dx, (B, IC, C))

    def max_pool1d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:7840 max_pool1d_backward (the 2-D view [B;1;W;C], window [1;k])."""
        return self._pool1d_backward("max", padding, input, kernel, stride, output_, out)

    def avg_pool1d_backward(self, padding, input, kernel, stride, output_, out=None):
        """G:8158 avg_pool1d_backward."""
        return self._pool1d_backward("avg", padding, input, kernel, stride, output_, out)

    # ======================= upsampling2d (G:8223-8330) =======================

    def upsampling2d(self, input, size, out=None):
        """G:8223 upsampling2d: `repeat input [|1; size0; size1; 1|]`."""
        _verify(self._dims(input) == 4 and len(size) == 2,
                lambda: f"upsampling2d: input dimension = {self._dims(input)} (should be 4); "
                f"size dimension = {len(size)} (should be 2).")
        B, IC, IR, C = self._shape(input)
        cs, rs = size
        output = self._out(out, input, (B, IC * cs, IR * rs, C))
        self.b.stub(_kind(input), "upsampling_spatial", input, output, B, IC, IR, C, IC * cs,
                    IR * rs, cs, rs)
        return output

    def upsampling2d_backward(self, input, size, output, out=None):
        """G:8249 upsampling2d_backward input size output: the gradient for
        `input` from the output gradient `output`."""
        _verify(self._dims(input) == 4 and len(size) == 2,
                lambda: f"upsampling2d_backward: input dimension = {self._dims(input)} (should be "
                f"4); size dimension = {len(size)} (should be 2).")
        B, IC, IR, C = self._shape(input)
        cs, rs = size
        osh = self._shape(output)
        OC, OR = IC * cs, IR * rs
        _verify(len(osh) == 4 and OC == osh[1] and OR == osh[2],
                lambda: f"upsampling2d_backward: output shape is {list(osh)}; scaled output cols "
                f"is {OC}, should be equal to the 2nd dimension of output shape; scaled output "
                f"rows is {OR}, should be equal to the 3rd dimension of output shape.")
        input_ = self._out(out, input, (B, IC, IR, C))
        self.b.stub(_kind(input), "upsampling_spatial_backward", input_, output, B, IC, IR, C,
                    OC, OR, cs, rs)
        return input_

def _int64_like(a) -> Any:
    if type(a).__module__.startswith("torch"):
        import torch

        return torch.int64
    return np.int64
