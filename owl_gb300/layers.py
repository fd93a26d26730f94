"""The layers around the convolutions of a training or serving step, on the
device in libowlgpu's own kernels.

Owl builds its networks from neurons (src/base/neural/owl_neural_neuron.ml):
``Conv2D.run`` computes ``conv2d x w s + b`` (:1253) and an ``Activation``
neuron follows; ``FullyConnected.run`` computes ``(x *@ w) + b`` (:1907);
the classifier's loss is ``Cross_entropy`` of a softmax over the batch
(owl_optimise_generic.ml:172, :646-649) and the optimiser moves each weight
by ``-rate * gradient``.  These are OCaml compositions of ndarray operations
in Owl, with no C stub of their own; the library exports them as extension
entry points (include/owlgpu.h, "Extensions") so that a step stays in its
kernels:

* ``conv2d_bias_act``: the convolution with bias and ReLU applied in the
  tensor-core epilogue;
* ``bias_act_backward``: the ReLU mask and the bias gradient in one pass;
* ``dot``: the dense layer's product on a tcgen05 GEMM (split-K, fixed-order
  sum), in all three orientations its forward and backward need;
* ``softmax_cross_entropy``: the batch-mean loss and its gradient;
* ``sgd_update``: ``w -= lr * g``.

With the GPU backend every call takes contiguous CUDA tensors and runs on
torch's current stream.  Over any other stub provider (the CPU oracle in the
tests) the same functions are computed by composing that provider's
convolutions with numpy, as Owl composes its ndarray operations.
"""

from __future__ import annotations

import numpy as np

from .dense import NN, GpuBackend, InvalidArgument

ACT_NONE = 0
ACT_RELU = 1


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _kind(a) -> str:
    dt = str(a.dtype)
    if "float32" in dt:
        return "float32"
    if "float64" in dt:
        return "float64"
    raise InvalidArgument(f"{dt}: the layer kernels take float32 or float64 arrays")


class Layers:
    """The layer functions over one stub provider (``nn.b``)."""

    def __init__(self, nn: NN):
        self.nn = nn
        self.gpu = isinstance(nn.b, GpuBackend)
        if self.gpu:
            from . import _lib

            self._lib = _lib
            self.precision = nn.b.precision

    # -- plumbing
    def _dev(self, *arrays) -> bool:
        """True when the GPU kernels run: GPU backend and CUDA tensors."""
        if not self.gpu:
            return False
        for a in arrays:
            if a is None:
                continue
            if not (_is_torch(a) and a.is_cuda and a.is_contiguous()):
                raise InvalidArgument("the layer kernels take contiguous CUDA tensors")
        return True

    @staticmethod
    def _p(a) -> int | None:
        return None if a is None else a.data_ptr()

    @staticmethod
    def _stream():
        import torch

        return torch.cuda.current_stream().cuda_stream

    def _empty(self, like, shape):
        import torch

        return torch.empty(tuple(shape), dtype=like.dtype, device=like.device)

    # -- convolution + bias + activation
    def conv2d_bias_act(self, x, w, b, stride, padding="SAME", act=ACT_RELU):
        """act(conv2d x w stride + b): Owl's Conv2D neuron and the Activation
        after it (owl_neural_neuron.ml:1253)."""
        if not self._dev(x, w, b):
            y = self.nn.conv2d(x, w, stride, padding)
            if b is not None:
                y = y + b
            return np.maximum(y, 0) if act == ACT_RELU else y
        from .dense import _pad_typ, calc_conv2d_output_shape

        B, IC, IR, Ci = x.shape
        KC, KR, kci, Co = w.shape
        if Ci != kci or len(stride) != 2:
            raise InvalidArgument("conv2d_bias_act: bad shapes")
        cs, rs = stride
        OC, OR = calc_conv2d_output_shape(padding, IC, IR, KC, KR, rs, cs)
        y = self._empty(x, (B, OC, OR, Co))
        self._lib.call(f"owlgpu_{_kind(x)}_ndarray_conv_spatial_bias_act", x.data_ptr(),
                       w.data_ptr(), y.data_ptr(), B, IC, IR, Ci, KC, KR, OC, OR, Co, rs, cs,
                       _pad_typ(padding), 1, 1, self._p(b), act, self.precision, self._stream())
        return y

    def bias_act_backward(self, y, dy, act=ACT_RELU, bias_grad=True):
        """(adjoint before the activation, adjoint of the bias) from the
        layer's output `y` and its adjoint `dy` ([..., channels])."""
        C = y.shape[-1]
        if not self._dev(y, dy):
            dz = dy * (y > 0) if act == ACT_RELU else dy
            db = dz.reshape(-1, C).sum(axis=0) if bias_grad else None
            return dz, db
        dz = self._empty(dy, dy.shape)
        db = self._empty(dy, (C,)) if bias_grad else None
        self._lib.call(f"owlgpu_{_kind(y)}_bias_act_backward", y.data_ptr(), dy.data_ptr(),
                       dz.data_ptr(), self._p(db), y.numel() // max(C, 1), C, act,
                       self._stream())
        return dz, db

    # -- dense layer
    def dot(self, a, b, trans_a=False, trans_b=False, bias=None, act=ACT_NONE):
        """act(op(a) @ op(b) + bias), row-major matrices."""
        if not self._dev(a, b, bias):
            aa = a.T if trans_a else a
            bb = b.T if trans_b else b
            c = aa @ bb
            if bias is not None:
                c = c + bias
            return np.maximum(c, 0) if act == ACT_RELU else c
        m = a.shape[1] if trans_a else a.shape[0]
        k = a.shape[0] if trans_a else a.shape[1]
        n = b.shape[0] if trans_b else b.shape[1]
        if (b.shape[1] if trans_b else b.shape[0]) != k:
            raise InvalidArgument("dot: inner dimensions differ")
        c = self._empty(a, (m, n))
        self._lib.call(f"owlgpu_{_kind(a)}_dot", a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n,
                       k, int(trans_a), int(trans_b), self._p(bias), act, self.precision,
                       self._stream())
        return c

    # -- loss
    def softmax_cross_entropy(self, logits, labels, dloss=None, want_loss=True,
                              want_grad=False):
        """(batch-mean cross-entropy of softmax(logits) against labels, and
        the logits' adjoint for a loss adjoint `dloss` (None = 1))."""
        n = logits.shape[0]
        if not self._dev(logits, labels, dloss):
            z = logits
            m = z.max(axis=1, keepdims=True)
            lsm = z - m - np.log(np.exp(z - m).sum(axis=1, keepdims=True))
            loss = -(labels * lsm).sum() / n if want_loss else None
            g = None
            if want_grad:
                g = (np.exp(lsm) - labels) * ((1.0 if dloss is None else dloss) / n)
            return loss, g
        loss = self._empty(logits, ()) if want_loss else None
        g = self._empty(logits, logits.shape) if want_grad else None
        self._lib.call(f"owlgpu_{_kind(logits)}_softmax_cross_entropy", logits.data_ptr(),
                       labels.data_ptr(), self._p(loss), self._p(g), self._p(dloss), n,
                       logits.shape[1], self._stream())
        return loss, g

    # -- optimiser
    def sgd_update(self, w, g, lr):
        """w -= lr * g in place."""
        if not self._dev(w, g):
            w -= lr * g
            return w
        self._lib.call(f"owlgpu_{_kind(w)}_sgd_update", w.data_ptr(), g.data_ptr(), w.numel(),
                       float(lr), self._stream())
        return w
