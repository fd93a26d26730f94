"""Reverse-mode Algodiff over the conv/pool stubs.

Owl differentiates its convolutions and poolings as custom operations
registered with two builders (src/base/algodiff/owl_algodiff_ops.ml:2260-2900,
builder signatures in owl_algodiff_ops_builder_sig.ml:16-112):

  * ``build_piso`` (pair in, single out) for every convolution: ``ff_bb``
    is the forward stub, ``dr_a`` / ``dr_b`` / ``dr_ab`` call the
    backward_input / backward_kernel stubs on the output adjoint;
  * ``build_siso`` (single in, single out) for every pooling: ``ff_arr`` is
    the forward stub, ``dr`` the pool backward stub (the max-pool mask is
    recomputed from the saved input, never stored); forward mode (``df``)
    fails, as in Owl.

This module keeps that structure: the same builders, the same op labels and
argument orders (``conv2d a b s ~padding``, ``max_pool2d padding a b s``),
over any stub provider of :mod:`owl_gb300.dense` -- the GPU library for the
product, the CPU oracle for the tests.  The tape is a plain reverse sweep
(Owl's ``reverse_prop``); a few Maths ops (add with bias broadcast, relu,
dot, reshape, softmax cross-entropy) make a small CNN trainable end to end.
Gradients of the weights come from the deterministic backward_kernel
kernels, so repeated steps give identical results.

A node's adjoint is handed to ``dr`` as a value (Owl passes a ``t ref``
and dereferences it with ``!ca``).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Callable, Sequence

import numpy as np

from .dense import NN as _NN
from .dense import SAME
from .layers import ACT_NONE, ACT_RELU, Layers

# ---- array helpers (numpy for the oracle, torch for the GPU) ----------------


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _relu(a):
    return a.clamp_min(0) if _is_torch(a) else np.maximum(a, 0)


def _relu_mask(a, g):
    return g * (a > 0)


def _sum_to(g, shape):
    """Sum a broadcast adjoint back to `shape` (trailing-aligned)."""
    shape = tuple(shape)
    if tuple(g.shape) == shape:
        return g
    lead = len(g.shape) - len(shape)
    axes = tuple(range(lead)) + tuple(
        i + lead for i, n in enumerate(shape) if n == 1 and g.shape[i + lead] != 1)
    if _is_torch(g):
        out = g.sum(dim=axes) if axes else g
    else:
        out = g.sum(axis=axes) if axes else g
    return out.reshape(shape)


def _log_softmax(z):
    if _is_torch(z):
        m = z.amax(dim=1, keepdim=True)
        s = (z - m).exp().sum(dim=1, keepdim=True).log()
    else:
        m = z.max(axis=1, keepdims=True)
        s = np.log(np.exp(z - m).sum(axis=1, keepdims=True))
    return z - m - s


def _exp(a):
    return a.exp() if _is_torch(a) else np.exp(a)


def _scalar(a) -> float:
    return float(a.item()) if hasattr(a, "item") else float(a)


# ---- the tape -----------------------------------------------------------------


class Node:
    """A value on the reverse tape: primal `p`, adjoint `adj`, and how to
    hand an adjoint back to its inputs (`parents`, `backprop`)."""

    __slots__ = ("p", "adj", "parents", "backprop", "label")

    def __init__(self, p, parents=(), backprop=None, label="var"):
        self.p = p
        self.adj = None
        self.parents = parents
        self.backprop = backprop
        self.label = label

    @property
    def shape(self):
        return tuple(self.p.shape)

    def __repr__(self):
        return f"Node({self.label}, shape={self.shape})"


def make_reverse(p, label="var") -> Node:
    """A differentiable variable (Owl's ``make_reverse``)."""
    return Node(p, (), None, label)


def primal(x):
    return x.p if isinstance(x, Node) else x


def adjval(x):
    return x.adj


def _tracked(x) -> bool:
    return isinstance(x, Node)


def reverse_prop(v, out: Node) -> None:
    """Propagate adjoint `v` of `out` to every tracked input (Owl's
    ``reverse_prop``): topological order, adjoints summed at fan-in."""
    order, seen, stack = [], set(), [(out, False)]
    while stack:
        n, done = stack.pop()
        if done:
            order.append(n)
            continue
        if id(n) in seen:
            continue
        seen.add(id(n))
        stack.append((n, True))
        for p in n.parents:
            if _tracked(p) and id(p) not in seen:
                stack.append((p, False))
    out.adj = v
    for n in reversed(order):
        if n.backprop is None or n.adj is None:
            continue
        grads = n.backprop(n.adj)
        for p, g in zip(n.parents, grads):
            if g is None or not _tracked(p):
                continue
            p.adj = g if p.adj is None else p.adj + g
        n.adj = None  # interior adjoints are not kept


def grad(f: Callable, x):
    """Gradient of a scalar function at `x` (Owl's ``grad``)."""
    xv = make_reverse(x)
    y = f(xv)
    reverse_prop(_ones_like(y.p), y)
    return xv.adj


def _ones_like(a):
    if _is_torch(a):
        import torch

        return torch.ones_like(a)
    return np.ones_like(a)


# ---- custom-op builders -----------------------------------------------------------


def build_siso(spec) -> Callable:
    """Single input, single output (owl_algodiff_ops_builder_sig.ml:15-27):
    `spec` has ``label``, ``ff_arr(a)``, ``df(cp, ap, at)`` and
    ``dr(a, cp, ca)`` returning the adjoint of ``a``."""

    def op(a):
        ap = primal(a)
        cp = spec.ff_arr(ap)
        if not _tracked(a):
            return cp
        node = Node(cp, (a,), None, spec.label)
        node.backprop = lambda ca: (spec.dr(ap, cp, ca),)
        return node

    op.__name__ = spec.label
    return op


def build_piso(spec) -> Callable:
    """Pair input, single output (owl_algodiff_ops_builder_sig.ml:75-112):
    ``ff_bb(a, b)`` computes the result; ``dr_ab`` / ``dr_a`` / ``dr_b``
    return the adjoints of whichever inputs are tracked."""

    def op(a, b):
        ap, bp = primal(a), primal(b)
        cp = spec.ff_bb(ap, bp)
        ta, tb = _tracked(a), _tracked(b)
        if not (ta or tb):
            return cp
        node = Node(cp, (a, b), None, spec.label)
        if ta and tb:
            node.backprop = lambda ca: spec.dr_ab(ap, bp, cp, ca)
        elif ta:
            node.backprop = lambda ca: (spec.dr_a(ap, bp, cp, ca), None)
        else:
            node.backprop = lambda ca: (None, spec.dr_b(ap, bp, cp, ca))
        return node

    op.__name__ = spec.label
    return op


@dataclass
class _Siso:
    label: str
    ff_arr: Callable
    dr: Callable

    def df(self, cp, ap, at):
        raise NotImplementedError(f"{self.label}:df")


@dataclass
class _Piso:
    label: str
    ff_bb: Callable
    dr_a: Callable
    dr_b: Callable

    def dr_ab(self, a, b, cp, ca):
        return self.dr_a(a, b, cp, ca), self.dr_b(a, b, cp, ca)

    def df_da(self, cp, ap, at, bp):
        raise NotImplementedError(f"{self.label}:df")


# ---- Maths ----------------------------------------------------------------------


class Maths:
    """The elementwise / linear-algebra ops a small CNN needs."""

    @staticmethod
    def add(a, b):
        ap, bp = primal(a), primal(b)
        cp = ap + bp
        if not (_tracked(a) or _tracked(b)):
            return cp
        sa, sb = tuple(ap.shape), tuple(bp.shape)
        return Node(cp, (a, b), lambda g: (_sum_to(g, sa), _sum_to(g, sb)), "add")

    @staticmethod
    def relu(a):
        ap = primal(a)
        cp = _relu(ap)
        if not _tracked(a):
            return cp
        return Node(cp, (a,), lambda g: (_relu_mask(ap, g),), "relu")

    @staticmethod
    def dot(a, b):
        ap, bp = primal(a), primal(b)
        cp = ap @ bp
        if not (_tracked(a) or _tracked(b)):
            return cp
        return Node(cp, (a, b), lambda g: (g @ bp.T, ap.T @ g), "dot")

    @staticmethod
    def reshape(a, shape):
        ap = primal(a)
        old = tuple(ap.shape)
        cp = ap.reshape(tuple(shape))
        if not _tracked(a):
            return cp
        return Node(cp, (a,), lambda g: (g.reshape(old),), "reshape")

    @staticmethod
    def softmax_cross_entropy(logits, onehot):
        """mean over the batch of -sum(onehot * log softmax(logits)); the
        adjoint of the logits is (softmax - onehot) / batch."""
        zp = primal(logits)
        lsm = _log_softmax(zp)
        n = zp.shape[0]
        loss = -(onehot * lsm).sum() / n
        if not _tracked(logits):
            return loss
        return Node(loss, (logits,), lambda g: ((_exp(lsm) - onehot) * (g / n),), "softmax_ce")


# ---- NN: the registered conv / pool ops -------------------------------------------


class _NNOps:
    """Owl's ``Algodiff.NN`` conv/pool functions bound to one stub provider
    (owl_algodiff_ops.ml:2260-2900), and the layers around them
    (:mod:`owl_gb300.layers`) as differentiable ops."""

    def __init__(self, g: _NN):
        self.g = g
        self.layers = Layers(g)

    # ---- layers (owl_neural_neuron.ml), each one tape node -------------------

    def conv2d_bias_act(self, a, w, b, s, padding=SAME, act=ACT_RELU):
        """act(conv2d a w s + b): Owl's Conv2D neuron (owl_neural_neuron.ml:1253)
        and the Activation after it, one fused forward.  Reverse: the ReLU
        mask and bias gradient in one pass, then the convolution's
        backward_input / backward_kernel on the masked adjoint."""
        L, g = self.layers, self.g
        ap, wp, bp = primal(a), primal(w), primal(b)
        cp = L.conv2d_bias_act(ap, wp, bp, s, padding, act)
        if not (_tracked(a) or _tracked(w) or _tracked(b)):
            return cp

        def back(ca):
            dz, db = L.bias_act_backward(cp, ca, act, bias_grad=_tracked(b))
            dx = g.conv2d_backward_input(ap, wp, s, dz) if _tracked(a) else None
            dw = g.conv2d_backward_kernel(ap, wp, s, dz) if _tracked(w) else None
            return dx, dw, db

        return Node(cp, (a, w, b), back, "conv2d_bias_act")

    def fully_connected(self, a, w, b, act=ACT_NONE):
        """act(a *@ w + b): Owl's FullyConnected neuron (owl_neural_neuron.ml:1907)
        with an optional ReLU, on the library's GEMM.  Reverse: dz = the
        activation-masked adjoint, da = dz w^T, dw = a^T dz, db = sum of dz."""
        L = self.layers
        ap, wp, bp = primal(a), primal(w), primal(b)
        cp = L.dot(ap, wp, bias=bp, act=act)
        if not (_tracked(a) or _tracked(w) or _tracked(b)):
            return cp

        def back(ca):
            if act == ACT_NONE and not _tracked(b):
                dz, db = ca, None
            else:
                dz, db = L.bias_act_backward(cp, ca, act, bias_grad=_tracked(b))
            da = L.dot(dz, wp, trans_b=True) if _tracked(a) else None
            dw = L.dot(ap, dz, trans_a=True) if _tracked(w) else None
            return da, dw, db

        return Node(cp, (a, w, b), back, "fully_connected")

    def softmax_cross_entropy(self, logits, labels):
        """Batch-mean cross-entropy of softmax(logits) against `labels`
        (owl_optimise_generic.ml:172 and :646-649); reverse: (softmax -
        labels) * adjoint / batch."""
        L = self.layers
        zp = primal(logits)
        loss, _ = L.softmax_cross_entropy(zp, labels, want_loss=True)
        if not _tracked(logits):
            return loss

        def back(g):
            _, dz = L.softmax_cross_entropy(zp, labels, dloss=g, want_loss=False,
                                            want_grad=True)
            return (dz,)

        return Node(loss, (logits,), back, "softmax_cross_entropy")

    # conv family: ff_bb = forward stub, dr_a = backward_input, dr_b = backward_kernel
    def _conv(self, label, fwd, bwd_i, bwd_k, a, b):
        spec = _Piso(label, fwd,
                     lambda ap, bp, cp, ca: bwd_i(ap, bp, ca),
                     lambda ap, bp, cp, ca: bwd_k(ap, bp, ca))
        return build_piso(spec)(a, b)

    def conv1d(self, a, b, s, padding=SAME):
        """AD:2276 conv1d."""
        g = self.g
        return self._conv("conv1d", lambda x, w: g.conv1d(x, w, s, padding),
                          lambda x, w, o: g.conv1d_backward_input(x, w, s, o),
                          lambda x, w, o: g.conv1d_backward_kernel(x, w, s, o), a, b)

    def conv2d(self, a, b, s, padding=SAME):
        """AD:2327-2375 conv2d."""
        g = self.g
        return self._conv("conv2d", lambda x, w: g.conv2d(x, w, s, padding),
                          lambda x, w, o: g.conv2d_backward_input(x, w, s, o),
                          lambda x, w, o: g.conv2d_backward_kernel(x, w, s, o), a, b)

    def conv3d(self, a, b, s, padding=SAME):
        """AD:2378-2424 conv3d."""
        g = self.g
        return self._conv("conv3d", lambda x, w: g.conv3d(x, w, s, padding),
                          lambda x, w, o: g.conv3d_backward_input(x, w, s, o),
                          lambda x, w, o: g.conv3d_backward_kernel(x, w, s, o), a, b)

    def dilated_conv1d(self, a, b, s, r, padding=SAME):
        g = self.g
        return self._conv("dilated_conv1d", lambda x, w: g.dilated_conv1d(x, w, s, r, padding),
                          lambda x, w, o: g.dilated_conv1d_backward_input(x, w, s, r, o),
                          lambda x, w, o: g.dilated_conv1d_backward_kernel(x, w, s, r, o), a, b)

    def dilated_conv2d(self, a, b, s, r, padding=SAME):
        """AD:2477-2524 dilated_conv2d."""
        g = self.g
        return self._conv("dilated_conv2d", lambda x, w: g.dilated_conv2d(x, w, s, r, padding),
                          lambda x, w, o: g.dilated_conv2d_backward_input(x, w, s, r, o),
                          lambda x, w, o: g.dilated_conv2d_backward_kernel(x, w, s, r, o), a, b)

    def dilated_conv3d(self, a, b, s, r, padding=SAME):
        g = self.g
        return self._conv("dilated_conv3d", lambda x, w: g.dilated_conv3d(x, w, s, r, padding),
                          lambda x, w, o: g.dilated_conv3d_backward_input(x, w, s, r, o),
                          lambda x, w, o: g.dilated_conv3d_backward_kernel(x, w, s, r, o), a, b)

    def transpose_conv1d(self, a, b, s, padding=SAME):
        g = self.g
        return self._conv("transpose_conv1d", lambda x, w: g.transpose_conv1d(x, w, s, padding),
                          lambda x, w, o: g.transpose_conv1d_backward_input(x, w, s, o),
                          lambda x, w, o: g.transpose_conv1d_backward_kernel(x, w, s, o), a, b)

    def transpose_conv2d(self, a, b, s, padding=SAME):
        """AD:2629-2676 transpose_conv2d."""
        g = self.g
        return self._conv("transpose_conv2d", lambda x, w: g.transpose_conv2d(x, w, s, padding),
                          lambda x, w, o: g.transpose_conv2d_backward_input(x, w, s, o),
                          lambda x, w, o: g.transpose_conv2d_backward_kernel(x, w, s, o), a, b)

    def transpose_conv3d(self, a, b, s, padding=SAME):
        """AD:2677-2724 transpose_conv3d."""
        g = self.g
        return self._conv("transpose_conv3d", lambda x, w: g.transpose_conv3d(x, w, s, padding),
                          lambda x, w, o: g.transpose_conv3d_backward_input(x, w, s, o),
                          lambda x, w, o: g.transpose_conv3d_backward_kernel(x, w, s, o), a, b)

    # pool family: ff_arr = forward stub, dr = pool backward (mask recomputed)
    def _pool(self, label, fwd, bwd, a):
        return build_siso(_Siso(label, fwd, lambda ap, cp, ca: bwd(ap, ca)))(a)

    def max_pool1d(self, padding, a, b, s):
        g = self.g
        return self._pool("max_pool1d", lambda x: g.max_pool1d(x, b, s, padding),
                          lambda x, o: g.max_pool1d_backward(padding, x, b, s, o), a)

    def avg_pool1d(self, padding, a, b, s):
        g = self.g
        return self._pool("avg_pool1d", lambda x: g.avg_pool1d(x, b, s, padding),
                          lambda x, o: g.avg_pool1d_backward(padding, x, b, s, o), a)

    def max_pool2d(self, padding, a, b, s):
        """AD:2754-2778 max_pool2d."""
        g = self.g
        return self._pool("max_pool2d", lambda x: g.max_pool2d(x, b, s, padding),
                          lambda x, o: g.max_pool2d_backward(padding, x, b, s, o), a)

    def max_pool3d(self, padding, a, b, s):
        """AD:2781-2805 max_pool3d."""
        g = self.g
        return self._pool("max_pool3d", lambda x: g.max_pool3d(x, b, s, padding),
                          lambda x, o: g.max_pool3d_backward(padding, x, b, s, o), a)

    def avg_pool2d(self, padding, a, b, s):
        """AD:2835-2859 avg_pool2d."""
        g = self.g
        return self._pool("avg_pool2d", lambda x: g.avg_pool2d(x, b, s, padding),
                          lambda x, o: g.avg_pool2d_backward(padding, x, b, s, o), a)

    def avg_pool3d(self, padding, a, b, s):
        """AD:2862-2886 avg_pool3d."""
        g = self.g
        return self._pool("avg_pool3d", lambda x: g.avg_pool3d(x, b, s, padding),
                          lambda x, o: g.avg_pool3d_backward(padding, x, b, s, o), a)

    def upsampling2d(self, a, s):
        """AD:2889-2910 upsampling2d (a:input, s:size); reverse =
        upsampling2d_backward on the output adjoint."""
        g = self.g
        return self._pool("upsampling2d", lambda x: g.upsampling2d(x, s),
                          lambda x, o: g.upsampling2d_backward(x, s, o), a)


class Algodiff:
    """``Algodiff`` over one stub provider: ``ad.NN`` (conv/pool),
    ``ad.Maths`` and the tape functions."""

    def __init__(self, nn: _NN):
        self.nn = nn
        self.NN = _NNOps(nn)
        self._one = {}
        self.Maths = Maths
        self.make_reverse = make_reverse
        self.reverse_prop = reverse_prop
        self.grad = grad
        self.primal = primal
        self.build_siso = build_siso
        self.build_piso = build_piso


# ---- central-difference check (owl_algodiff_check.ml:22-98) -----------------------


def check_grad(loss: Callable[[dict], Any], params: dict, grads: dict, name: str,
               indices: Sequence[int], eps: float = 1e-6, floor: float = 1e-2):
    """Compare ``grads[name]`` with central differences of `loss` at the flat
    `indices` of ``params[name]``: returns (max error, per-index (analytic,
    numeric)), the error being |analytic - numeric| / max(|analytic|,
    |numeric|, floor) -- relative for gradients above `floor`, absolute
    (scaled by 1/floor) below it, where the difference quotient's own
    rounding noise (about 1e-16 |loss| / eps) dominates.  `loss` must
    evaluate without the tape."""
    p = params[name]
    flat = p.reshape(-1)
    out = []
    worst = 0.0
    ga = grads[name].reshape(-1)
    for i in indices:
        i = int(i)
        old = _scalar(flat[i])
        flat[i] = old + eps
        lp = _scalar(loss(params))
        flat[i] = old - eps
        lm = _scalar(loss(params))
        flat[i] = old
        num = (lp - lm) / (2 * eps)
        ana = _scalar(ga[i])
        scale = max(abs(num), abs(ana), floor)
        worst = max(worst, abs(num - ana) / scale)
        out.append((ana, num))
    return worst, out


# ---- the small CNN of the training-step workload (examples/mnist_cnn.ml) ----------

MNIST_CNN = (("w1", (5, 5, 1, 32)), ("b1", (32,)), ("w2", (5, 5, 32, 64)), ("b2", (64,)),
             ("w3", (3136, 1024)), ("b3", (1024,)), ("w4", (1024, 10)), ("b4", (10,)))


def init_mnist_cnn(seed: int = 0, dtype=np.float32) -> dict:
    """He-initialised weights (N(0, 2/fan_in)), zero biases."""
    rng = np.random.default_rng(seed)
    params = {}
    for name, shape in MNIST_CNN:
        if name.startswith("w"):
            fan_in = int(np.prod(shape[:-1]))
            params[name] = (rng.standard_normal(shape) * math.sqrt(2.0 / fan_in)).astype(dtype)
        else:
            params[name] = np.zeros(shape, dtype=dtype)
    return params


def mnist_cnn_loss(ad: Algodiff, p: dict, x, onehot):
    """conv 5x5x1x32 SAME + bias, ReLU, max_pool 2x2, conv 5x5x32x64 SAME +
    bias, ReLU, max_pool 2x2, dense 3136->1024 + bias, ReLU, dense 1024->10 +
    bias, softmax cross-entropy (mean over the batch).  Each conv + bias +
    ReLU and each dense layer is one fused op of the library."""
    M, N = ad.Maths, ad.NN
    h = N.conv2d_bias_act(x, p["w1"], p["b1"], [1, 1], SAME, ACT_RELU)
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = N.conv2d_bias_act(h, p["w2"], p["b2"], [1, 1], SAME, ACT_RELU)
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = M.reshape(h, (primal(h).shape[0], 3136))
    h = N.fully_connected(h, p["w3"], p["b3"], ACT_RELU)
    z = N.fully_connected(h, p["w4"], p["b4"], ACT_NONE)
    return N.softmax_cross_entropy(z, onehot)


def mnist_cnn_loss_composed(ad: Algodiff, p: dict, x, onehot):
    """The same network from Owl's separate operations (conv2d, add, relu,
    dot, softmax cross-entropy), as Owl's neurons compose them: the
    reference the fused ops are checked against."""
    M, N = ad.Maths, ad.NN
    h = M.relu(M.add(N.conv2d(x, p["w1"], [1, 1], SAME), p["b1"]))
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = M.relu(M.add(N.conv2d(h, p["w2"], [1, 1], SAME), p["b2"]))
    h = N.max_pool2d(SAME, h, [2, 2], [2, 2])
    h = M.reshape(h, (primal(h).shape[0], 3136))
    h = M.relu(M.add(M.dot(h, p["w3"]), p["b3"]))
    z = M.add(M.dot(h, p["w4"]), p["b4"])
    return M.softmax_cross_entropy(z, onehot)


def _seed(ad: Algodiff, loss):
    """The loss adjoint 1.  On the device: one cached value, so that a
    captured step launches no fill kernel."""
    if ad.NN.layers.gpu and _is_torch(loss):
        key = (loss.dtype, loss.device)
        one = ad._one.get(key)
        if one is None:
            one = ad._one[key] = _ones_like(loss)
        return one
    return _ones_like(loss)


def loss_and_grads(ad: Algodiff, params: dict, x, onehot, model=mnist_cnn_loss):
    """One reverse sweep: (loss value, {name: gradient})."""
    nodes = {k: make_reverse(v, k) for k, v in params.items()}
    loss = model(ad, nodes, x, onehot)
    reverse_prop(_seed(ad, loss.p), loss)
    return loss.p, {k: n.adj for k, n in nodes.items()}


def sgd_step(ad: Algodiff, params: dict, x, onehot, lr: float = 0.01, model=mnist_cnn_loss):
    """A training step: loss, gradients, and in-place SGD update (the
    library's update kernel on the device)."""
    loss, grads = loss_and_grads(ad, params, x, onehot, model)
    for k, g in grads.items():
        ad.NN.layers.sgd_update(params[k], g, lr)
    return loss, grads
