"""A device for Owl's lazy computation graph, for the conv/pool path.

Owl evaluates a computation graph through a device module
(src/base/types/owl_types_computation_device.ml:6-30: make_device,
arr_to_value, value_to_arr, ...) and an engine that first plans one output
buffer per node (owl_computation_cpu_init.ml, `_init_terms`; buffers are
shared between nodes whose lifetimes do not overlap) and then runs every
node into its buffer with the `_ ~out` variant of its ndarray function
(owl_computation_cpu_eval.ml:180-281, e.g. `Conv2d (padding, stride) ->
A.conv2d_ ~out ~padding x.(0) x.(1) stride`).  The CPU device is the only
one Owl ships; the type `device_type = CPU | OpenCL | CUDA`
(owl_types_common.ml:48-51) names the others.

This module is that device and engine for a GPU, over the NN function set
of owl_gb300.dense: values are the backend's arrays (CUDA tensors for the
libowlgpu backend), every node runs the NN function of its Owl symbol with
`out=` its planned buffer, and a planned graph can be captured once as a
CUDA graph and replayed with new input values (Owl re-evaluates a graph
after `assign_arr`).  The layers keep Owl's names: symbols (`var_arr`,
`pack_arr`, `assign_arr`, `unpack_arr`), operators (`conv2d`, `max_pool2d`,
... building nodes named as Owl's symbols: `Conv2d`, `MaxPool2d`, ...), the
graph (`make_graph`) and the engine (`eval_graph`).  Shapes are inferred when
a node is built, by the NN functions' own shape rules (so a bad shape raises
Owl's error at build time, as Owl's operators do), run over shape-only
placeholders.
"""

from __future__ import annotations

from collections import defaultdict

import numpy as np

from .dense import NN, SAME, Backend, InvalidArgument

# Owl symbols of the conv/pool family (owl_computation_cpu_eval.ml:180-281)
# and the NN function each runs with `out=`.
_OPS = {
    "Conv1d": "conv1d", "Conv2d": "conv2d", "Conv3d": "conv3d",
    "TransposeConv1d": "transpose_conv1d", "TransposeConv2d": "transpose_conv2d",
    "TransposeConv3d": "transpose_conv3d",
    "DilatedConv1d": "dilated_conv1d", "DilatedConv2d": "dilated_conv2d",
    "DilatedConv3d": "dilated_conv3d",
    "MaxPool1d": "max_pool1d", "MaxPool2d": "max_pool2d", "MaxPool3d": "max_pool3d",
    "AvgPool1d": "avg_pool1d", "AvgPool2d": "avg_pool2d", "AvgPool3d": "avg_pool3d",
    "UpSampling2d": "upsampling2d",
    "Conv1dBackwardInput": "conv1d_backward_input",
    "Conv1dBackwardKernel": "conv1d_backward_kernel",
    "Conv2dBackwardInput": "conv2d_backward_input",
    "Conv2dBackwardKernel": "conv2d_backward_kernel",
    "Conv3dBackwardInput": "conv3d_backward_input",
    "Conv3dBackwardKernel": "conv3d_backward_kernel",
    "TransposeConv1dBackwardInput": "transpose_conv1d_backward_input",
    "TransposeConv1dBackwardKernel": "transpose_conv1d_backward_kernel",
    "TransposeConv2dBackwardInput": "transpose_conv2d_backward_input",
    "TransposeConv2dBackwardKernel": "transpose_conv2d_backward_kernel",
    "TransposeConv3dBackwardInput": "transpose_conv3d_backward_input",
    "TransposeConv3dBackwardKernel": "transpose_conv3d_backward_kernel",
    "DilatedConv1dBackwardInput": "dilated_conv1d_backward_input",
    "DilatedConv1dBackwardKernel": "dilated_conv1d_backward_kernel",
    "DilatedConv2dBackwardInput": "dilated_conv2d_backward_input",
    "DilatedConv2dBackwardKernel": "dilated_conv2d_backward_kernel",
    "DilatedConv3dBackwardInput": "dilated_conv3d_backward_input",
    "DilatedConv3dBackwardKernel": "dilated_conv3d_backward_kernel",
    "MaxPool1dBackward": "max_pool1d_backward", "MaxPool2dBackward": "max_pool2d_backward",
    "MaxPool3dBackward": "max_pool3d_backward", "AvgPool1dBackward": "avg_pool1d_backward",
    "AvgPool2dBackward": "avg_pool2d_backward", "AvgPool3dBackward": "avg_pool3d_backward",
    "UpSampling2dBackward": "upsampling2d_backward",
}


# ---- shape-only placeholders (build-time shape inference) ----------------------

def _np_dtype(d) -> np.dtype:
    """The numpy dtype of a numpy or torch element type."""
    if type(d).__module__.startswith("torch"):
        return np.dtype(str(d).replace("torch.", ""))
    return np.dtype(d)


class _Shape:
    """An array that has only a shape and an element kind."""

    __slots__ = ("shape", "dtype")

    def __init__(self, shape, dtype):
        self.shape = tuple(int(d) for d in shape)
        self.dtype = _np_dtype(dtype)

    def reshape(self, shape):
        return _Shape(shape, self.dtype)


class _ShapeBackend(Backend):
    """Runs the NN functions' argument checks and shape rules, nothing else."""

    name = "shape"

    def empty(self, like, shape, dtype=None):
        return _Shape(shape, dtype or like.dtype)

    def stub(self, kind, op, *args):
        pass

    def reshape(self, a, shape):
        return _Shape(shape, a.dtype)


_SHAPE_NN = NN(_ShapeBackend())


# ---- symbols --------------------------------------------------------------------

class Node:
    """A graph node: an input variable (`Var`) or an Owl symbol applied to
    parent nodes and constant parameters, with its inferred shape; `value`
    holds its array once assigned (variables) or evaluated."""

    def __init__(self, op: str, args=(), kwargs=None, shape=(), dtype=np.float32, name=""):
        self.op = op
        self.args = tuple(args)
        self.kwargs = dict(kwargs or {})
        self.parents = [a for a in (*self.args, *self.kwargs.values()) if isinstance(a, Node)]
        self.shape = tuple(int(d) for d in shape)
        self.dtype = _np_dtype(dtype)
        self.name = name
        self.value = None   # the current array
        self.buffer = None  # planned output buffer (operator nodes)

    def __repr__(self) -> str:
        return f"Node({self.op}{' ' + self.name if self.name else ''}, shape={list(self.shape)})"


def var_arr(shape, name: str = "", dtype=np.float32) -> Node:
    """owl_computation_symbol.ml `var_arr ?shape name`: an input variable."""
    return Node("Var", shape=shape, dtype=dtype, name=name)


def assign_arr(x: Node, arr) -> None:
    """owl_computation_symbol.ml `assign_arr`: bind a variable to an array of
    its shape and element type."""
    if x.op != "Var":
        raise InvalidArgument("assign_arr: only a variable can be assigned")
    if tuple(arr.shape) != x.shape or _np_dtype(arr.dtype) != x.dtype:
        raise InvalidArgument(f"assign_arr: {arr.dtype} {list(arr.shape)} should be "
                              f"{x.dtype} {list(x.shape)}")
    x.value = arr


def pack_arr(arr, name: str = "") -> Node:
    """owl_computation_symbol.ml `pack_arr`: a variable holding `arr`."""
    x = var_arr(arr.shape, name, arr.dtype)
    x.value = arr
    return x


def unpack_arr(x: Node):
    """owl_computation_symbol.ml `unpack_arr`: the node's array (after
    evaluation for operator nodes)."""
    if x.value is None:
        raise InvalidArgument(f"unpack_arr: {x!r} has no value yet (evaluate its graph)")
    return x.value


# ---- operators ------------------------------------------------------------------

def _make(op: str, *args, **kwargs) -> Node:
    """owl_computation_operator.ml `make_then_connect`: a node for symbol `op`
    over `args`; its shape comes from the NN function's own shape rule."""
    ph = lambda a: _Shape(a.shape, a.dtype) if isinstance(a, Node) else a  # noqa: E731
    y = getattr(_SHAPE_NN, _OPS[op])(*map(ph, args), **{k: ph(v) for k, v in kwargs.items()})
    return Node(op, args, kwargs, y.shape, y.dtype)


def conv1d(input, kernel, stride, padding=SAME):
    return _make("Conv1d", input, kernel, list(stride), padding)


def conv2d(input, kernel, stride, padding=SAME):
    return _make("Conv2d", input, kernel, list(stride), padding)


def conv3d(input, kernel, stride, padding=SAME):
    return _make("Conv3d", input, kernel, list(stride), padding)


def transpose_conv1d(input, kernel, stride, padding=SAME):
    return _make("TransposeConv1d", input, kernel, list(stride), padding)


def transpose_conv2d(input, kernel, stride, padding=SAME):
    return _make("TransposeConv2d", input, kernel, list(stride), padding)


def transpose_conv3d(input, kernel, stride, padding=SAME):
    return _make("TransposeConv3d", input, kernel, list(stride), padding)


def dilated_conv1d(input, kernel, stride, rate, padding=SAME):
    return _make("DilatedConv1d", input, kernel, list(stride), list(rate), padding)


def dilated_conv2d(input, kernel, stride, rate, padding=SAME):
    return _make("DilatedConv2d", input, kernel, list(stride), list(rate), padding)


def dilated_conv3d(input, kernel, stride, rate, padding=SAME):
    return _make("DilatedConv3d", input, kernel, list(stride), list(rate), padding)


def max_pool1d(input, kernel, stride, padding=SAME):
    return _make("MaxPool1d", input, list(kernel), list(stride), padding)


def max_pool2d(input, kernel, stride, padding=SAME):
    return _make("MaxPool2d", input, list(kernel), list(stride), padding)


def max_pool3d(input, kernel, stride, padding=SAME):
    return _make("MaxPool3d", input, list(kernel), list(stride), padding)


def avg_pool1d(input, kernel, stride, padding=SAME):
    return _make("AvgPool1d", input, list(kernel), list(stride), padding)


def avg_pool2d(input, kernel, stride, padding=SAME):
    return _make("AvgPool2d", input, list(kernel), list(stride), padding)


def avg_pool3d(input, kernel, stride, padding=SAME):
    return _make("AvgPool3d", input, list(kernel), list(stride), padding)


def upsampling2d(input, size):
    return _make("UpSampling2d", input, list(size))


def upsampling2d_backward(input, size, output_):
    return _make("UpSampling2dBackward", input, list(size), output_)


def _bwd(op):
    def f(input, kernel, stride, output_):
        return _make(op, input, kernel, list(stride), output_)

    f.__name__ = _OPS[op]
    f.__doc__ = f"owl_computation_operator.ml `{_OPS[op]}`: symbol {op}."
    return f


def _bwd_dilated(op):
    def f(input, kernel, stride, rate, output_):
        return _make(op, input, kernel, list(stride), list(rate), output_)

    f.__name__ = _OPS[op]
    f.__doc__ = f"owl_computation_operator.ml `{_OPS[op]}`: symbol {op}."
    return f


def _pool_bwd(op):
    def f(padding, input, kernel, stride, output_):
        return _make(op, padding, input, list(kernel), list(stride), output_)

    f.__name__ = _OPS[op]
    f.__doc__ = f"owl_computation_operator.ml `{_OPS[op]}`: symbol {op}."
    return f


conv1d_backward_input = _bwd("Conv1dBackwardInput")
conv1d_backward_kernel = _bwd("Conv1dBackwardKernel")
conv2d_backward_input = _bwd("Conv2dBackwardInput")
conv2d_backward_kernel = _bwd("Conv2dBackwardKernel")
conv3d_backward_input = _bwd("Conv3dBackwardInput")
conv3d_backward_kernel = _bwd("Conv3dBackwardKernel")
transpose_conv1d_backward_input = _bwd("TransposeConv1dBackwardInput")
transpose_conv1d_backward_kernel = _bwd("TransposeConv1dBackwardKernel")
transpose_conv2d_backward_input = _bwd("TransposeConv2dBackwardInput")
transpose_conv2d_backward_kernel = _bwd("TransposeConv2dBackwardKernel")
transpose_conv3d_backward_input = _bwd("TransposeConv3dBackwardInput")
transpose_conv3d_backward_kernel = _bwd("TransposeConv3dBackwardKernel")
dilated_conv1d_backward_input = _bwd_dilated("DilatedConv1dBackwardInput")
dilated_conv1d_backward_kernel = _bwd_dilated("DilatedConv1dBackwardKernel")
dilated_conv2d_backward_input = _bwd_dilated("DilatedConv2dBackwardInput")
dilated_conv2d_backward_kernel = _bwd_dilated("DilatedConv2dBackwardKernel")
dilated_conv3d_backward_input = _bwd_dilated("DilatedConv3dBackwardInput")
dilated_conv3d_backward_kernel = _bwd_dilated("DilatedConv3dBackwardKernel")
max_pool1d_backward = _pool_bwd("MaxPool1dBackward")
max_pool2d_backward = _pool_bwd("MaxPool2dBackward")
max_pool3d_backward = _pool_bwd("MaxPool3dBackward")
avg_pool1d_backward = _pool_bwd("AvgPool1dBackward")
avg_pool2d_backward = _pool_bwd("AvgPool2dBackward")
avg_pool3d_backward = _pool_bwd("AvgPool3dBackward")


# ---- device -----------------------------------------------------------------------

class Device:
    """owl_types_computation_device.ml `device`: the NN function set the
    nodes run on (libowlgpu for a GPU device, any stub provider otherwise)."""

    def __init__(self, nn: NN):
        self.nn = nn

    # value <-> array: values are the backend's arrays themselves
    @staticmethod
    def arr_to_value(arr):
        return arr

    @staticmethod
    def value_to_arr(value):
        return value

    @staticmethod
    def is_arr(value) -> bool:
        return hasattr(value, "shape")


def make_device(precision: str = "fp32") -> Device:
    """owl_types_computation_device.ml `make_device`: a GPU device running
    libowlgpu at `precision` (fp32, tf32, bf16, bf16x3)."""
    from .dense import GpuBackend

    return Device(NN(GpuBackend(precision)))


# ---- graph and engine --------------------------------------------------------------

class Graph:
    """owl_computation_graph.ml `make_graph ~input ~output name`: the nodes
    reachable from `output`, in an order where each follows its parents."""

    def __init__(self, input, output, name: str = ""):
        self.input = list(input)
        self.output = list(output)
        self.name = name
        order, seen = [], set()

        def visit(n):
            if id(n) in seen:
                return
            seen.add(id(n))
            for p in n.parents:
                visit(p)
            order.append(n)

        for o in self.output:
            visit(o)
        self.order = order
        for n in order:
            if n.op == "Var" and n not in self.input and n.value is None:
                raise InvalidArgument(f"make_graph: variable {n!r} is neither an input nor packed")
        self.buffers = 0  # distinct output buffers planned
        self._planned_for = None

    def _plan(self, device: Device) -> None:
        """Owl's init pass: one buffer per operator node, a buffer reused by a
        later node of the same shape and kind once every reader of its
        previous owner has run (outputs keep theirs)."""
        like = next(n.value for n in self.order if n.op == "Var")
        readers = defaultdict(int)
        for n in self.order:
            for p in set(map(id, n.parents)):
                readers[p] += 1
        keep = set(map(id, self.output))
        free = defaultdict(list)
        count = 0
        for n in self.order:
            if n.op == "Var":
                continue
            key = (n.shape, str(n.dtype))
            if free[key]:
                n.buffer = free[key].pop()
            else:
                n.buffer = device.nn.b.empty(like, n.shape, _like_dtype(like, n.dtype))
                count += 1
            for p in {id(q): q for q in n.parents}.values():
                readers[id(p)] -= 1
                if readers[id(p)] == 0 and p.op != "Var" and id(p) not in keep:
                    free[(p.shape, str(p.dtype))].append(p.buffer)
        self.buffers = count
        self._planned_for = (id(device), tuple(_where(n.value) for n in self.order
                                                if n.op == "Var"))

    def _run(self, device: Device) -> None:
        val = lambda a: a.value if isinstance(a, Node) else a  # noqa: E731
        for n in self.order:
            if n.op == "Var":
                continue
            getattr(device.nn, _OPS[n.op])(*map(val, n.args), out=n.buffer,
                                           **{k: val(v) for k, v in n.kwargs.items()})
            n.value = n.buffer

    def compile(self, device: Device) -> "CompiledGraph":
        """Plan the buffers, run once, and capture the evaluation as a CUDA
        graph (device values only); replay it with new input values."""
        return CompiledGraph(self, device)


def _where(a) -> str:
    return str(getattr(a, "device", "host"))


def _like_dtype(like, dtype):
    """`dtype` in the array library of `like` (numpy or torch)."""
    if type(like).__module__.startswith("torch"):
        import torch

        return getattr(torch, str(dtype))  # float32, float64, complex64, complex128
    return dtype


def make_graph(input, output, name: str = "") -> Graph:
    return Graph(input, output, name)


def eval_graph(graph: Graph, device: Device):
    """owl_computation_cpu_engine.ml `eval_graph`: plan (once per device and
    input placement), then run every node into its buffer; returns the
    outputs' arrays."""
    for n in graph.input:
        if n.value is None:
            raise InvalidArgument(f"eval_graph: input {n!r} is not assigned")
    key = (id(device), tuple(_where(n.value) for n in graph.order if n.op == "Var"))
    if graph._planned_for != key:
        graph._plan(device)
    graph._run(device)
    return [unpack_arr(o) for o in graph.output]


class CompiledGraph:
    """A planned graph captured once as a CUDA graph.  `run(inputs)` copies
    each input array into its variable's buffer and replays the captured
    kernels; the outputs are the graph's output buffers (overwritten by the
    next run).  Packed arrays (weights) are captured by address: update them
    in place (`copy_`), not by rebinding the node to a new array."""

    def __init__(self, graph: Graph, device: Device):
        import torch

        self.graph, self.device = graph, device
        # inputs live in buffers owned by the compiled graph
        for n in graph.input:
            if n.value is None:
                raise InvalidArgument(f"compile: input {n!r} is not assigned")
            n.value = n.value.clone()
        eval_graph(graph, device)  # plans, warms the library's per-shape state
        torch.cuda.synchronize()
        self._g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self._g):
            graph._run(device)
        torch.cuda.synchronize()

    def run(self, inputs: dict):
        for n, arr in inputs.items():
            if n not in self.graph.input:
                raise InvalidArgument(f"run: {n!r} is not an input of the graph")
            n.value.copy_(arr)
        self._g.replay()
        return [o.value for o in self.graph.output]
