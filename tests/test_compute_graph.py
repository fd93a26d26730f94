"""The lazy computation-graph device (owl_gb300.compute) on the CPU.

A graph of Owl's conv/pool symbols, evaluated by the engine into planned
buffers, gives the same arrays as calling the same functions eagerly; freed
buffers are reused by later nodes of the same shape; shapes are inferred
(and bad shapes rejected) when a node is built; a graph re-evaluates after
`assign_arr` (owl_computation_cpu_engine.ml eval_graph).  Run on the oracle."""

import numpy as np
import pytest

from owl_gb300 import compute as C
from owl_gb300.dense import InvalidArgument

SAME, VALID = "SAME", "VALID"


def _u(rng, shape):
    return rng.uniform(-1, 1, shape).astype(np.float32)


def _cnn(rng):
    """x -> conv -> maxpool -> conv -> conv -> upsample -> dilated conv,
    then both conv2d gradients of the first layer against the result."""
    x = C.var_arr((2, 8, 8, 3), "x")
    w1 = C.pack_arr(_u(rng, (3, 3, 3, 4)), "w1")
    w2 = C.pack_arr(_u(rng, (3, 3, 4, 4)), "w2")
    w3 = C.pack_arr(_u(rng, (3, 3, 4, 4)), "w3")
    w4 = C.pack_arr(_u(rng, (3, 3, 4, 4)), "w4")
    y1 = C.conv2d(x, w1, [1, 1])
    p = C.max_pool2d(y1, [2, 2], [2, 2])
    y2 = C.conv2d(p, w2, [1, 1])
    y3 = C.conv2d(y2, w3, [1, 1])
    u = C.upsampling2d(y3, [2, 2])
    d = C.dilated_conv2d(u, w4, [1, 1], [2, 2])
    gi = C.conv2d_backward_input(x, w1, [1, 1], d)
    gk = C.conv2d_backward_kernel(x, w1, [1, 1], d)
    return x, (w1, w2, w3, w4), (y1, p, y2, y3, u, d, gi, gk)


def _eager(nn, xv, ws):
    w1, w2, w3, w4 = (C.unpack_arr(w) for w in ws)
    y1 = nn.conv2d(xv, w1, [1, 1])
    p = nn.max_pool2d(y1, [2, 2], [2, 2])
    y3 = nn.conv2d(nn.conv2d(p, w2, [1, 1]), w3, [1, 1])
    d = nn.dilated_conv2d(nn.upsampling2d(y3, [2, 2]), w4, [1, 1], [2, 2])
    return nn.conv2d_backward_input(xv, w1, [1, 1], d), nn.conv2d_backward_kernel(xv, w1, [1, 1], d)


def test_inferred_shapes():
    rng = np.random.default_rng(70)
    _, _, (y1, p, y2, y3, u, d, gi, gk) = _cnn(rng)
    assert y1.shape == (2, 8, 8, 4) and p.shape == (2, 4, 4, 4) and y3.shape == (2, 4, 4, 4)
    assert u.shape == (2, 8, 8, 4) and d.shape == (2, 8, 8, 4)
    assert gi.shape == (2, 8, 8, 3) and gk.shape == (3, 3, 3, 4)
    assert [n.op for n in (y1, p, u, d, gi, gk)] == [
        "Conv2d", "MaxPool2d", "UpSampling2d", "DilatedConv2d", "Conv2dBackwardInput",
        "Conv2dBackwardKernel"]
    v = C.var_arr((1, 9, 9, 2))
    assert C.conv2d(v, C.var_arr((3, 3, 2, 5)), [2, 2], VALID).shape == (1, 4, 4, 5)
    assert C.avg_pool3d(C.var_arr((1, 4, 4, 4, 2)), [2, 2, 2], [2, 2, 2]).shape == (1, 2, 2, 2, 2)
    assert C.transpose_conv1d(C.var_arr((2, 5, 3)), C.var_arr((3, 3, 4)), [2]).shape == (2, 10, 4)


def test_bad_shapes_fail_when_built():
    x = C.var_arr((2, 8, 8, 3))
    with pytest.raises(InvalidArgument):
        C.conv2d(x, C.var_arr((3, 3, 4, 4)), [1, 1])  # in-channels 3 vs 4
    with pytest.raises(InvalidArgument):
        C.max_pool2d(x, [2, 2], [2, 2], "FULL")
    with pytest.raises(InvalidArgument):
        C.assign_arr(x, np.zeros((2, 8, 8, 4), np.float32))
    with pytest.raises(InvalidArgument):
        C.assign_arr(x, np.zeros((2, 8, 8, 3)))  # float64 into a float32 variable


def test_every_symbol_has_a_builder():
    for op, fn in C._OPS.items():
        assert callable(getattr(C, fn)), op


def test_graph_equals_eager_and_reuses_buffers(oracle_nn):
    rng = np.random.default_rng(71)
    x, ws, nodes = _cnn(rng)
    gi, gk = nodes[-2:]
    g = C.make_graph([x], [gi, gk], "cnn")
    dev = C.Device(oracle_nn)
    for seed in (72, 73):
        xv = _u(np.random.default_rng(seed), x.shape)
        C.assign_arr(x, xv)
        got = C.eval_graph(g, dev)
        ref = _eager(oracle_nn, xv, ws)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    # 8 operator nodes: p's buffer goes to y3 and y1's to u, so 6 buffers
    assert g.buffers == 6
    assert nodes[3].buffer is nodes[1].buffer and nodes[4].buffer is nodes[0].buffer
    # outputs keep buffers of their own
    owners = [n.buffer for n in nodes[:-2]]
    assert all(gi.buffer is not b and gk.buffer is not b for b in owners)


def test_graph_1d_3d_and_pool_backward(oracle_nn):
    rng = np.random.default_rng(74)
    x1 = C.var_arr((2, 9, 3))
    k1 = C.pack_arr(_u(rng, (3, 3, 4)))
    y1 = C.conv1d(x1, k1, [2])
    x3 = C.var_arr((1, 5, 4, 5, 2))
    k3 = C.pack_arr(_u(rng, (2, 2, 2, 2, 3)))
    y3 = C.max_pool3d(C.conv3d(x3, k3, [1, 1, 1]), [2, 2, 2], [2, 2, 2])
    q = C.var_arr((2, 6, 6, 3))
    dq = C.var_arr((2, 3, 3, 3))
    pb = C.avg_pool2d_backward(SAME, q, [2, 2], [2, 2], dq)
    g = C.make_graph([x1, x3, q, dq], [y1, y3, pb])
    v = {n: _u(rng, n.shape) for n in (x1, x3, q, dq)}
    for n, a in v.items():
        C.assign_arr(n, a)
    got = C.eval_graph(g, C.Device(oracle_nn))
    nn = oracle_nn
    ref = [nn.conv1d(v[x1], C.unpack_arr(k1), [2]),
           nn.max_pool3d(nn.conv3d(v[x3], C.unpack_arr(k3), [1, 1, 1]), [2, 2, 2], [2, 2, 2]),
           nn.avg_pool2d_backward(SAME, v[q], [2, 2], [2, 2], v[dq])]
    for a, b in zip(got, ref):
        assert a.shape == b.shape and np.array_equal(a, b)


def test_unassigned_inputs_are_errors(oracle_nn):
    x = C.var_arr((1, 4, 4, 2))
    y = C.max_pool2d(x, [2, 2], [2, 2])
    with pytest.raises(InvalidArgument):
        C.make_graph([], [y])  # a variable that is neither input nor packed
    g = C.make_graph([x], [y])
    with pytest.raises(InvalidArgument):
        C.eval_graph(g, C.Device(oracle_nn))
    with pytest.raises(InvalidArgument):
        C.unpack_arr(y)


def test_complex_graph(oracle_nn):
    """Complex64 (Owl's Complex32) nodes plan and evaluate like real ones."""
    rng = np.random.default_rng(75)
    c = lambda s: (rng.uniform(-1, 1, s) + 1j * rng.uniform(-1, 1, s)).astype(np.complex64)  # noqa: E731
    x = C.var_arr((2, 6, 6, 2), "x", np.complex64)
    w = C.pack_arr(c((3, 3, 2, 3)))
    y = C.avg_pool2d(C.conv2d(x, w, [1, 1]), [2, 2], [2, 2])
    assert y.dtype == np.complex64 and y.shape == (2, 3, 3, 3)
    g = C.make_graph([x], [y])
    xv = c(x.shape)
    C.assign_arr(x, xv)
    (got,) = C.eval_graph(g, C.Device(oracle_nn))
    ref = oracle_nn.avg_pool2d(oracle_nn.conv2d(xv, C.unpack_arr(w), [1, 1]), [2, 2], [2, 2])
    assert np.array_equal(got, ref)


class _TorchOracle:
    """The oracle over torch CPU tensors (shared-memory numpy views), so the
    engine's torch path (buffer allocation, element types) runs on the CPU."""

    name = "torch-oracle"

    def __init__(self, inner):
        self.inner = inner

    def stub(self, kind, op, *args):
        import torch

        self.inner.stub(kind, op, *[a.numpy() if isinstance(a, torch.Tensor) else a
                                    for a in args])

    def empty(self, like, shape, dtype=None):
        import torch

        return torch.empty(tuple(shape), dtype=dtype or like.dtype)

    def shape(self, a):
        return tuple(a.shape)

    def reshape(self, a, shape):
        return a.reshape(shape)


@pytest.mark.parametrize("dt", [np.float32, np.complex128])
def test_graph_on_torch_tensors(oracle_nn, dt):
    import torch

    from owl_gb300.dense import NN

    rng = np.random.default_rng(76)
    u = lambda s: (rng.uniform(-1, 1, s) + (1j * rng.uniform(-1, 1, s) if dt == np.complex128
                                             else 0)).astype(dt)  # noqa: E731
    x = C.var_arr((2, 8, 8, 3), "x", dt)
    w = C.pack_arr(torch.from_numpy(u((3, 3, 3, 4))))
    y = C.avg_pool2d(C.conv2d(x, w, [1, 1]), [2, 2], [2, 2])
    g = C.make_graph([x], [C.conv2d_backward_kernel(x, w, [1, 1], C.upsampling2d(y, [2, 2]))])
    xv = u(x.shape)
    C.assign_arr(x, torch.from_numpy(xv))
    (got,) = C.eval_graph(g, C.Device(NN(_TorchOracle(oracle_nn.b))))
    assert isinstance(got, torch.Tensor) and got.dtype == getattr(torch, np.dtype(dt).name)
    wv = C.unpack_arr(w).numpy()
    up = oracle_nn.upsampling2d(oracle_nn.avg_pool2d(oracle_nn.conv2d(xv, wv, [1, 1]), [2, 2],
                                                     [2, 2]), [2, 2])
    assert np.array_equal(got.numpy(), oracle_nn.conv2d_backward_kernel(xv, wv, [1, 1], up))


def test_graph_whose_output_is_an_input(oracle_nn):
    """A variable listed as an output is returned as assigned; operator nodes
    between it and the other outputs still run."""
    x = C.var_arr((1, 4, 4, 2), "x")
    y = C.avg_pool2d(x, [2, 2], [2, 2])
    g = C.make_graph([x], [x, y])
    xv = np.arange(32, dtype=np.float32).reshape(x.shape)
    C.assign_arr(x, xv)
    a, b = C.eval_graph(g, C.Device(oracle_nn))
    assert a is xv and np.array_equal(b, oracle_nn.avg_pool2d(xv, [2, 2], [2, 2]))
    assert g.buffers == 1
