"""The lazy computation-graph device on the GPU: a graph of Owl's conv/pool
symbols evaluated through libowlgpu into planned device buffers equals the
same calls made eagerly (bit for bit: the kernels are deterministic), stays
within the fp32 bound of the oracle, and a graph captured once as a CUDA
graph replays with new input values to the eager results."""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev
from owl_gb300 import compute as C
from test_compute_graph import _cnn, _eager, _u

pytestmark = pytest.mark.gpu


def _device_graph(rng):
    x, ws, nodes = _cnn(rng)
    for w in ws:  # weights move to the device
        w.value = to_dev(w.value)
    return x, ws, nodes


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_graph_equals_eager_on_device(gpu_lib, oracle_nn, precision):
    rng = np.random.default_rng(80)
    x, ws, nodes = _device_graph(rng)
    gi, gk = nodes[-2:]
    g = C.make_graph([x], [gi, gk])
    dev = C.make_device(precision)
    for seed in (81, 82):
        xv = _u(np.random.default_rng(seed), x.shape)
        C.assign_arr(x, to_dev(xv))
        got = [from_dev(a) for a in C.eval_graph(g, dev)]
        ref = [from_dev(a) for a in _eager(dev.nn, x.value, ws)]
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
        if precision == "fp32":
            host_ws = [type(w)("Var") for w in ws]
            for h, w in zip(host_ws, ws):
                h.value = from_dev(w.value).astype(np.float64)
            orc = _eager(oracle_nn, xv.astype(np.float64), host_ws)
            for a, b in zip(got, orc):
                assert rel(a, b) < 1e-5
    assert g.buffers == 6


def test_captured_graph_replays_new_inputs(gpu_lib):
    import torch

    rng = np.random.default_rng(83)
    x, ws, nodes = _device_graph(rng)
    gi, gk = nodes[-2:]
    g = C.make_graph([x], [gi, gk])
    dev = C.make_device("bf16")
    C.assign_arr(x, to_dev(_u(rng, x.shape)))
    cg = g.compile(dev)
    for seed in (84, 85, 86):
        xv = to_dev(_u(np.random.default_rng(seed), x.shape))
        got = [from_dev(a) for a in cg.run({x: xv})]
        ref = [from_dev(a) for a in _eager(dev.nn, xv, ws)]
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    torch.cuda.synchronize()
