"""Complex32 / Complex64 on the GPU through the C ABI: device-resident
(torch complex tensors) and host drop-in (numpy) calls against outputs of
Owl's own complex stubs (tests/golden/owl_complex.npz) -- pooling, argmax
and upsampling bit for bit, convolutions within 1e-5 (complex32) / 1e-12
(complex64) -- and a larger convolution against the oracle."""

import numpy as np
import pytest

from golden.make_complex_fixtures import CASES, KINDS, call
from gpu_util import from_dev, to_dev
from test_complex import FIX, check, fixture_inputs, rel, tol

pytestmark = pytest.mark.gpu
SAME = "SAME"


@pytest.fixture(scope="module")
def gpu_nn(gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend("fp32"))


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("name", list(CASES))
def test_device_matches_owl_complex_stubs(gpu_nn, kind, name):
    got = call(gpu_nn, name, [to_dev(a) for a in fixture_inputs(kind, name)])
    check(kind, name, from_dev(got))


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("name", ["conv2d_s1_same", "conv2d_bwd_kernel", "conv3d_bwd_input",
                                  "avg_pool2d", "max_pool2d_bwd", "upsampling2d_bwd"])
def test_host_drop_in_matches_owl_complex_stubs(gpu_nn, kind, name):
    check(kind, name, call(gpu_nn, name, fixture_inputs(kind, name)))


@pytest.mark.parametrize("kind", list(KINDS))
def test_argmax_matches_owl(gpu_nn, kind):
    x = fixture_inputs(kind, "max_pool2d")[0]
    v, i = gpu_nn.max_pool2d_argmax(to_dev(x), [2, 2], [2, 2], SAME)
    assert np.array_equal(from_dev(v), FIX[f"{kind}/max_pool2d_argmax/value"])
    assert np.array_equal(from_dev(i), FIX[f"{kind}/max_pool2d_argmax/index"])


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_larger_conv_against_oracle(gpu_nn, oracle_nn, dt):
    rng = np.random.default_rng(12)
    c = lambda s: (rng.uniform(-1, 1, s) + 1j * rng.uniform(-1, 1, s)).astype(dt)  # noqa: E731
    x, w = c((4, 20, 18, 24)), c((3, 3, 24, 40))
    kind = "complex32" if dt == np.complex64 else "complex64"
    y = from_dev(gpu_nn.conv2d(to_dev(x), to_dev(w), [1, 1], SAME))
    assert rel(y, oracle_nn.conv2d(x, w, [1, 1], SAME)) < tol(kind)
    dy = c(y.shape)
    dw = from_dev(gpu_nn.conv2d_backward_kernel(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    assert rel(dw, oracle_nn.conv2d_backward_kernel(x, w, [1, 1], dy)) < tol(kind)
    dx = from_dev(gpu_nn.conv2d_backward_input(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    assert rel(dx, oracle_nn.conv2d_backward_input(x, w, [1, 1], dy)) < tol(kind)
    # overlapping max-pool backward over many windows: all into element 0
    g = c((4, 20, 18, 24))
    dxp = from_dev(gpu_nn.max_pool2d_backward(SAME, to_dev(x), [3, 3], [1, 1], to_dev(g)))
    assert np.array_equal(dxp, oracle_nn.max_pool2d_backward(SAME, x, [3, 3], [1, 1], g))
