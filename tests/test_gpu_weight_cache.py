"""The weight-image cache of the tensor-core convolutions
(owlgpu_weights_declare / owlgpu_weights_forget): a declared kernel tensor's
re-laid-out images are built once per version and layout and reused, with
results bit-identical to the per-call re-layout; a new version after an
in-place change of the weights takes effect; a call captured in a CUDA graph
after the first call launches no re-layout.  No counterpart in Owl."""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu


def _nn(prec="bf16"):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend(prec))


@pytest.fixture
def declared(gpu_lib):
    """Kernel tensors declared in a test; forgotten afterwards, before
    torch may reuse their addresses."""
    from owl_gb300 import _lib

    held = []

    def declare(t, version):
        _lib.call("owlgpu_weights_declare", t.data_ptr(), version)
        held.append(t)

    yield declare
    for t in held:
        _lib.call("owlgpu_weights_forget", t.data_ptr())


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
def test_cached_images_give_the_same_results(declared, prec):
    rng = np.random.default_rng(61)
    x = to_dev(rng.uniform(-1, 1, (2, 20, 18, 64)).astype(np.float32))
    w_np = (rng.standard_normal((3, 3, 64, 96)) * 0.06).astype(np.float32)
    dy = to_dev(rng.standard_normal((2, 20, 18, 96)).astype(np.float32))
    G = _nn(prec)
    plain = to_dev(w_np)  # never declared: re-laid out per call
    ref_y = from_dev(G.conv2d(x, plain, [1, 1], "SAME"))
    ref_dx = from_dev(G.conv2d_backward_input(x, plain, [1, 1], dy))
    w = to_dev(w_np)
    declared(w, 0)
    for _ in range(3):  # the first call builds each layout's image, the others reuse it
        assert np.array_equal(from_dev(G.conv2d(x, w, [1, 1], "SAME")), ref_y)
        assert np.array_equal(from_dev(G.conv2d_backward_input(x, w, [1, 1], dy)), ref_dx)


def test_new_version_after_an_in_place_change(declared, oracle_nn):
    rng = np.random.default_rng(62)
    x_np = rng.uniform(-1, 1, (1, 16, 16, 32)).astype(np.float32)
    x = to_dev(x_np)
    w = to_dev((rng.standard_normal((3, 3, 32, 64)) * 0.08).astype(np.float32))
    G = _nn()
    declared(w, 7)
    G.conv2d(x, w, [1, 1], "SAME")
    w.mul_(-2.0)  # the caller changes the weights ...
    declared(w, 8)  # ... and declares their new contents
    y = from_dev(G.conv2d(x, w, [1, 1], "SAME"))
    ref = oracle_nn.conv2d(x_np.astype(np.float64), from_dev(w).astype(np.float64), [1, 1],
                           "SAME")
    assert rel(y, ref) <= 1e-2


def test_captured_call_launches_no_relayout(declared):
    import torch

    from owl_gb300 import _lib

    rng = np.random.default_rng(63)
    x = to_dev(rng.uniform(-1, 1, (4, 28, 28, 64)).astype(np.float32))
    w = to_dev((rng.standard_normal((3, 3, 64, 128)) * 0.05).astype(np.float32))
    G = _nn()
    ref = from_dev(G.conv2d(x, w, [1, 1], "SAME"))
    declared(w, 0)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        G.conv2d(x, w, [1, 1], "SAME")  # builds the image, outside capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    n0 = _lib.launch_count()
    with torch.cuda.graph(g):
        y = G.conv2d(x, w, [1, 1], "SAME")
    assert _lib.launch_count() - n0 == 1  # the convolution alone
    g.replay()
    assert np.array_equal(from_dev(y), ref)
    del g


@pytest.mark.parametrize("case", ["strided", "transpose"])
def test_cached_multi_segment_layouts(declared, case):
    """Layouts with several segments: a stride-2 backward_input (one
    segment per residue class) and a kernel = stride transpose convolution
    (classes fused into one launch): cached images give the per-call
    results bit for bit."""
    rng = np.random.default_rng(64)
    G = _nn()
    if case == "strided":
        x = to_dev(rng.uniform(-1, 1, (2, 15, 15, 32)).astype(np.float32))
        w_np = (rng.standard_normal((3, 3, 32, 64)) * 0.08).astype(np.float32)
        dy = to_dev(rng.standard_normal((2, 7, 7, 64)).astype(np.float32))
        run = lambda w: G.conv2d_backward_input(x, w, [2, 2], dy)
    else:
        x = to_dev(rng.uniform(-1, 1, (2, 7, 9, 48)).astype(np.float32))
        w_np = (rng.standard_normal((2, 2, 48, 40)) * 0.2).astype(np.float32)
        run = lambda w: G.transpose_conv2d(x, w, [2, 2], "SAME")
    ref = from_dev(run(to_dev(w_np)))
    w = to_dev(w_np)
    declared(w, 3)
    for _ in range(2):
        assert np.array_equal(from_dev(run(w)), ref)
