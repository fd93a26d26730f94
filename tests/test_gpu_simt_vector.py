"""The float32 CUDA-core vector kernels (conv_f32v_kernel: 16-byte operand
gathers, 128x128, 128x64 or 256x32 tiles, 16-deep k slabs) at the edges of
where they apply, against the float32 oracle (Owl's S path restated) at
1e-4: output channels that fill no tile width (partial column tiles),
reduction lengths that end inside a k slab, several split-K partials,
strides, dilation and 3-D windows, kernel = stride backward_input as one
window-scatter GEMM, and operands that are not 16-byte aligned (which take
the scalar kernel instead, with the same results)."""

import numpy as np
import pytest

from gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _nn():
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend("fp32"))


def _vector_ran():
    from owl_gb300 import _lib

    L = _lib.lib()
    assert L.owlgpu_device_status() == 0, _lib.last_error()
    assert L.owlgpu_last_conv_path() == 0  # CUDA-core family


# input, kernel, stride, rate: Ci % 16 == 0 for the forward's vector path,
# output channels above 32 and a multiple of 4
CASES2D = [
    ((3, 11, 13, 32), (3, 3, 32, 100), [1, 1], [1, 1], "SAME"),   # 100 = 64 + 36 columns
    ((2, 9, 10, 48), (3, 3, 48, 36), [1, 1], [1, 1], "SAME"),     # 128x64 tile, 36 columns
    ((2, 17, 15, 64), (3, 3, 64, 68), [2, 2], [1, 1], "VALID"),   # strided, ragged pixels
    ((2, 16, 16, 32), (3, 3, 32, 132), [1, 1], [2, 3], "SAME"),   # dilated, 2 column tiles
    ((1, 7, 5, 16), (2, 2, 16, 40), [1, 2], [1, 1], "SAME"),      # 35 output pixels
]


@pytest.mark.parametrize("case", CASES2D)
def test_vector_conv2d_edges(gpu_lib, oracle_nn, case):
    xs, ks, st, rate, pad = case
    rng = np.random.default_rng(71)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.1).astype(np.float32)
    G, O = _nn(), oracle_nn
    xd, wd = to_dev(x), to_dev(w)
    y = O.dilated_conv2d(x, w, st, rate, pad)
    assert rel(from_dev(G.dilated_conv2d(xd, wd, st, rate, pad)), y) <= TOL
    _vector_ran()
    dy = rng.standard_normal(y.shape).astype(np.float32)
    dyd = to_dev(dy)
    assert rel(from_dev(G.dilated_conv2d_backward_input(xd, wd, st, rate, dyd)),
               O.dilated_conv2d_backward_input(x, w, st, rate, dy)) <= TOL
    assert rel(from_dev(G.dilated_conv2d_backward_kernel(xd, wd, st, rate, dyd)),
               O.dilated_conv2d_backward_kernel(x, w, st, rate, dy)) <= TOL


def test_vector_conv3d(gpu_lib, oracle_nn):
    rng = np.random.default_rng(72)
    x = rng.uniform(-1, 1, (2, 7, 6, 9, 32)).astype(np.float32)
    w = (rng.standard_normal((3, 2, 3, 32, 72)) * 0.1).astype(np.float32)
    G, O = _nn(), oracle_nn
    st = [1, 2, 1]
    y = O.conv3d(x, w, st, "SAME")
    assert rel(from_dev(G.conv3d(to_dev(x), to_dev(w), st, "SAME")), y) <= TOL
    dy = rng.standard_normal(y.shape).astype(np.float32)
    assert rel(from_dev(G.conv3d_backward_input(to_dev(x), to_dev(w), st, to_dev(dy))),
               O.conv3d_backward_input(x, w, st, dy)) <= TOL
    assert rel(from_dev(G.conv3d_backward_kernel(to_dev(x), to_dev(w), st, to_dev(dy))),
               O.conv3d_backward_kernel(x, w, st, dy)) <= TOL


def test_vector_backward_kernel_many_splits(gpu_lib, oracle_nn):
    """A long reduction (8 x 37 x 29 = 8584 output pixels, not a multiple of
    16) over few output tiles: split-K partials, the last slab partial."""
    rng = np.random.default_rng(73)
    x = rng.uniform(-1, 1, (8, 37, 29, 16)).astype(np.float32)
    w = (rng.standard_normal((3, 3, 16, 48)) * 0.1).astype(np.float32)
    dy = rng.standard_normal((8, 37, 29, 48)).astype(np.float32)
    G, O = _nn(), oracle_nn
    dw = from_dev(G.conv2d_backward_kernel(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    assert rel(dw, O.conv2d_backward_kernel(x, w, [1, 1], dy)) <= TOL
    again = from_dev(G.conv2d_backward_kernel(to_dev(x), to_dev(w), [1, 1], to_dev(dy)))
    assert np.array_equal(dw, again)  # fixed split and summation order


def test_unaligned_operands_give_the_same_results(gpu_lib):
    """Operands offset by 4 bytes from a 16-byte boundary run the scalar
    kernel; its sums run over k in the same order, so a forward gives the
    same bits as the vector kernel on aligned copies."""
    import torch

    from owl_gb300 import _lib

    rng = np.random.default_rng(74)
    xs, ks = (2, 12, 12, 32), (3, 3, 32, 96)
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.1).astype(np.float32)
    ys = (2, 12, 12, 96)
    aligned = from_dev(_nn().conv2d(to_dev(x), to_dev(w), [1, 1], "SAME"))

    def shifted(a):  # a device copy of `a` starting 4 bytes past an allocation
        buf = torch.zeros(a.size + 1, dtype=torch.float32, device="cuda")
        buf[1:] = torch.from_numpy(a.ravel()).cuda()
        return buf, buf[1:]

    xb, xv = shifted(x)
    wb, wv = shifted(w)
    yb, yv = shifted(np.zeros(ys, np.float32))
    assert xv.data_ptr() % 16 == 4
    stream = torch.cuda.current_stream().cuda_stream
    _lib.call("owlgpu_float32_ndarray_conv_spatial", xv.data_ptr(), wv.data_ptr(), yv.data_ptr(),
              2, 12, 12, 32, 3, 3, 12, 12, 96, 1, 1, 0, 1, 1, _lib.PREC["fp32"], stream)
    torch.cuda.synchronize()
    assert np.array_equal(yv.cpu().numpy().reshape(ys), aligned)
    del xb, wb, yb


@pytest.mark.parametrize("dims", [2, 3])
def test_window_backward_input(gpu_lib, oracle_nn, dims):
    """A backward_input whose kernel equals its stride (and the transpose
    convolution forward that is one) runs as one GEMM with a window-scatter
    epilogue; every dX element written once, against the float32 oracle."""
    rng = np.random.default_rng(75)
    G, O = _nn(), oracle_nn
    if dims == 2:
        xs, ks, st = (3, 12, 10, 36), (2, 2, 36, 48), [2, 2]
        bwd, conv = G.conv2d_backward_input, O.conv2d_backward_input
        tconv_g, tconv_o = G.transpose_conv2d, O.transpose_conv2d
    else:
        xs, ks, st = (2, 6, 8, 4, 20), (2, 2, 2, 20, 32), [2, 2, 2]
        bwd, conv = G.conv3d_backward_input, O.conv3d_backward_input
        tconv_g, tconv_o = G.transpose_conv3d, O.transpose_conv3d
    x = rng.uniform(-1, 1, xs).astype(np.float32)
    w = (rng.standard_normal(ks) * 0.2).astype(np.float32)
    oshape = (xs[0],) + tuple(d // s for d, s in zip(xs[1:-1], st)) + (ks[-1],)
    dy = rng.standard_normal(oshape).astype(np.float32)
    dx = from_dev(bwd(to_dev(x), to_dev(w), st, to_dev(dy)))
    assert rel(dx, conv(x, w, st, dy)) <= TOL
    # transpose convolution forward: kernel [.., in=Co, out=Ci]
    wt = np.ascontiguousarray(np.swapaxes(w, -1, -2))
    y = from_dev(tconv_g(to_dev(dy), to_dev(wt), st, "SAME"))
    assert rel(y, tconv_o(dy, wt, st, "SAME")) <= TOL
