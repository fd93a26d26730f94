"""The MEC and naive host drop-in spellings on the GPU: Owl's conv2d /
conv3d known-answer tests through each (as Owl's unit_conv_mec_naive.ml
runs them), and results identical to the im2col / GEBP entry points."""

import numpy as np
import pytest

from golden_cases import CASES, MEC, MEC_NAIVE_FILES, NAIVE, Spelling, case_id, matches, run_case

pytestmark = pytest.mark.gpu
SPELLINGS = {"mec": MEC, "naive": NAIVE}
CONV_CASES = [c for c in CASES if c["file"] in MEC_NAIVE_FILES]


@pytest.fixture(scope="module")
def gpu_backend(gpu_lib):
    from owl_gb300.dense import GpuBackend

    return GpuBackend("fp32")


@pytest.mark.parametrize("sp", list(SPELLINGS))
@pytest.mark.parametrize("c", CONV_CASES, ids=[case_id(c) for c in CONV_CASES])
def test_spelling_passes_owl_known_answers(gpu_backend, sp, c):
    from owl_gb300.dense import NN

    ok, err = matches(run_case(NN(Spelling(gpu_backend, SPELLINGS[sp])), c), c)
    assert ok, f"sum|diff| = {err}"


@pytest.mark.parametrize("sp", list(SPELLINGS))
@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex64])
def test_spelling_identical_to_im2col(gpu_backend, sp, dt):
    from owl_gb300.dense import NN

    G, S = NN(gpu_backend), NN(Spelling(gpu_backend, SPELLINGS[sp]))
    rng = np.random.default_rng(22)
    u = lambda s: (rng.uniform(-1, 1, s) + (1j * rng.uniform(-1, 1, s) if dt == np.complex64
                                             else 0)).astype(dt)  # noqa: E731
    x, w = u((2, 9, 7, 6)), u((3, 3, 6, 5))
    y = G.conv2d(x, w, [2, 1], "SAME")
    assert np.array_equal(S.conv2d(x, w, [2, 1], "SAME"), y)
    dy = u(y.shape)
    for f in ("conv2d_backward_input", "conv2d_backward_kernel"):
        assert np.array_equal(getattr(S, f)(x, w, [2, 1], dy), getattr(G, f)(x, w, [2, 1], dy)), f
    x3, w3 = u((1, 5, 4, 6, 2)), u((2, 3, 2, 2, 3))
    y3 = G.conv3d(x3, w3, [1, 2, 1], "VALID")
    assert np.array_equal(S.conv3d(x3, w3, [1, 2, 1], "VALID"), y3)
    dy3 = u(y3.shape)
    for f in ("conv3d_backward_input", "conv3d_backward_kernel"):
        assert np.array_equal(getattr(S, f)(x3, w3, [1, 2, 1], dy3),
                              getattr(G, f)(x3, w3, [1, 2, 1], dy3)), f
