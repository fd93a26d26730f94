"""Owl's MEC and naive conv spellings.  The C ABI declares and exports them
for every kind; Owl's own compiled MEC and naive stubs give the same results
as its im2col / GEBP stubs (which the host drop-in aliases them to) and pass
Owl's conv2d / conv3d known-answer tests, as Owl's unit_conv_mec_naive.ml
checks."""

import numpy as np
import pytest

from golden_cases import CASES, MEC, MEC_NAIVE_FILES, NAIVE, Spelling, case_id, matches, run_case

SPELLINGS = {"mec": MEC, "naive": NAIVE}
CONV_CASES = [c for c in CASES if c["file"] in MEC_NAIVE_FILES]


def test_header_declares_every_spelling():
    from owl_gb300._lib import PROTOS

    for names in SPELLINGS.values():
        for base, alias in names.items():
            for kind in ("float32", "float64", "complex32", "complex64"):
                a, b = PROTOS[f"owl_{kind}_ndarray_{alias}"], PROTOS[f"owl_{kind}_ndarray_{base}"]
                assert a == b, alias


@pytest.fixture(scope="module")
def ref_backend():
    import oracle

    if not oracle.ref_available():
        pytest.skip("compiled reference stubs not available on this machine")
    return oracle.RefBackend()


def test_known_answer_cases_exist():
    assert len(CONV_CASES) >= 40


@pytest.mark.parametrize("sp", list(SPELLINGS))
@pytest.mark.parametrize("c", CONV_CASES, ids=[case_id(c) for c in CONV_CASES])
def test_owl_spelling_passes_owl_known_answers(ref_backend, sp, c):
    from owl_gb300.dense import NN

    ok, err = matches(run_case(NN(Spelling(ref_backend, SPELLINGS[sp])), c), c)
    assert ok, f"sum|diff| = {err}"


@pytest.mark.parametrize("sp", list(SPELLINGS))
@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex128])
@pytest.mark.parametrize("case", [((2, 7, 9, 5), (3, 2, 5, 4), (1, 1), "SAME"),
                                  ((1, 8, 8, 3), (3, 3, 3, 6), (2, 2), "VALID"),
                                  ((1, 5, 6, 4), (2, 3, 4, 2), (2, 1), "SAME")])
def test_owl_spelling_equals_im2col(ref_backend, sp, dt, case):
    from owl_gb300.dense import NN

    R, S = NN(ref_backend), NN(Spelling(ref_backend, SPELLINGS[sp]))
    xs, ks, st, pad = case
    rng = np.random.default_rng(21)
    u = lambda s: (rng.uniform(-1, 1, s) + (1j * rng.uniform(-1, 1, s) if dt == np.complex128
                                             else 0)).astype(dt)  # noqa: E731
    x, w = u(xs), u(ks)
    t = 1e-5 if dt == np.float32 else 1e-12
    rel = lambda a, b: np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)  # noqa: E731
    y = R.conv2d(x, w, list(st), pad)
    assert rel(S.conv2d(x, w, list(st), pad), y) < t
    dy = u(y.shape)
    for f in ("conv2d_backward_input", "conv2d_backward_kernel"):
        assert rel(getattr(S, f)(x, w, list(st), dy), getattr(R, f)(x, w, list(st), dy)) < t, f
    x3, w3 = u((1, 5, 4, 6, 2)), u((2, 3, 2, 2, 3))
    y3 = R.conv3d(x3, w3, [1, 2, 1], pad)
    assert rel(S.conv3d(x3, w3, [1, 2, 1], pad), y3) < t
    dy3 = u(y3.shape)
    for f in ("conv3d_backward_input", "conv3d_backward_kernel"):
        assert rel(getattr(S, f)(x3, w3, [1, 2, 1], dy3), getattr(R, f)(x3, w3, [1, 2, 1], dy3)) < t
