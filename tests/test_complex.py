"""Complex32 / Complex64 conv, pool and upsampling on the CPU: the oracle
against outputs of Owl's own complex C stubs (tests/golden/owl_complex.npz,
made by make_complex_fixtures.py) and, where the compiled stubs are present,
against them live; the semantics of Owl's complex max pooling; the C header's
complex entry points."""

from pathlib import Path

import numpy as np
import pytest

from golden.make_complex_fixtures import CASES, KINDS, call

FIX = np.load(Path(__file__).resolve().parent / "golden" / "owl_complex.npz")
SAME, VALID = "SAME", "VALID"
EXACT = ("pool", "upsampling")  # element-wise order-fixed ops: bit for bit


def fixture_inputs(kind, name):
    n = len(CASES[name][1])
    return [FIX[f"{kind}/{name}/in{i}"] for i in range(n)]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def tol(kind):
    return 1e-5 if kind == "complex32" else 1e-12


def check(kind, name, got):
    want = FIX[f"{kind}/{name}"]
    assert got.dtype == want.dtype and got.shape == want.shape
    if any(k in CASES[name][0] for k in EXACT):
        assert np.array_equal(got, want), name
    else:
        assert rel(got, want) < tol(kind), name


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("name", list(CASES))
def test_oracle_matches_owl_complex_stubs(oracle_nn, kind, name):
    check(kind, name, call(oracle_nn, name, fixture_inputs(kind, name)))


@pytest.mark.parametrize("kind", list(KINDS))
def test_oracle_argmax_matches_owl(oracle_nn, kind):
    x = fixture_inputs(kind, "max_pool2d")[0]
    v, i = oracle_nn.max_pool2d_argmax(x, [2, 2], [2, 2], SAME)
    assert np.array_equal(v, FIX[f"{kind}/max_pool2d_argmax/value"])
    assert np.array_equal(i, FIX[f"{kind}/max_pool2d_argmax/index"])


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
@pytest.mark.parametrize("case", [((2, 7, 9, 5), (3, 2, 5, 4), (1, 1), SAME),
                                  ((1, 5, 6, 4), (2, 3, 4, 2), (2, 1), VALID)])
def test_oracle_vs_compiled_stubs_live(oracle_nn, ref_nn, dt, case):
    xs, ks, st, pad = case
    rng = np.random.default_rng(9)
    c = lambda s: (rng.uniform(-1, 1, s) + 1j * rng.uniform(-1, 1, s)).astype(dt)  # noqa: E731
    x, w = c(xs), c(ks)
    t = 1e-5 if dt == np.complex64 else 1e-12
    y = oracle_nn.conv2d(x, w, list(st), pad)
    assert rel(y, ref_nn.conv2d(x, w, list(st), pad)) < t
    dy = c(y.shape)
    for f in ("conv2d_backward_input", "conv2d_backward_kernel"):
        a = getattr(oracle_nn, f)(x, w, list(st), dy)
        assert rel(a, getattr(ref_nn, f)(x, w, list(st), dy)) < t, f
    for f in ("max_pool2d", "avg_pool2d"):
        assert np.array_equal(getattr(oracle_nn, f)(x, [2, 3], list(st), pad),
                              getattr(ref_nn, f)(x, [2, 3], list(st), pad)), f


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_complex_max_pool_semantics(oracle_nn, dt):
    """Owl's complex max pooling starts its accumulator at -INFINITY, the
    complex (-inf, 0), whose magnitude is infinite: the magnitude-then-argument
    comparison never prefers an input, so every output is (-inf, 0), every
    argmax -1, and the backward routes every gradient to flat element 0 (the
    initial max_idx), summed in output order."""
    rng = np.random.default_rng(3)
    x = ((rng.uniform(-1, 1, (2, 6, 6, 3)) + 1j * rng.uniform(-1, 1, (2, 6, 6, 3))) * 100).astype(dt)
    y = oracle_nn.max_pool2d(x, [2, 2], [2, 2], SAME)
    assert np.all(y.real == -np.inf) and np.all(y.imag == 0)
    _, idx = oracle_nn.max_pool2d_argmax(x, [2, 2], [2, 2], SAME)
    assert np.all(idx == -1)
    dy = (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)).astype(dt)
    dx = oracle_nn.max_pool2d_backward(SAME, x, [2, 2], [2, 2], dy)
    s = dt(0)
    for v in dy.ravel():
        s = dt(s + v)
    assert dx.ravel()[0] == s and np.count_nonzero(dx.ravel()[1:]) == 0


@pytest.mark.parametrize("dt,rt", [(np.complex64, np.float32), (np.complex128, np.float64)])
def test_complex_avg_pool_is_the_real_pool_of_both_parts(oracle_nn, dt, rt):
    """Complex average pooling sums componentwise and divides by the count:
    the real pool over the (re, im) pairs seen as twice the channels."""
    rng = np.random.default_rng(4)
    x = (rng.uniform(-1, 1, (2, 7, 5, 3)) + 1j * rng.uniform(-1, 1, (2, 7, 5, 3))).astype(dt)
    y = oracle_nn.avg_pool2d(x, [3, 2], [2, 1], SAME)
    yr = oracle_nn.avg_pool2d(x.view(rt), [3, 2], [2, 1], SAME)
    assert np.array_equal(y.view(rt), yr)


def test_header_declares_complex_entry_points():
    from owl_gb300._lib import PROTOS

    # (the allocation-free entry point and the bias + activation extensions
    # are float32 / float64 only: an activation orders values)
    real = [n for n in PROTOS if "_float32_ndarray_" in n and not n.endswith("_noalloc")
            and not n.endswith("_bias_act")]
    assert len(real) > 40
    for n in real:
        for kind in ("complex32", "complex64"):
            c = n.replace("float32", kind)
            assert c in PROTOS, c
            assert len(PROTOS[c][1]) == len(PROTOS[n][1]), c
            assert all("complex" in t for t, _ in PROTOS[c][1] if "float" in t or "double" in t)
