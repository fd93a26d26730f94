"""upsampling2d (Owl's G:8223-8330 and the upsampling backward stub) on the
CPU: the oracle against Owl's known-answer tests and against Owl's own
compiled stub, the host mirror's argument checks, and Algodiff."""

import numpy as np
import pytest

from upsampling_cases import UP_CASES, run_up_case, up_id


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("c", UP_CASES, ids=[up_id(c) for c in UP_CASES])
def test_oracle_matches_owl_golden(oracle_nn, c, dt):
    got, expected = run_up_case(oracle_nn, c, dt)
    # Owl's tolerance is sum |a - b| < 5e-4; the values are small integers,
    # so the sums are exact
    assert np.abs(got - expected).sum() < 5e-4
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("c", [c for c in UP_CASES if c["op"] == "backward"],
                         ids=[up_id(c) for c in UP_CASES if c["op"] == "backward"])
def test_compiled_reference_matches_owl_golden(ref_nn, c):
    got, expected = run_up_case(ref_nn, c)
    assert np.array_equal(got, expected)


SHAPES = [((2, 5, 7, 4), (2, 3)), ((3, 4, 3, 5), (3, 1)), ((1, 6, 6, 16), (1, 1)),
          ((2, 3, 5, 3), (4, 2))]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("shape,size", SHAPES)
def test_oracle_backward_bit_exact_with_reference(oracle_nn, ref_nn, dt, shape, size):
    rng = np.random.default_rng(17)
    x = rng.uniform(-1, 1, shape).astype(dt)
    oshape = (shape[0], shape[1] * size[0], shape[2] * size[1], shape[3])
    dy = rng.standard_normal(oshape).astype(dt)
    a = oracle_nn.upsampling2d_backward(x, list(size), dy)
    b = ref_nn.upsampling2d_backward(x, list(size), dy)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("oc,or_", [(9, 5), (5, 9), (2, 3)])
def test_stub_clamps_like_owl(oracle_nn, ref_nn, dt, oc, or_):
    """Called directly (not through G), the stub accepts any output extent:
    output cols/rows past input*scale add into the last input col/row and
    missing ones contribute nothing.  IC = 3, IR = 2, scales 2 x 2."""
    rng = np.random.default_rng(5)
    dy = rng.standard_normal((2, oc, or_, 3)).astype(dt)
    outs = []
    for nn in (oracle_nn, ref_nn):
        dx = np.empty((2, 3, 2, 3), dtype=dt)
        nn.b.stub("float32" if dt == np.float32 else "float64", "upsampling_spatial_backward",
                  dx, dy, 2, 3, 2, 3, oc, or_, 2, 2)
        outs.append(dx)
    assert np.array_equal(outs[0], outs[1])


def test_forward_is_repeat(oracle_nn):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 4, 3, 5))
    y = oracle_nn.upsampling2d(x, [3, 2])
    assert np.array_equal(y, x.repeat(3, axis=1).repeat(2, axis=2))


def test_argument_checks_follow_owl(oracle_nn):
    from owl_gb300.dense import InvalidArgument

    x = np.zeros((1, 2, 3, 4))
    with pytest.raises(InvalidArgument, match="input dimension = 3"):
        oracle_nn.upsampling2d(np.zeros((2, 3, 4)), [2, 2])
    with pytest.raises(InvalidArgument, match="size dimension = 1"):
        oracle_nn.upsampling2d(x, [2])
    with pytest.raises(InvalidArgument, match="scaled output cols is 4"):
        oracle_nn.upsampling2d_backward(x, [2, 2], np.zeros((1, 5, 6, 4)))


def test_out_variant_overwrites(oracle_nn):
    x = np.ones((1, 2, 2, 2))
    out = np.full((1, 4, 2, 2), 7.0)
    r = oracle_nn.upsampling2d(x, [2, 1], out=out)
    assert r is out and np.array_equal(out, np.ones((1, 4, 2, 2)))
