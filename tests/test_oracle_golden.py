"""Pin the CPU oracle (and Owl's own compiled stubs, where available) to the
known-answer tests in Owl's test suite."""

import numpy as np
import pytest

from golden_cases import CASES, case_id, matches, run_case


@pytest.mark.parametrize("c", CASES, ids=[case_id(c) for c in CASES])
def test_oracle_matches_owl_golden(oracle_nn, c):
    ok, err = matches(run_case(oracle_nn, c), c)
    assert ok, f"sum|diff| = {err}"


@pytest.mark.parametrize("c", CASES, ids=[case_id(c) for c in CASES])
def test_oracle_float64_matches_owl_golden(oracle_nn, c):
    ok, err = matches(run_case(oracle_nn, c, dtype=np.float64), c)
    assert ok, f"sum|diff| = {err}"


@pytest.mark.parametrize("c", CASES, ids=[case_id(c) for c in CASES])
def test_compiled_reference_matches_owl_golden(ref_nn, c):
    ok, err = matches(run_case(ref_nn, c), c)
    assert ok, f"sum|diff| = {err}"
