"""Owl's own conv/pool known-answer tests through the CUDA library, on both
the host drop-in entry points and the device-resident ones."""

import numpy as np
import pytest

from golden_cases import CASES, case_id, matches, run_case
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_nn(gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    return NN(GpuBackend("fp32"))


@pytest.mark.parametrize("c", CASES, ids=[case_id(c) for c in CASES])
def test_host_dropin_float32(gpu_nn, c):
    ok, err = matches(run_case(gpu_nn, c), c)
    assert ok, f"sum|diff| = {err}"


@pytest.mark.parametrize("c", CASES, ids=[case_id(c) for c in CASES])
def test_device_resident_float64(gpu_nn, c):
    ok, err = matches(run_case(gpu_nn, c, dtype=np.float64, to_dev=to_dev, from_dev=from_dev), c)
    assert ok, f"sum|diff| = {err}"
