"""Owl's own conv/pool known-answer tests through the CUDA library, on both
the host drop-in entry points and the device-resident ones, and Owl's conv
cases once more through the tcgen05 tensor-core kernels at BF16 and TF32."""

import numpy as np
import pytest

from golden_cases import CASES, HELPERS, case_id, matches, run_case
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


CONV_CASES = [c for c in CASES if c["helper"] != "test_forward"
              and not HELPERS[c["helper"]][0].startswith(("max_pool", "avg_pool"))]
# the bars of the conv workloads; rounding both operands of these cases to
# BF16 moves them by at most 1.5e-3, to TF32 by at most 1.9e-4
TC_TOL = {"bf16": 1e-2, "tf32": 5e-3}


@pytest.fixture(scope="module", params=sorted(TC_TOL))
def tc_nn(request, gpu_lib):
    from owl_gb300.dense import NN, GpuBackend

    return request.param, NN(GpuBackend(request.param))


@pytest.mark.parametrize("c", CONV_CASES, ids=[case_id(c) for c in CONV_CASES])
def test_tensor_core(tc_nn, c):
    """Owl's conv, dilated and transpose known answers (forward and both
    backwards, 2-D and 3-D) on the tcgen05 kernels with BF16 or TF32
    operands and FP32 accumulation: max|result - expected| within the
    precision's bar times max|expected|.  Owl's own absolute bar (sum |diff|
    < 5e-4) is a float32 bar; these inputs are integer sequences that BF16
    and TF32 do not hold exactly."""
    from owl_gb300 import _lib

    prec, nn = tc_nn
    r = np.asarray(run_case(nn, c, to_dev=to_dev, from_dev=from_dev), np.float64).reshape(-1)
    exp = np.asarray(c["expected"], np.float64)
    assert r.size == exp.size
    assert np.abs(r - exp).max() <= TC_TOL[prec] * np.abs(exp).max()
    assert _lib.lib().owlgpu_last_conv_path() == 1  # the tcgen05 kernels ran
