"""The serving loop on the GPU: requests of mixed sides and batches go
through the continuous-batching scheduler (grouped, padded to buckets,
replayed from captured CUDA graphs on several streams) and each result is
compared with the same request computed alone (eager, same precision).

Each image is computed independently by the conv and pool kernels and the
accumulation order of a convolution does not depend on the batch, so the
results are expected to be identical; the bound stated is 1e-6 relative
(float32 reassociation level), far below the BF16 error against float64
(checked separately: at most 1e-2 of max|y| after 21 BF16 convolutions, the
accuracy bar the served results are reported at)."""

import numpy as np
import pytest

from gpu_util import from_dev, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(gpu_lib):
    import torch

    from owl_gb300.dense import NN, GpuBackend
    from owl_gb300.serving import (GraphExecutor, ResidualStack, Scheduler, attach_pixels,
                                   init_stack, poisson_stream)

    w = {k: torch.from_numpy(v).cuda() for k, v in init_stack(0).items()}
    stack = ResidualStack(w, NN(GpuBackend("bf16")))
    reqs = poisson_stream(40, 4000.0, seed=7, sides=(14, 28, 56), max_batch=24)
    attach_pixels(reqs, seed=8, pool=32, pinned=True)
    ex = GraphExecutor(stack, streams=4)
    sch = Scheduler(ex, hbm_budget=8 << 30, max_group=48)
    st = sch.run(reqs)
    sch.close()
    yield stack, reqs, st
    stack.release()


def test_every_request_served(served):
    _, reqs, st = served
    assert st.completed == len(reqs)
    assert st.groups < len(reqs)  # some requests shared a forward pass
    assert all(r.output is not None and r.output.shape == (r.batch, 10) for r in reqs)


def test_result_same_alone_and_in_the_mix(served):
    import torch

    stack, reqs, _ = served
    worst = 0.0
    for r in reqs:
        alone = from_dev(stack.forward(r.pixels.cuda()))
        worst = max(worst, rel(r.output, alone))
    print("max relative difference, mixed vs alone:", worst)
    assert worst <= 1e-6


def test_bf16_error_against_float64(served):
    import torch

    from owl_gb300.dense import NN, GpuBackend
    from owl_gb300.serving import ResidualStack, init_stack

    stack, reqs, _ = served
    w64 = {k: torch.from_numpy(v.astype(np.float64)).cuda() for k, v in init_stack(0).items()}
    s64 = ResidualStack(w64, NN(GpuBackend("fp32")))
    errs = []
    for r in reqs[:6]:
        y64 = from_dev(s64.forward(r.pixels.double().cuda()))
        errs.append(rel(r.output, y64))
    s64.release()
    print("BF16 serving error vs float64:", max(errs))
    assert max(errs) <= 1e-2
