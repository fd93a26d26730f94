"""owl_gb300 -- Owl's dense-ndarray convolution and pooling path on GB300.

* ``libowlgpu.so`` (``csrc/``): the CUDA kernels behind a C ABI
  (``include/owlgpu.h``) whose entry points replace Owl's conv/pool C stubs.
* ``dense``: the shape/padding/dispatch layer of Owl's ndarray NN functions,
  restated over any stub provider (``NN(GpuBackend())``).
* ``algodiff``: conv/pool registered as reverse-mode differentiable ops.
* ``serving``: a continuous-batching inference loop over the conv/pool ops.
"""

from .dense import NN, SAME, VALID, GpuBackend, InvalidArgument  # noqa: F401


def gpu(precision: str = "fp32") -> NN:
    """The Owl conv/pool function set on the GPU library."""
    return NN(GpuBackend(precision))
