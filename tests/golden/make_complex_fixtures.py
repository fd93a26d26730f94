"""Generate owl_complex.npz: outputs of Owl's own complex conv / pool /
upsampling C stubs on seeded inputs.

Owl's tests hold no complex vectors, so these fixtures are made by running
the reference itself: its C stubs compiled unmodified (oracle/Makefile,
`make ref`) and driven through the Python restatement of Owl's OCaml layer
(owl_gb300.dense.NN over oracle.RefBackend).  Only this script needs the
reference; the fixtures travel with the tests.

    python tests/golden/make_complex_fixtures.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "owl_complex.npz"
SAME, VALID = "SAME", "VALID"

# name -> (NN function, shapes of the complex array arguments, the other
# arguments in call order with "A<i>" marking array i)
CASES = {
    "conv2d_s1_same": ("conv2d", [(2, 7, 6, 3), (3, 3, 3, 4)], ["A0", "A1", [1, 1], SAME]),
    "conv2d_s2_valid": ("conv2d", [(2, 8, 7, 3), (3, 2, 3, 5)], ["A0", "A1", [2, 2], VALID]),
    "conv2d_bwd_input": ("conv2d_backward_input", [(2, 7, 6, 3), (3, 3, 3, 4), (2, 4, 3, 4)],
                         ["A0", "A1", [2, 2], "A2"]),
    "conv2d_bwd_kernel": ("conv2d_backward_kernel", [(2, 7, 6, 3), (3, 3, 3, 4), (2, 4, 3, 4)],
                          ["A0", "A1", [2, 2], "A2"]),
    "dilated_conv2d": ("dilated_conv2d", [(1, 9, 8, 2), (3, 3, 2, 3)],
                       ["A0", "A1", [1, 1], [2, 2], SAME]),
    "dilated_conv2d_bwd_kernel": ("dilated_conv2d_backward_kernel",
                                  [(1, 9, 8, 2), (3, 3, 2, 3), (1, 9, 8, 3)],
                                  ["A0", "A1", [1, 1], [2, 2], "A2"]),
    "transpose_conv2d": ("transpose_conv2d", [(2, 4, 3, 3), (2, 2, 3, 2)],
                         ["A0", "A1", [2, 2], SAME]),
    "conv3d": ("conv3d", [(1, 5, 4, 5, 2), (2, 2, 2, 2, 3)], ["A0", "A1", [1, 1, 1], SAME]),
    "conv3d_bwd_input": ("conv3d_backward_input", [(1, 5, 4, 5, 2), (2, 2, 2, 2, 3),
                                                   (1, 5, 4, 5, 3)],
                         ["A0", "A1", [1, 1, 1], "A2"]),
    "conv1d": ("conv1d", [(2, 9, 3), (3, 3, 4)], ["A0", "A1", [2], SAME]),
    "max_pool2d": ("max_pool2d", [(2, 6, 5, 3)], ["A0", [2, 2], [2, 2], SAME]),
    "avg_pool2d": ("avg_pool2d", [(2, 6, 5, 3)], ["A0", [3, 3], [1, 1], SAME]),
    "max_pool2d_bwd": ("max_pool2d_backward", [(2, 6, 5, 3), (2, 3, 3, 3)],
                       [SAME, "A0", [2, 2], [2, 2], "A1"]),
    "avg_pool2d_bwd": ("avg_pool2d_backward", [(2, 6, 5, 3), (2, 6, 5, 3)],
                       [SAME, "A0", [3, 3], [1, 1], "A1"]),
    "max_pool3d": ("max_pool3d", [(1, 4, 4, 4, 2)], ["A0", [2, 2, 2], [2, 2, 2], VALID]),
    "avg_pool3d_bwd": ("avg_pool3d_backward", [(1, 4, 4, 4, 2), (1, 2, 2, 2, 2)],
                       [VALID, "A0", [2, 2, 2], [2, 2, 2], "A1"]),
    "upsampling2d_bwd": ("upsampling2d_backward", [(2, 3, 4, 3), (2, 6, 8, 3)],
                         ["A0", [2, 2], "A1"]),
}

KINDS = {"complex32": np.complex64, "complex64": np.complex128}


def inputs(name: str, kind: str):
    """Seeded complex inputs of one case."""
    _, shapes, _ = CASES[name]
    rng = np.random.default_rng(sum(map(ord, name + kind)))
    dt = KINDS[kind]
    return [(rng.uniform(-1, 1, s) + 1j * rng.uniform(-1, 1, s)).astype(dt) for s in shapes]


def call(nn, name: str, arrays):
    fn, _, spec = CASES[name]
    args = [arrays[int(a[1:])] if isinstance(a, str) and a.startswith("A") and a[1:].isdigit()
            else a for a in spec]
    return getattr(nn, fn)(*args)


def main() -> None:
    import oracle
    from owl_gb300.dense import NN

    ref = NN(oracle.RefBackend())
    out = {}
    for kind in KINDS:
        for name in CASES:
            arrays = inputs(name, kind)
            for i, a in enumerate(arrays):  # stored: the tests do not rely on the RNG
                out[f"{kind}/{name}/in{i}"] = a
            out[f"{kind}/{name}"] = call(ref, name, arrays)
        x = inputs("max_pool2d", kind)[0]
        v, i = ref.max_pool2d_argmax(x, [2, 2], [2, 2], SAME)
        out[f"{kind}/max_pool2d_argmax/value"], out[f"{kind}/max_pool2d_argmax/index"] = v, i
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
