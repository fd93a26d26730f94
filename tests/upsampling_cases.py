"""Owl's upsampling2d known-answer tests (test/unit_upsampling_generic.ml),
read from tests/golden/owl_golden.json, and the replay of one case through
any stub provider (oracle, compiled reference, GPU)."""

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "owl_golden.json"
UP_CASES = json.loads(GOLDEN.read_text())["upsampling_cases"]


def up_id(c) -> str:
    return f"{c['fun']}-{c['op']}-{'x'.join(map(str, c['shape']))}-s{'x'.join(map(str, c['size']))}"


def run_up_case(nn, c, dtype=np.float32, conv=lambda a: a, back=lambda a: a):
    """(result, expected).  Forward: N.sequential input (from 0) against
    repeat; backward: input = ones, output' = sequential (from 0)."""
    shape, size = tuple(c["shape"]), list(c["size"])
    if c["op"] == "forward":
        x = np.arange(np.prod(shape), dtype=dtype).reshape(shape)
        expected = x.repeat(size[0], axis=1).repeat(size[1], axis=2)
        return back(nn.upsampling2d(conv(x), size)), expected
    inp = np.ones(shape, dtype=dtype)
    oshape = (shape[0], shape[1] * size[0], shape[2] * size[1], shape[3])
    outp = np.arange(np.prod(oshape), dtype=dtype).reshape(oshape)
    got = back(nn.upsampling2d_backward(conv(inp), size, conv(outp)))
    return got, np.asarray(c["expected"], dtype=dtype).reshape(shape)
