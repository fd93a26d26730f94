"""Extract Owl's conv/pool known-answer tests into tests/golden/owl_golden.json.

Run where the Owl sources are checked out, naming the checkout with --ref
or the OWL_REF_ROOT environment variable:

    python tests/golden/make_golden.py --ref <owl checkout>

It also records, in tests/golden/owl_externals.json, the number of arguments
of every `external` in Owl's conv, pool and upsampling bindings
(src/owl/core/owl_ndarray_{conv,pool,upsampling}.ml), which the OCaml
binding test checks the generated externals against.

It reads the alcotest files listed in FILES, finds every
``let funNN () = ... verify_value <helper> <shapes..> PAD expected`` (or
``test_forward ...``) case, and records the helper name, its array
arguments, labelled arguments (``~stride``, ``~seq``), the padding and the
expected values exactly as written in the reference test.  HELPERS restates,
for each test helper, how that test builds its inputs (sequential from 1,
sequential from 0, ones, normalised) and which NN function it calls; the
parity tests replay each case through ``owl_gb300.dense.NN`` with any stub
provider and compare with Owl's own tolerance (sum |a - b| < 5e-4).
"""

from __future__ import annotations

import argparse
import json
import os
import re
from pathlib import Path

FILES = [
    "unit_conv2d_generic.ml", "unit_conv3d_generic.ml", "unit_dilated_conv2d.ml",
    "unit_dilated_conv3d.ml", "unit_transpose_conv2d.ml", "unit_transpose_conv3d.ml",
    "unit_pool2d_generic.ml", "unit_pool3d_generic.ml",
]

# helper -> (NN function, input recipe, kernel recipe, output' recipe)
# recipes: "seq1" = sequential ~a:1., "seq0" = sequential ~a:0., "ones",
# "seq1n" = sequential ~a:1. divided by its element count, "seqk" = ones
# or sequential depending on ~seq, None = not used.
HELPERS = {
    # test/unit_conv2d_generic.ml:16-46
    "test_conv2d": ("conv2d", "seq1", "seq1", None),
    "test_conv2d_back_input": ("conv2d_backward_input", "seq1", "seq1", "seq1"),
    "test_conv2d_back_kernel": ("conv2d_backward_kernel", "seq1", "seq1", "seq1"),
    "test_conv2d_back_kernel_02": ("conv2d_backward_kernel", "ones", "ones", "ones"),
    # test/unit_conv3d_generic.ml:16-41
    "test_conv3d": ("conv3d", "seq1n", "seq1n", None),
    "test_conv3d_back_input": ("conv3d_backward_input", "seq1", "seq1", "seq0"),
    "test_conv3d_back_kernel": ("conv3d_backward_kernel", "seq1", "seq1", "seq0"),
    # test/unit_dilated_conv2d.ml:14-35 (third array argument is the rate)
    "test_dilated_conv2d": ("dilated_conv2d", "seq1", "seq1", None),
    "test_dilated_conv2d_bi": ("dilated_conv2d_backward_input", "seq1", "seq1", "seq1"),
    "test_dilated_conv2d_bk": ("dilated_conv2d_backward_kernel", "seq1", "seq1", "seq1"),
    # test/unit_dilated_conv3d.ml:14-35
    "test_dilated_conv3d": ("dilated_conv3d", "seq1", "seq1", None),
    "test_dilated_conv3d_bi": ("dilated_conv3d_backward_input", "seq1", "seq1", "seq0"),
    "test_dilated_conv3d_bk": ("dilated_conv3d_backward_kernel", "seq1", "seq1", "seq1"),
    # test/unit_transpose_conv2d.ml:14-38 and unit_transpose_conv3d.ml:14-39
    "compute_trans_conv2d": ("transpose_conv2d", "ones", "seqk", None),
    "compute_trans_conv2d_bi": ("transpose_conv2d_backward_input", "ones", "seqk", "ones"),
    "compute_trans_conv2d_bk": ("transpose_conv2d_backward_kernel", "ones", "ones", "seqk"),
    "compute_trans_conv3d": ("transpose_conv3d", "ones", "seqk", None),
    "compute_trans_conv3d_bi": ("transpose_conv3d_backward_input", "ones", "seqk", "ones"),
    "compute_trans_conv3d_bk": ("transpose_conv3d_backward_kernel", "ones", "ones", "seqk"),
    # test/unit_pool2d_generic.ml:16-39 and unit_pool3d_generic.ml:16-39
    "test_maxpool2d": ("max_pool2d", "seq1", None, None),
    "test_avgpool2d": ("avg_pool2d", "seq1", None, None),
    "test_maxpool2d_back": ("max_pool2d_backward", "seq1", None, "seq1"),
    "test_avgpool2d_back": ("avg_pool2d_backward", "seq1", None, "seq1"),
    "test_maxpool3d": ("max_pool3d", "seq1", None, None),
    "test_avgpool3d": ("avg_pool3d", "seq1", None, None),
    "test_maxpool3d_back": ("max_pool3d_backward", "seq1", None, "seq1"),
    "test_avgpool3d_back": ("avg_pool3d_backward", "seq1", None, "seq1"),
}

ARR = r"\[\|(.*?)\|\]"


def _nums(s: str) -> list[float]:
    return [float(t) for t in re.split(r"[;\s]+", s.strip()) if t]


def _strip_comments(text: str) -> list[tuple[int, str]]:
    """Return (position, comment text) pairs; comments are kept in the text."""
    return [(m.start(), m.group(1).strip()) for m in re.finditer(r"\(\*(.*?)\*\)", text, re.S)]


def parse_file(path: Path) -> list[dict]:
    text = path.read_text()
    comments = _strip_comments(text)
    cases = []
    for mod in re.finditer(r"module (To_test_\w+) = struct(.*?)\n\s*end\b", text, re.S):
        mname, body = mod.group(1), mod.group(2)
        base = mod.start(2)
        starts = [m for m in re.finditer(r"let (fun\d+) \(\) =", body)]
        for i, m in enumerate(starts):
            end = starts[i + 1].start() if i + 1 < len(starts) else len(body)
            blk = body[m.end():end]
            blk_nc = re.sub(r"\(\*.*?\*\)", " ", blk, flags=re.S)
            title = ""
            for pos, c in comments:
                if pos < base + m.start():
                    title = c
            rec = {"file": path.name, "module": mname, "fun": m.group(1), "title": title}
            ex = re.search(r"let expected\s*=\s*" + ARR, blk_nc, re.S)
            call = re.search(r"\b(verify_value|test_forward)\b(.*)", blk_nc, re.S)
            if not call:
                continue
            head, rest = call.group(1), call.group(2)
            labels = {}
            for lm in re.finditer(r"~(\w+):(" + ARR + r"|\w+)", rest, re.S):
                val = lm.group(2)
                labels[lm.group(1)] = _nums(lm.group(3)) if val.startswith("[|") else val
            rest_nl = re.sub(r"~\w+:(" + ARR + r"|\w+)", " ", rest, flags=re.S)
            if head == "test_forward":
                helper = "test_forward"
            else:
                hm = re.search(r"\b((?:test|compute)_\w+)", rest_nl)
                helper = hm.group(1)
            arrays = [_nums(a) for a in re.findall(ARR, rest_nl, re.S)]
            pad = re.search(r"\b(SAME|VALID)\b", rest_nl).group(1)
            rec.update(head=head, helper=helper, labels=labels, pad=pad)
            if head == "test_forward":
                rec.update(args=[[int(v) for v in a] for a in arrays[:3]], magic=arrays[3])
            else:
                rec.update(args=[[int(v) for v in a] for a in arrays],
                           expected=_nums(ex.group(1)) if ex else None)
                if rec["expected"] is None:
                    continue
                if helper not in HELPERS:
                    raise SystemExit(f"{path.name}:{mname}.{m.group(1)}: unknown helper {helper}")
            cases.append(rec)
    return cases


def parse_upsampling(path: Path) -> list[dict]:
    """test/unit_upsampling_generic.ml: forward cases compare upsampling2d
    with ``repeat`` (``test_upsampling2d_forward shape size``); backward
    cases run upsampling2d_backward with input = ones and output' =
    sequential (from 0) and list the expected input gradient
    (``verify_value shape size expected``)."""
    text = re.sub(r"\(\*.*?\*\)", " ", path.read_text(), flags=re.S)
    mod = re.search(r"module To_test_upsampling2d = struct(.*?)\n\s*end\b", text, re.S)
    body = mod.group(1)
    starts = list(re.finditer(r"let (fun\d+) \(\) =", body))
    cases = []
    for i, m in enumerate(starts):
        blk = body[m.end():starts[i + 1].start() if i + 1 < len(starts) else len(body)]
        fwd = re.search(r"test_upsampling2d_forward\s*" + ARR + r"\s*" + ARR, blk, re.S)
        if fwd:
            cases.append({"file": path.name, "fun": m.group(1), "op": "forward",
                          "shape": [int(v) for v in _nums(fwd.group(1))],
                          "size": [int(v) for v in _nums(fwd.group(2))]})
            continue
        ex = re.search(r"let expected\s*=\s*" + ARR, blk, re.S)
        vv = re.search(r"verify_value\s*" + ARR + r"\s*" + ARR, blk, re.S)
        if ex and vv:
            cases.append({"file": path.name, "fun": m.group(1), "op": "backward",
                          "shape": [int(v) for v in _nums(vv.group(1))],
                          "size": [int(v) for v in _nums(vv.group(2))],
                          "expected": _nums(ex.group(1))})
    return cases


EXTERNAL_FILES = ["owl_ndarray_conv.ml", "owl_ndarray_pool.ml", "owl_ndarray_upsampling.ml"]


def external_arities(core: Path) -> dict:
    """{external name: number of arguments} over Owl's conv/pool/upsampling
    bindings (a leading underscore dropped, as the generated externals do)."""
    out = {}
    for f in EXTERNAL_FILES:
        text = (core / f).read_text()
        for m in re.finditer(r"external\s+(\w+)\s*:(.*?)=\s*\"", text, flags=re.S):
            out[m.group(1).lstrip("_")] = m.group(2).count("->")
    return dict(sorted(out.items()))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("OWL_REF_ROOT"),
                    help="Owl source checkout (default: $OWL_REF_ROOT)")
    ap.add_argument("--out", default=str(Path(__file__).with_name("owl_golden.json")))
    a = ap.parse_args()
    if not a.ref:
        ap.error("name the Owl checkout with --ref or OWL_REF_ROOT")
    ext = external_arities(Path(a.ref) / "src" / "owl" / "core")
    ext_out = Path(a.out).with_name("owl_externals.json")
    ext_out.write_text(json.dumps({"source": "src/owl/core/" + ",".join(EXTERNAL_FILES),
                                   "arities": ext}, indent=0) + "\n")
    tdir = Path(a.ref) / "test"
    cases = []
    for f in FILES:
        cases += parse_file(tdir / f)
    up = parse_upsampling(tdir / "unit_upsampling_generic.ml")
    doc = {"source": "owl test/ alcotest files", "files": FILES,
           "tolerance_sum_abs": 5e-4, "helpers": HELPERS, "cases": cases}
    lines = ",\n".join(json.dumps(c, separators=(",", ":")) for c in cases)
    up_lines = ",\n".join(json.dumps(c, separators=(",", ":")) for c in up)
    head = json.dumps({k: v for k, v in doc.items() if k != "cases"}, separators=(",", ":"))
    Path(a.out).write_text(head[:-1] + ',"cases":[\n' + lines + '\n],"upsampling_cases":[\n' +
                           up_lines + "\n]}\n")
    print(f"{len(cases)} cases + {len(up)} upsampling cases -> {a.out}; "
          f"{len(ext)} external arities -> {ext_out}")


if __name__ == "__main__":
    main()
