"""Generate the OCaml side of the drop-in from include/owlgpu.h.

For every host drop-in entry point `owl_<kind>_ndarray_<op>` the header
declares, this writes

* `owlgpu_stubs.c`: the OCaml C stub pair a maintainer links into Owl
  (`owlgpu_stub_<kind>_ndarray_<op>_native` and `_bytecode`).  It unpacks
  the Bigarray data pointers and OCaml ints as Owl's own stubs do
  (owl_ndarray_conv_impl.h:259-275), releases the runtime lock around the
  synchronous GPU call (the arrays are registered roots meanwhile), and turns
  a negative status into `Failure` where Owl's stub would `exit(1)`;
* `owlgpu_externals.ml`: the `external` declarations that bind Owl's names to
  those stubs, with the arities of Owl's externals (owl_ndarray_conv.ml,
  owl_ndarray_pool.ml, owl_ndarray_upsampling.ml).

    python owl_gb300/ocaml/make_stubs.py
"""

from __future__ import annotations

import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

C_OUT = HERE / "owlgpu_stubs.c"
ML_OUT = HERE / "owlgpu_externals.ml"


def host_entry_points():
    from owl_gb300._lib import parse_header

    protos = parse_header(ROOT / "include" / "owlgpu.h")
    return [(n, p) for n, (_, p) in protos.items() if n.startswith("owl_")]


def _c_stub(name, params):
    stub = "owlgpu_stub_" + name[len("owl_"):]
    vs = [f"v{i}" for i in range(len(params))]
    arrays = [(t, a, v) for (t, a), v in zip(params, vs) if "*" in t]
    lines = [_wrap(f"CAMLprim value {stub}_native(", [f"value {v}" for v in vs], ") {", 4)]
    lines.append(f"  CAMLparam{len(arrays)}({', '.join(v for _, _, v in arrays)});")
    for t, a, v in arrays:
        base = t.replace("const", "").strip()
        lines.append(f"  {base}{a} = ({base})Caml_ba_data_val({v});")
    args = [a if "*" in t else f"Long_val({v})" for (t, a), v in zip(params, vs)]
    lines.append("  int rc;")
    lines.append("  caml_enter_blocking_section();")
    lines.append(_wrap(f"  rc = {name}(", args, ");", 6))
    lines.append("  caml_leave_blocking_section();")
    lines.append("  if (rc != 0) caml_failwith(owlgpu_last_error());")
    lines.append("  CAMLreturn(Val_unit);")
    lines.append("}")
    lines.append(_wrap(f"CAMLprim value {stub}_bytecode(", ["value *argv", "int argn"], ") {", 4))
    lines.append("  (void)argn;")
    lines.append(_wrap(f"  return {stub}_native(", [f"argv[{i}]" for i in range(len(params))],
                       ");", 6))
    lines.append("}")
    return "\n".join(lines)


def _ml_external(name, params):
    stub = "owlgpu_stub_" + name[len("owl_"):]
    types = []
    for t, a in params:
        if "int64_t" in t:
            types.append("(int64, Bigarray.int64_elt) owl_arr")
        elif "*" in t:
            types.append("('a, 'b) owl_arr")
        else:
            types.append("int")
    return (f"external {name}\n  :  " + "\n  -> ".join(types + ["unit"]) +
            f'\n  = "{stub}_bytecode"\n    "{stub}_native"')


def _wrap(head, items, tail, indent, width=92):
    """head + items joined by ", " + tail, broken between items so that no
    line passes `width`; continuation lines start `indent` spaces in."""
    out, cur = [], head
    for i, it in enumerate(items):
        tok = it + (", " if i < len(items) - 1 else tail)
        if len(cur) + len(tok.rstrip()) > width and cur.strip():
            out.append(cur.rstrip())
            cur = " " * indent
        cur += tok
    out.append(cur.rstrip())
    return "\n".join(out)


def render():
    eps = host_entry_points()
    c = ["/* owlgpu_stubs.c -- OCaml C stubs binding Owl's conv / pool / upsampling",
         " * externals to libowlgpu's host drop-in entry points (include/owlgpu.h).",
         " * Generated by make_stubs.py; link with -lowlgpu. */",
         "#include <caml/bigarray.h>",
         "#include <caml/fail.h>",
         "#include <caml/memory.h>",
         "#include <caml/mlvalues.h>",
         "#include <caml/signals.h>",
         "#include <stdint.h>",
         "",
         '#include "owlgpu.h"', ""]
    c += [_c_stub(n, p) + "\n" for n, p in eps]
    ml = ["(* owlgpu_externals.ml -- Owl's conv / pool / upsampling externals bound to",
          "   libowlgpu through owlgpu_stubs.c.  Generated by make_stubs.py. *)",
          "",
          "open Owl_core_types", ""]
    ml += [_ml_external(n, p) + "\n" for n, p in eps]
    return "\n".join(c), "\n".join(ml), len(eps)


def main() -> None:
    c, ml, n = render()
    C_OUT.write_text(c)
    ML_OUT.write_text(ml)
    print(f"wrote {C_OUT.name} and {ML_OUT.name}: {n} entry points")


if __name__ == "__main__":
    main()
