"""Generate the OCaml side of the drop-in from include/owlgpu.h.

Host drop-in (Owl's own externals, host Bigarrays).  For every host drop-in
entry point `owl_<kind>_ndarray_<op>` the header declares, this writes

* `owlgpu_stubs.c`: the OCaml C stub pair a maintainer links into Owl
  (`owlgpu_stub_<kind>_ndarray_<op>_native` and `_bytecode`).  It unpacks
  the Bigarray data pointers and OCaml ints as Owl's own stubs do
  (owl_ndarray_conv_impl.h:259-275), releases the runtime lock around the
  synchronous GPU call (the arrays are registered roots meanwhile), and turns
  a negative status into `Failure` where Owl's stub would `exit(1)`;
* `owlgpu_externals.ml`: the `external` declarations that bind Owl's names to
  those stubs, with the arities of Owl's externals (owl_ndarray_conv.ml,
  owl_ndarray_pool.ml, owl_ndarray_upsampling.ml).

Device resident (arrays that stay in GPU memory between calls, for Owl's
Graph and training loops, owl_neural_graph.ml:194-210).  For every
device-resident entry point `owlgpu_*` that takes a stream, this writes

* `owlgpu_device_stubs.c`: device buffers and streams held in OCaml custom
  blocks (`owlgpu.buf`: device pointer and byte size, freed by the block's
  finaliser on the legacy default stream, after all earlier work on every
  stream; `owlgpu.stream`: a CUDA stream, destroyed by its finaliser;
  neither compares, hashes nor serialises), Bigarray upload / download, and
  a stub pair per entry point taking buffers, ints, a precision and a
  stream.  The stubs only enqueue work: they neither allocate on the OCaml
  heap nor release the runtime lock, so their arguments need no roots;
  the copies and `stream_sync` release the lock while they wait.  A
  negative status raises `Failure`;
* `owlgpu_device.ml`: the abstract types `buf` and `stream` and the
  `external`s.  Pointer arguments the C entry point accepts as NULL (an
  absent bias, a loss adjoint of 1, an output not wanted) are `buf option`.

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
DC_OUT = HERE / "owlgpu_device_stubs.c"
DML_OUT = HERE / "owlgpu_device.ml"

# stream / buffer housekeeping: bound by the hand-written stubs below
HOUSEKEEPING = {"owlgpu_stream_create", "owlgpu_stream_destroy", "owlgpu_stream_synchronize",
                "owlgpu_device_alloc", "owlgpu_device_free", "owlgpu_copy_to_device",
                "owlgpu_copy_to_host"}
# pointer parameters the C entry points accept as NULL
NULLABLE = {"bias", "dloss", "pre_grad", "bias_grad", "loss", "dlogits"}


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


def device_entry_points():
    """The device-resident compute entry points: every `owlgpu_*` function
    with a `stream` parameter, except the stream / buffer housekeeping."""
    from owl_gb300._lib import parse_header

    protos = parse_header(ROOT / "include" / "owlgpu.h")
    return [(n, p) for n, (_, p) in protos.items()
            if n.startswith("owlgpu_") and n not in HOUSEKEEPING
            and any(a == "stream" for _, a in p)]


def _d_arg(t, a, v):
    """C expression for parameter (type t, name a) from OCaml value v."""
    if a == "stream":
        return f"Stream_val({v})"
    if "*" in t:
        base = t.replace("const", "").strip()
        if a in NULLABLE:
            return f"({base})(Is_block({v}) ? Buf_ptr(Field({v}, 0)) : NULL)"
        return f"({base})Buf_ptr({v})"
    if t == "double":
        return f"Double_val({v})"
    return f"Long_val({v})"


def _d_stub(name, params):
    stub = "owlgpu_dstub_" + name[len("owlgpu_"):]
    vs = [f"v{i}" for i in range(len(params))]
    lines = [_wrap(f"CAMLprim value {stub}_native(", [f"value {v}" for v in vs], ") {", 4)]
    args = [_d_arg(t, a, v) for (t, a), v in zip(params, vs)]
    lines.append(_wrap(f"  int rc = {name}(", args, ");", 6))
    lines.append("  if (rc != 0) caml_failwith(owlgpu_last_error());")
    lines.append("  return Val_unit;")
    lines.append("}")
    if len(params) <= 5:  # OCaml calls one stub with the values in both modes
        return "\n".join(lines)
    lines.append(_wrap(f"CAMLprim value {stub}_bytecode(", ["value *argv", "int argn"], ") {", 4))
    lines.append("  (void)argn;")
    lines.append(_wrap(f"  return {stub}_native(", [f"argv[{i}]" for i in range(len(params))],
                       ");", 6))
    lines.append("}")
    return "\n".join(lines)


def _d_external(name, params):
    stub = "owlgpu_dstub_" + name[len("owlgpu_"):]
    types = []
    for t, a in params:
        if a == "stream":
            types.append("stream")
        elif "*" in t:
            types.append("buf option" if a in NULLABLE else "buf")
        elif t == "double":
            types.append("float")
        else:
            types.append("int")
    names = (f'"{stub}_native"' if len(params) <= 5 else
             f'"{stub}_bytecode"\n    "{stub}_native"')
    return (f"external {name[len('owlgpu_'):]}\n  :  " + "\n  -> ".join(types + ["unit"]) +
            f"\n  = {names}")


DEVICE_C_HEAD = r"""/* owlgpu_device_stubs.c -- device-resident Owl arrays for OCaml: device
 * buffers and CUDA streams held in custom blocks, and the stubs of
 * libowlgpu's device-resident entry points (include/owlgpu.h).  Generated
 * by make_stubs.py; link with -lowlgpu. */
#include <caml/alloc.h>
#include <caml/bigarray.h>
#include <caml/custom.h>
#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>
#include <caml/signals.h>
#include <stddef.h>
#include <stdint.h>

#include "owlgpu.h"

/* ---- owlgpu.buf: device memory owned by the block ---------------------- */

typedef struct {
  void *ptr;
  uint64_t bytes;
} owlgpu_buf;

#define Buf_val(v) ((owlgpu_buf *)Data_custom_val(v))
#define Buf_ptr(v) (Buf_val(v)->ptr)

/* Released on the legacy default stream: after all earlier work on every
 * stream of the library (they are blocking streams), whichever stream the
 * buffer was used on. */
static void owlgpu_buf_finalize(value v) {
  owlgpu_buf *b = Buf_val(v);
  if (b->ptr) owlgpu_device_free(b->ptr, NULL);
  b->ptr = NULL;
  b->bytes = 0;
}

static struct custom_operations owlgpu_buf_ops = {
    "owlgpu.buf",           owlgpu_buf_finalize,         custom_compare_default,
    custom_hash_default,    custom_serialize_default,    custom_deserialize_default,
    custom_compare_ext_default, custom_fixed_length_default};

/* ---- owlgpu.stream: a CUDA stream owned by the block (NULL: the legacy
 * default stream, not destroyed) ----------------------------------------- */

typedef struct {
  void *s;
} owlgpu_stream;

#define Stream_val(v) (((owlgpu_stream *)Data_custom_val(v))->s)

static void owlgpu_stream_finalize(value v) {
  owlgpu_stream *st = (owlgpu_stream *)Data_custom_val(v);
  if (st->s) owlgpu_stream_destroy(st->s);
  st->s = NULL;
}

static struct custom_operations owlgpu_stream_ops = {
    "owlgpu.stream",        owlgpu_stream_finalize,      custom_compare_default,
    custom_hash_default,    custom_serialize_default,    custom_deserialize_default,
    custom_compare_ext_default, custom_fixed_length_default};

static value alloc_stream(void *s) {
  value v = caml_alloc_custom(&owlgpu_stream_ops, sizeof(owlgpu_stream), 0, 1);
  ((owlgpu_stream *)Data_custom_val(v))->s = s;
  return v;
}

CAMLprim value owlgpu_dstub_stream_create(value unit) {
  void *s = NULL;
  (void)unit;
  if (owlgpu_stream_create(&s) != 0) caml_failwith(owlgpu_last_error());
  return alloc_stream(s);
}

CAMLprim value owlgpu_dstub_stream_default(value unit) {
  (void)unit;
  return alloc_stream(NULL);
}

CAMLprim value owlgpu_dstub_stream_sync(value vs) {
  void *s = Stream_val(vs);
  int rc;
  caml_enter_blocking_section();
  rc = owlgpu_stream_synchronize(s);
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  return Val_unit;
}

/* buf_create bytes stream: uninitialised device memory, allocated in order
 * on `stream`. */
CAMLprim value owlgpu_dstub_buf_create(value vbytes, value vs) {
  CAMLparam2(vbytes, vs);
  CAMLlocal1(v);
  void *p = NULL;
  intnat n = Long_val(vbytes);
  if (n < 0) caml_failwith("owlgpu buf_create: negative size");
  if (owlgpu_device_alloc(&p, (uint64_t)n, Stream_val(vs)) != 0)
    caml_failwith(owlgpu_last_error());
  v = caml_alloc_custom(&owlgpu_buf_ops, sizeof(owlgpu_buf), 0, 1);
  Buf_val(v)->ptr = p;
  Buf_val(v)->bytes = (uint64_t)n;
  CAMLreturn(v);
}

CAMLprim value owlgpu_dstub_buf_bytes(value vb) { return Val_long((intnat)Buf_val(vb)->bytes); }

/* buf_free b: release now (the finaliser then has nothing to do); later
 * calls on b see a buffer of 0 bytes. */
CAMLprim value owlgpu_dstub_buf_free(value vb) {
  owlgpu_buf_finalize(vb);
  return Val_unit;
}

/* buf_upload b a stream / buf_download b a stream: copy the Bigarray's
 * bytes into / out of the buffer; they return when the bytes have arrived. */
static value copy_ba(value vb, value va, value vs, int to_device) {
  CAMLparam3(vb, va, vs);
  owlgpu_buf *b = Buf_val(vb);
  void *host = Caml_ba_data_val(va);
  uint64_t n = (uint64_t)caml_ba_byte_size(Caml_ba_array_val(va));
  void *dev = b->ptr, *s = Stream_val(vs);
  int rc;
  if (n > b->bytes) caml_failwith("owlgpu buf copy: the array is larger than the buffer");
  caml_enter_blocking_section();
  rc = to_device ? owlgpu_copy_to_device(dev, host, n, s) : owlgpu_copy_to_host(host, dev, n, s);
  caml_leave_blocking_section();
  if (rc != 0) caml_failwith(owlgpu_last_error());
  CAMLreturn(Val_unit);
}

CAMLprim value owlgpu_dstub_buf_upload(value vb, value va, value vs) {
  return copy_ba(vb, va, vs, 1);
}

CAMLprim value owlgpu_dstub_buf_download(value vb, value va, value vs) {
  return copy_ba(vb, va, vs, 0);
}

/* ---- device-resident entry points ------------------------------------ */
"""

DEVICE_ML_HEAD = """(* owlgpu_device.ml -- device-resident Owl arrays for OCaml: libowlgpu's
   device-resident entry points over GPU buffers held in custom blocks.
   Generated by make_stubs.py.

   A [buf] is device memory, freed by its finaliser (or [buf_free]) after
   all earlier work on every stream.  A [stream] orders the calls made on
   it; the entry points only enqueue work, [stream_sync] waits for it.
   Shapes, strides and padding follow Owl's stub arguments, as for the host
   externals; each buffer must hold the bytes its argument covers. *)

type buf
type stream

external stream_create : unit -> stream = "owlgpu_dstub_stream_create"
external stream_default : unit -> stream = "owlgpu_dstub_stream_default"
external stream_sync : stream -> unit = "owlgpu_dstub_stream_sync"
external buf_create : int -> stream -> buf = "owlgpu_dstub_buf_create"
external buf_bytes : buf -> int = "owlgpu_dstub_buf_bytes"
external buf_free : buf -> unit = "owlgpu_dstub_buf_free"
external buf_upload
  :  buf -> ('a, 'b, Bigarray.c_layout) Bigarray.Genarray.t -> stream -> unit
  = "owlgpu_dstub_buf_upload"
external buf_download
  :  buf -> ('a, 'b, Bigarray.c_layout) Bigarray.Genarray.t -> stream -> unit
  = "owlgpu_dstub_buf_download"
"""


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


def render_device():
    eps = device_entry_points()
    c = [DEVICE_C_HEAD] + [_d_stub(n, p) + "\n" for n, p in eps]
    ml = [DEVICE_ML_HEAD] + [_d_external(n, p) + "\n" for n, p in eps]
    return "\n".join(c), "\n".join(ml), len(eps)


def main() -> None:
    c, ml, n = render()
    C_OUT.write_text(c)
    ML_OUT.write_text(ml)
    dc, dml, dn = render_device()
    DC_OUT.write_text(dc)
    DML_OUT.write_text(dml)
    print(f"wrote {C_OUT.name} and {ML_OUT.name}: {n} host entry points; "
          f"{DC_OUT.name} and {DML_OUT.name}: {dn} device entry points")


if __name__ == "__main__":
    main()
