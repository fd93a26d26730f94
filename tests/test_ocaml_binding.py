"""The OCaml side of the drop-in (owl_gb300/ocaml/): the generated stubs and
externals are current, the stubs compile warning-free against OCaml's header
interface and link against libowlgpu, every external has the arity of Owl's
external of the same name, and a stub called the way OCaml calls it (tagged
ints, Bigarray descriptors) releases the runtime lock around the call and
raises Failure with the library's message on a bad argument.

The device-resident binding (owlgpu_device_stubs.c, owlgpu_device.ml): a
stub per device entry point with the C function's arity, custom blocks for
buffers and streams with finalisers and no compare / hash / serialise, and
its argument checks, all without a GPU."""

import ctypes
import json
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
OCAML = ROOT / "owl_gb300" / "ocaml"
# Owl's external arities, recorded from its sources by tests/golden/make_golden.py
OWL_EXTERNALS = ROOT / "tests" / "golden" / "owl_externals.json"

sys.path.insert(0, str(OCAML))


def build_stubs(out_dir: Path) -> Path:
    """Compile owlgpu_stubs.c with the test runtime stand-ins into a shared
    library linked against libowlgpu."""
    so = out_dir / "libowlgpu_ocaml_stubs.so"
    lib_dir = ROOT / "owl_gb300"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-O1", "-fPIC", "-shared",
           "-I", str(ROOT / "oracle" / "ref_shim"), "-I", str(ROOT / "include"),
           str(OCAML / "owlgpu_stubs.c"), str(OCAML / "owlgpu_device_stubs.c"),
           str(ROOT / "tests" / "ocaml_runtime_shim.c"),
           "-L", str(lib_dir), "-lowlgpu", f"-Wl,-rpath,{lib_dir}", "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return so


@pytest.fixture(scope="module")
def stubs(tmp_path_factory):
    from owl_gb300 import _lib

    _lib.lib()  # libowlgpu must exist
    L = ctypes.CDLL(str(build_stubs(tmp_path_factory.mktemp("ocaml"))))
    L.shim_last_failure.restype = ctypes.c_char_p
    return L


def test_generated_files_are_current():
    import make_stubs

    c, ml, n = make_stubs.render()
    assert (OCAML / "owlgpu_stubs.c").read_text() == c
    assert (OCAML / "owlgpu_externals.ml").read_text() == ml
    assert n == 152
    dc, dml, dn = make_stubs.render_device()
    assert (OCAML / "owlgpu_device_stubs.c").read_text() == dc
    assert (OCAML / "owlgpu_device.ml").read_text() == dml
    assert dn == 105


def test_every_entry_point_has_a_stub_pair(stubs):
    import make_stubs

    for name, params in make_stubs.host_entry_points():
        s = "owlgpu_stub_" + name[len("owl_"):]
        assert getattr(stubs, s + "_native") is not None
        assert getattr(stubs, s + "_bytecode") is not None


def _externals(text):
    """{name: number of arguments} of the `external` declarations in `text`."""
    out = {}
    for m in re.finditer(r"external\s+(\w+)\s*:(.*?)=\s*\"", text, flags=re.S):
        out[m.group(1).lstrip("_")] = m.group(2).count("->")
    return out


def test_externals_match_stub_arities():
    import make_stubs

    ours = _externals((OCAML / "owlgpu_externals.ml").read_text())
    for name, params in make_stubs.host_entry_points():
        assert ours[name] == len(params), name


def test_externals_have_owls_arities():
    ours = _externals((OCAML / "owlgpu_externals.ml").read_text())
    owl = json.loads(OWL_EXTERNALS.read_text())["arities"]
    shared = [n for n in ours if n in owl]
    # every Owl conv/pool/upsampling external has a drop-in of the same name
    # (Owl's argmax external is spelled maxpool_argmax_spatial, as here)
    assert len(shared) == len(owl), sorted(set(owl) - set(ours))
    for n in shared:
        assert ours[n] == owl[n], n


class _CamlBa(ctypes.Structure):
    # struct caml_ba_array as declared by the stand-in <caml/bigarray.h>
    _fields_ = [("data", ctypes.c_void_p), ("num_dims", ctypes.c_long),
                ("flags", ctypes.c_long), ("proxy", ctypes.c_void_p),
                ("dim", ctypes.c_long * 8)]


def _tag(n):
    return ctypes.c_long((int(n) << 1) | 1)


def test_bad_argument_raises_failure_around_a_released_lock(stubs):
    buf = (ctypes.c_float * 16)()
    ba = _CamlBa(ctypes.cast(buf, ctypes.c_void_p), 1, 0, None)
    p = ctypes.pointer(ba)
    args = [ctypes.cast(p, ctypes.c_void_p)] * 3
    # conv_spatial with row_stride -1: rejected before any GPU work
    ints = [1, 2, 2, 1, 1, 1, 2, 2, 1, -1, 1, 0, 1, 1]
    f = stubs.owlgpu_stub_float32_ndarray_conv_spatial_native
    f.restype = ctypes.c_long
    stubs.shim_reset()
    r = f(*args, *map(_tag, ints))
    assert r == 1  # Val_unit
    assert b"stride" in stubs.shim_last_failure()
    assert stubs.shim_entered() == 1 and stubs.shim_left() == 1
    # the bytecode entry forwards the same arguments
    argv = (ctypes.c_long * 17)(*[a.value for a in args], *[_tag(i).value for i in ints])
    stubs.shim_reset()
    stubs.owlgpu_stub_float32_ndarray_conv_spatial_bytecode(argv, 17)
    assert b"stride" in stubs.shim_last_failure()


# ---- the device-resident binding ---------------------------------------------


def test_every_device_entry_point_has_its_stubs_and_arity(stubs):
    import make_stubs

    ours = _externals((OCAML / "owlgpu_device.ml").read_text())
    eps = make_stubs.device_entry_points()
    assert len(eps) == 105
    for name, params in eps:
        short = name[len("owlgpu_"):]
        assert ours[short] == len(params), name
        stub = "owlgpu_dstub_" + short
        assert getattr(stubs, stub + "_native") is not None
        if len(params) > 5:
            assert getattr(stubs, stub + "_bytecode") is not None
    for fixed in ("stream_create", "stream_default", "stream_sync", "buf_create", "buf_bytes",
                  "buf_free", "buf_upload", "buf_download"):
        assert getattr(stubs, "owlgpu_dstub_" + fixed) is not None
    text = (OCAML / "owlgpu_device.ml").read_text()
    assert "type buf" in text and "type stream" in text
    # nullable pointer arguments are options: the dense layer's bias
    assert "-> buf option" in text


def test_custom_blocks_without_gpu(stubs):
    """The default-stream block: identifier, a finaliser that leaves the
    legacy stream alone; a negative buffer size raises Failure before any
    CUDA call."""
    f = stubs.owlgpu_dstub_stream_default
    f.restype = ctypes.c_void_p
    v = f(_tag(0))
    stubs.shim_custom_id.restype = ctypes.c_char_p
    assert stubs.shim_custom_id(ctypes.c_void_p(v)) == b"owlgpu.stream"
    stubs.shim_finalize(ctypes.c_void_p(v))
    stubs.shim_reset()
    b = stubs.owlgpu_dstub_buf_create
    b.restype = ctypes.c_void_p
    b(_tag(-8), ctypes.c_void_p(v))
    assert b"negative size" in stubs.shim_last_failure()
    src = (OCAML / "owlgpu_device_stubs.c").read_text()
    # no equality, hashing or serialisation of device memory
    for op in ("custom_compare_default", "custom_hash_default", "custom_serialize_default"):
        assert src.count(op) == 2
