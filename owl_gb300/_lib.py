"""ctypes binding of libowlgpu.so (the C ABI in include/owlgpu.h).

The prototypes are read from the header itself, so the Python side always
agrees with the declarations a C or OCaml caller compiles against.  Loading
fails loudly if the library has not been built: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import re
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
HEADER = ROOT / "include" / "owlgpu.h"
LIBPATH = PKG / "libowlgpu.so"

PREC = {"fp32": 0, "tf32": 1, "bf16": 2, "bf16x3": 3}


class OwlGpuError(RuntimeError):
    """A libowlgpu entry point returned a negative status."""

    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed with status {status}: {msg}")
        self.status = status


def parse_header(path: Path = HEADER) -> dict[str, tuple[str, list[tuple[str, str]]]]:
    """Return {name: (return type, [(c type, arg name), ...])} for every
    function declared in owlgpu.h."""
    text = path.read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    text = text.replace("OWLGPU_DEVICE_ARGS", ", int precision, void *stream")
    out = {}
    for m in re.finditer(r"\b(long long|int|uint64_t|const char \*)\s*(owl\w+)\s*\(([^;{]*)\)\s*;",
                         text):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        params = []
        a = " ".join(args.split())
        if a and a != "void":
            for p in a.split(","):
                p = p.strip()
                mm = re.match(r"(.*?)(\w+)$", p)
                params.append((mm.group(1).strip(), mm.group(2)))
        out[name] = (ret, params)
    return out


def _ctype(t: str):
    if "*" in t:
        return ctypes.c_void_p
    t = t.replace("const", "").strip()
    return {"long": ctypes.c_long, "long long": ctypes.c_longlong, "int": ctypes.c_int,
            "uint64_t": ctypes.c_uint64, "double": ctypes.c_double}[t]


RESTYPE = {"int": ctypes.c_int, "long long": ctypes.c_longlong, "uint64_t": ctypes.c_uint64,
           "const char *": ctypes.c_char_p}


def bind(L: ctypes.CDLL) -> ctypes.CDLL:
    """Set every declared entry point's argument and result types on L."""
    for name, (ret, params) in PROTOS.items():
        f = getattr(L, name)
        f.argtypes = [_ctype(t) for t, _ in params]
        f.restype = RESTYPE[ret]
    return L


_lock = threading.Lock()
_lib = None
PROTOS = parse_header()


def lib() -> ctypes.CDLL:
    """Load libowlgpu.so once, with prototypes from the header."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIBPATH.exists():
            raise OSError(
                f"{LIBPATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                f"g.build()'` (there is no CPU fallback)")
        _lib = bind(ctypes.CDLL(str(LIBPATH)))
        return _lib


def last_error() -> str:
    return lib().owlgpu_last_error().decode()


_entry: dict = {}  # name -> bound entry point (lib() and getattr once per name)


def call(name: str, *args) -> None:
    """Call an `int`-returning entry point and raise on a negative status."""
    f = _entry.get(name)
    if f is None:
        f = _entry[name] = getattr(lib(), name)
    rc = f(*args)
    if rc != 0:
        raise OwlGpuError(name, rc, last_error())


def launch_count() -> int:
    return int(lib().owlgpu_launch_count())


def set_precision(p: str | int) -> int:
    v = PREC[p] if isinstance(p, str) else int(p)
    rc = lib().owlgpu_set_precision(v)
    if rc < 0:
        raise OwlGpuError("owlgpu_set_precision", rc, last_error())
    return rc
