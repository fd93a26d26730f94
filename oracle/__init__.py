"""CPU oracle for the Owl conv/pool path -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker (or the timed CPU
arm).  The product library never calls it.

Two stub providers, both usable with ``owl_gb300.dense.NN``:

* ``OracleBackend`` -- ``liboracle.so`` built from ``owl_oracle.c``, a C
  restatement of Owl's conv (im2col + BLAS GEMM) and pool (exact loops)
  stubs.  GEMMs go to the scipy/numpy-bundled OpenBLAS when one is found,
  matching Owl's use of ``cblas_?gemm``.
* ``RefBackend`` -- ``_ref/libowlref.so``: Owl's own unmodified C stubs
  compiled from the reference sources (see ``Makefile``).  Available only
  where the reference checkout exists; it pins the restatement.
"""

from __future__ import annotations

import ctypes
import glob
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REFLIB = HERE / "_ref" / "libowlref.so"

# Canonical op name (the OCaml external suffix used by the CUDA ABI) ->
# the suffix of Owl's C stub symbol.
STUB_NAME = {"maxpool_argmax_spatial": "maxpool_spatial_arg"}

_oracle = None
_ref = None


def _find_openblas():
    """Locate an OpenBLAS shipped with scipy (LP64) or numpy (ILP64)."""
    cands = []
    try:
        import scipy

        cands += [(p, False) for p in
                  glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs",
                                         "libscipy_openblas-*.so"))]
    except Exception:
        pass
    cands += [(p, True) for p in
              glob.glob(os.path.join(os.path.dirname(np.__file__), "..", "numpy.libs",
                                     "libscipy_openblas64_*.so"))]
    for path, ilp64 in cands:
        try:
            L = ctypes.CDLL(path)
            suf = "64_" if ilp64 else ""
            s = getattr(L, f"scipy_cblas_sgemm{suf}")
            d = getattr(L, f"scipy_cblas_dgemm{suf}")
            c = getattr(L, f"scipy_cblas_cgemm{suf}", None)
            z = getattr(L, f"scipy_cblas_zgemm{suf}", None)
            setter = getattr(L, f"scipy_openblas_set_num_threads{suf}", None)
            return L, s, d, c, z, ilp64, setter, path
        except (OSError, AttributeError):
            continue
    return None


_blas_info = {}


def load(threads: int | None = None) -> ctypes.CDLL:
    """Build (if needed) and load liboracle.so with a BLAS registered."""
    global _oracle
    if _oracle is None:
        newest = max((HERE / f).stat().st_mtime for f in ("owl_oracle.c", "oracle_impl.h"))
        if not LIB.exists() or LIB.stat().st_mtime < newest:
            subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
        L = ctypes.CDLL(str(LIB))
        L.oracle_set_blas.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_set_blas_complex.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        found = _find_openblas()
        if found:
            B, s, d, c, z, ilp64, setter, path = found
            L.oracle_set_blas(ctypes.cast(s, ctypes.c_void_p), ctypes.cast(d, ctypes.c_void_p),
                              1 if ilp64 else 0)
            if c is not None and z is not None:
                L.oracle_set_blas_complex(ctypes.cast(c, ctypes.c_void_p),
                                          ctypes.cast(z, ctypes.c_void_p), 1 if ilp64 else 0)
            _blas_info.update(lib=B, setter=setter, path=path, ilp64=ilp64)
        _oracle = L
    if threads is not None:
        set_threads(threads)
    return _oracle


def set_threads(n: int) -> None:
    s = _blas_info.get("setter")
    if s is not None:
        s.argtypes = [ctypes.c_int]
        s(int(n))


def blas_path() -> str | None:
    load()
    return _blas_info.get("path")


def _arg(a):
    if isinstance(a, (int, np.integer)):
        return ctypes.c_long(int(a))
    assert isinstance(a, np.ndarray) and a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


class _NumpyBackend:
    def empty(self, like, shape, dtype=None):
        return np.empty(tuple(shape), dtype=dtype or like.dtype)

    def shape(self, a):
        return tuple(a.shape)

    def reshape(self, a, shape):
        return a.reshape(shape)


class OracleBackend(_NumpyBackend):
    """The C restatement (owl_oracle.c)."""

    name = "oracle"

    def __init__(self, threads: int | None = None):
        self.L = load(threads)

    def stub(self, kind, op, *args):
        fn = getattr(self.L, f"oracle_{kind}_ndarray_{STUB_NAME.get(op, op)}")
        fn.restype = ctypes.c_int
        rc = fn(*[_arg(a) for a in args])
        if rc != 0:
            raise RuntimeError(f"oracle {op} failed ({rc})")


def ref_available() -> bool:
    return REFLIB.exists()


class _CamlBa(ctypes.Structure):
    # Layout of struct caml_ba_array in oracle/ref_shim/caml/bigarray.h.
    _fields_ = [("data", ctypes.c_void_p), ("num_dims", ctypes.c_long),
                ("flags", ctypes.c_long), ("proxy", ctypes.c_void_p),
                ("dim", ctypes.c_long * 8)]


class RefBackend(_NumpyBackend):
    """Owl's own C stubs compiled unmodified (only where the reference
    sources exist).  Arguments are marshalled the way OCaml passes them:
    Bigarrays as pointers to their descriptor, ints tagged (n << 1 | 1)."""

    name = "ref"

    def __init__(self):
        global _ref
        if _ref is None:
            if not REFLIB.exists():
                raise OSError("compiled reference stubs not built (make -C oracle ref)")
            _ref = ctypes.CDLL(str(REFLIB))
        self.L = _ref

    def stub(self, kind, op, *args):
        fn = getattr(self.L, f"stub_{kind}_ndarray_{STUB_NAME.get(op, op)}_native")
        keep = []
        cargs = []
        for a in args:
            if isinstance(a, (int, np.integer)):
                cargs.append(ctypes.c_long((int(a) << 1) | 1))
            else:
                ba = _CamlBa()
                ba.data = a.ctypes.data
                ba.num_dims = a.ndim
                for i, d in enumerate(a.shape):
                    ba.dim[i] = d
                keep.append(ba)
                cargs.append(ctypes.c_void_p(ctypes.addressof(ba)))
        fn.restype = ctypes.c_long
        fn(*cargs)
