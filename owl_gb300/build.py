"""Build libowlgpu.so (sm_103a) in-tree with nvcc.

Each ``csrc/*.cu`` file is compiled to an object in ``owl_gb300/_build`` in
parallel, then linked into ``owl_gb300/libowlgpu.so``.  Objects are rebuilt
only when a source or header is newer than the object, so a second build is a
no-op.  The library links the CUDA runtime statically and carries no torch
symbols: it is loadable from any host language through its C ABI
(``include/owlgpu.h``).
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libowlgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
              "--expt-extended-lambda"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libowlgpu")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(src: Path, obj: Path) -> tuple[Path, str]:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False) -> Path:
    """Compile every CUDA source for sm_103a and link libowlgpu.so."""
    BUILD.mkdir(exist_ok=True)
    deps = _headers()
    srcs = sorted(CSRC.glob("*.cu"))
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if _stale(o, s, deps)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for obj, err in ex.map(lambda so: _compile(*so), todo):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    if todo or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            # libcuda stubs may be absent on a build-only machine; the driver
            # API is reached through cudaGetDriverEntryPoint, so link without.
            cmd = cmd[:-1]
            r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_oracle(ref_root: str | os.PathLike | None = None) -> None:
    """Build the CPU oracle (test infrastructure) and, when an Owl source
    checkout is named (``ref_root``, else the OWL_REF_ROOT environment
    variable) and present, the compiled reference stubs used to pin it."""
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    ref_root = ref_root or os.environ.get("OWL_REF_ROOT")
    if ref_root and (Path(ref_root) / "src" / "owl" / "core").is_dir():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF_ROOT={ref_root}"],
                       check=False)


if __name__ == "__main__":
    print(build(verbose=True))
    build_oracle()
