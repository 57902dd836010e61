"""
Build the CUDA library ``_lib/libtad_dftd4_gb300.so`` in the source tree.

Every ``csrc/*.cu`` file is compiled for sm_103a (GB300) in parallel and
linked into one shared library exporting the C ABI of
``include/tad_dftd4_gb300.h``.  No CMake, no torch extension machinery.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = REPO / "include"
OUT_DIR = PKG / "_lib"
LIB_NAME = "libtad_dftd4_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    lib = lib_path()
    if not lib.exists():
        return False
    mtime = lib.stat().st_mtime
    return all(p.stat().st_mtime <= mtime for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if needed) and return the path of the shared library."""
    if not force and up_to_date():
        return lib_path()
    OUT_DIR.mkdir(exist_ok=True)
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    exe = nvcc()
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as pool:
        objs = list(pool.map(compile_one, _sources()))
    tmp = lib_path().with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build(force=True, verbose=True))
