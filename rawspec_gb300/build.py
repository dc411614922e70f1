"""Build recipe of the native library (librawspec.so) for sm_103a.

The library is built in-tree (rawspec_gb300/lib/librawspec.so): every .cu
file under rawspec_gb300/csrc is compiled to an object in parallel, then the
objects are linked into one shared library with the CUDA runtime linked
statically, so the library depends on the driver only.
"""
from __future__ import annotations

import concurrent.futures as cf
import contextlib
import fcntl
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "librawspec.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--split-compile=0", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librawspec")


def _sources() -> list[Path]:
    """CUDA translation units (nvcc) and host-only C files (the C compiler)."""
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.c"))


def _deps() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.c")) + list(CSRC.glob("*.cuh")) +
                  list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")) + [Path(__file__)])


def up_to_date() -> bool:
    if not LIB.exists() or _extra_flags():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _extra_flags() -> list[str]:
    """Tuning definitions from RAWSPEC_NVCC_FLAGS (e.g. "-DRSG_FUSED_TP_MINB=2")."""
    return os.environ.get("RAWSPEC_NVCC_FLAGS", "").split()


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.stem + src.suffix.replace(".", "_") + ".o")
    if src.suffix == ".c":
        cuda_inc = Path(nvcc()).resolve().parent.parent / "include"  # the runtime API header
        cmd = [os.environ.get("CC", "gcc"), "-std=gnu11", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall",
               f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda_inc}", "-c", str(src), "-o", str(obj)]
    else:
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *_extra_flags(), "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


@contextlib.contextmanager
def _build_lock():
    """Serialises builders (e.g. the ranks of a multi-process run that all
    call build()): the second one waits, then finds the library up to date."""
    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as fh:
        fcntl.flock(fh, fcntl.LOCK_EX)
        try:
            yield
        finally:
            fcntl.flock(fh, fcntl.LOCK_UN)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles librawspec.so if any source is newer than it; returns its path."""
    if not force and up_to_date():
        return LIB
    with _build_lock():
        if not force and up_to_date():
            return LIB
        return _build(verbose)


def _build(verbose: bool) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static", "-lpthread", "-ldl", "-lrt"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
