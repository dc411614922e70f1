"""Recipe for oracle/_ref/: the reference's own code, compiled unchanged from
its sources, as checkers and baselines (test infrastructure only; nothing
under oracle/ is part of the product).

  oracle/_ref/libref_io.so            <- rawspec_rawutils.c (GUPPI RAW header
                                         cards, with the header-only WCSTools
                                         hget.h it includes) and
                                         rawspec_fbutils.c (SIGPROC headers)
  oracle/_ref/libreference_rawspec.so <- rawspec_gpu.cu: the reference's GPU
                                         spectrometer (cuFFT plans with load
                                         and store callbacks), built with nvcc
                                         for sm_103a and linked against the
                                         static cuFFT, as the reference's
                                         Makefile does (librawspec.so target)

Where the reference tree lies is given by RAWSPEC_REFERENCE, by default the
path named below.  A GPU machine without the reference tree builds the GPU
library from a staged copy of its three unmodified source files in
baseline/_ref/rawspec_src/ (git-ignored: never part of the repository),
written by stage() on a machine that has the tree.  The reference's file
callback (rawspec_file.c includes HDF5 headers that these machines do not
have) and its CLI are not built.
"""
from __future__ import annotations

import fcntl
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref"
LIB = OUT / "libref_io.so"
GPU_LIB = OUT / "libreference_rawspec.so"
REFERENCE = Path(os.environ.get("RAWSPEC_REFERENCE", "/root/reference"))
STAGE = ROOT / "baseline" / "_ref" / "rawspec_src"
SOURCES = ["rawspec_rawutils.c", "rawspec_fbutils.c"]
# rawspec_gpu.cu includes rawspec.h, cufft_error_name.h and the generated
# rawspec_version.h (written by the reference's gen_version.sh from git tags;
# here a one-line stand-in is generated into the build folder).
GPU_SOURCES = ["rawspec_gpu.cu", "rawspec.h", "cufft_error_name.h"]
# cuFFT 12 removed three enumerators that cufft_error_name.h still names;
# defining them keeps the file unchanged (values outside cufftResult's range).
CUFFT_COMPAT = ["-DCUFFT_INCOMPLETE_PARAMETER_LIST=0x7001", "-DCUFFT_PARSE_ERROR=0x7002",
                "-DCUFFT_LICENSE_ERROR=0x7003"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def available() -> bool:
    return all((REFERENCE / s).exists() for s in SOURCES)


def build(force: bool = False) -> Path | None:
    """Compiles libref_io.so if the reference sources are present; returns its
    path (None without the sources)."""
    if not available():
        return LIB if LIB.exists() else None
    srcs = [REFERENCE / s for s in SOURCES]
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in srcs):
        return LIB
    OUT.mkdir(exist_ok=True)
    with open(OUT / ".lock", "w") as fh:
        fcntl.flock(fh, fcntl.LOCK_EX)
        tmp = LIB.with_suffix(".so.tmp")
        # the sources are compiled as they are: old-style definitions and
        # void-pointer arithmetic in them need gnu C and no warnings
        cmd = [os.environ.get("CC", "gcc"), "-std=gnu11", "-O1", "-fPIC", "-shared", "-w",
               f"-I{REFERENCE}", "-o", str(tmp), *map(str, srcs), "-lm"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference io build failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
        fcntl.flock(fh, fcntl.LOCK_UN)
    return LIB


def gpu_source_dir() -> Path | None:
    """The reference tree if present, else the staged copy, else None."""
    for d in (REFERENCE, STAGE):
        if all((d / s).exists() for s in GPU_SOURCES):
            return d
    return None


def stage() -> Path | None:
    """Copies the unmodified GPU sources into the git-ignored staging folder,
    so that a GPU machine without the reference tree can build them."""
    if not all((REFERENCE / s).exists() for s in GPU_SOURCES):
        return STAGE if gpu_source_dir() == STAGE else None
    STAGE.mkdir(parents=True, exist_ok=True)
    for s in GPU_SOURCES:
        src, dst = REFERENCE / s, STAGE / s
        if not dst.exists() or dst.read_bytes() != src.read_bytes():
            shutil.copyfile(src, dst)
    return STAGE


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return None


def build_gpu(force: bool = False) -> Path | None:
    """Builds libreference_rawspec.so from the reference's rawspec_gpu.cu
    (separate compilation for the cuFFT callbacks, static cuFFT); returns its
    path, or None without sources or nvcc.  Raises if the compiler fails."""
    src = gpu_source_dir()
    nvcc = _nvcc()
    if src is None or nvcc is None:
        return GPU_LIB if GPU_LIB.exists() else None
    srcs = [src / s for s in GPU_SOURCES]
    if not force and GPU_LIB.exists() and all(s.stat().st_mtime <= GPU_LIB.stat().st_mtime for s in srcs):
        return GPU_LIB
    gen = OUT / "gen"
    gen.mkdir(parents=True, exist_ok=True)
    with open(OUT / ".lock_gpu", "w") as fh:
        fcntl.flock(fh, fcntl.LOCK_EX)
        try:
            (gen / "rawspec_version.h").write_text("#define RAWSPEC_VERSION reference-build\n")
            obj = gen / "rawspec_gpu.o"
            tmp = GPU_LIB.with_suffix(".so.tmp")
            steps = [
                [nvcc, *ARCH, "-O3", "-Xcompiler", "-fPIC", "-dc", f"-I{gen}", f"-I{src}", *CUFFT_COMPAT, "-o",
                 str(obj), "-c", str(src / "rawspec_gpu.cu")],
                [nvcc, "-shared", *ARCH, "-Xcompiler", "-fPIC", "-o", str(tmp), str(obj), "-lcufft_static",
                 "-lculibos"],
            ]
            for cmd in steps:
                res = subprocess.run(cmd, capture_output=True, text=True)
                if res.returncode != 0:
                    raise RuntimeError(f"reference GPU build failed ({' '.join(cmd)}):\n{res.stdout}\n{res.stderr}")
            os.replace(tmp, GPU_LIB)
        finally:
            fcntl.flock(fh, fcntl.LOCK_UN)
    return GPU_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(stage())
    if "--gpu" in sys.argv:
        print(build_gpu(force="--force" in sys.argv))
