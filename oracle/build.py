"""Build recipe of the CPU restatements under oracle/ (test infrastructure).

Produces oracle/_build/liboracle.so from rawspec_oracle.c (FP64 checker) and
rawspec_cpu.c (FP32 OpenMP chain used as the CPU baseline) with gcc.
"""
from __future__ import annotations

import fcntl
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRCS = [HERE / "rawspec_oracle.c", HERE / "rawspec_cpu.c"]
DEPS = SRCS + [HERE / "rawspec_oracle.h", Path(__file__)]


def _fresh() -> bool:
    return LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in DEPS)


def build(force: bool = False) -> Path:
    if not force and _fresh():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with open(BUILD / ".lock", "w") as fh:  # one builder at a time; the others find it fresh
        fcntl.flock(fh, fcntl.LOCK_EX)
        try:
            if force or not _fresh():
                _build()
        finally:
            fcntl.flock(fh, fcntl.LOCK_UN)
    return LIB


# The FP64 restatement at -O2; the FP32 CPU chain at -O3 (its FFT loops
# vectorise with the base instruction set of either host; no -march)
OPT = {"rawspec_oracle.c": "-O2", "rawspec_cpu.c": "-O3"}


def _build() -> None:
    cc = os.environ.get("CC", "gcc")
    objs = []
    for src in SRCS:
        obj = BUILD / (src.stem + ".o")
        cmd = [cc, OPT[src.name], "-fPIC", "-fopenmp", "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
        objs.append(str(obj))
    tmp = LIB.with_suffix(".so.tmp")
    res = subprocess.run([cc, "-shared", "-fopenmp", "-o", str(tmp), *objs, "-lm"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
