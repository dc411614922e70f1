"""Recipe for oracle/_ref/: the reference's own host-side C for the callers
of the spectrometer path, compiled unchanged from its sources where they lie
(test infrastructure only; nothing under oracle/ is part of the product).

  oracle/_ref/libref_io.so  <- rawspec_rawutils.c (GUPPI RAW header cards,
                               with the header-only WCSTools hget.h it
                               includes) and rawspec_fbutils.c (SIGPROC
                               filterbank headers)

The reference's GPU code and its file callback (rawspec_file.c, which
includes HDF5 headers that this machine does not have) are not built.  The
library is built only where the reference sources exist; tests that use it
are skipped elsewhere.
"""
from __future__ import annotations

import fcntl
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_io.so"
REFERENCE = Path(os.environ.get("RAWSPEC_REFERENCE", "/root/reference"))
SOURCES = ["rawspec_rawutils.c", "rawspec_fbutils.c"]


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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
