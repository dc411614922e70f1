"""Writes abi_layout.json: the member offsets/sizes and constants of the
reference's rawspec_context, obtained by compiling abi_probe.c against the
reference header rawspec.h (run in a checkout where the reference sources
are available; the fixture is committed so tests need no reference tree).

usage: python tests/golden/make_abi_fixture.py [/path/to/reference]
(default: the reference tree the recipe oracle/ref_build.py resolves)
"""
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(ref: str) -> None:
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "abi_probe"
        subprocess.run(["gcc", "-O0", f"-I{ref}", "-o", str(exe), str(HERE / "abi_probe.c")], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    (HERE / "abi_layout.json").write_text(out)
    print(out)


if __name__ == "__main__":
    sys.path.insert(0, str(HERE.parent.parent))
    from oracle import ref_build
    main(sys.argv[1] if len(sys.argv) > 1 else str(ref_build.REFERENCE))
