"""A client of the reference interface compiles and links against this
library unchanged: the reference's own rawspectest.c (when the reference
sources are available on this machine; the binary is not run here)."""
import os
import subprocess
from pathlib import Path

import pytest

from oracle import ref_build

ROOT = Path(__file__).resolve().parent.parent
REF = ref_build.REFERENCE  # where the reference tree lies (the recipe under oracle/ resolves it)
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
CUDA_LIB = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "lib64"


@pytest.mark.skipif(not (REF / "rawspectest.c").exists(), reason="reference sources not available")
def test_reference_rawspectest_links(tmp_path):
    exe = tmp_path / "rawspectest"
    cmd = ["gcc", "-O2", f"-I{ROOT / 'include'}", f"-I{CUDA_INC}", "-o", str(exe), str(REF / "rawspectest.c"),
           f"-L{ROOT / 'rawspec_gb300' / 'lib'}", "-lrawspec", f"-Wl,-rpath,{ROOT / 'rawspec_gb300' / 'lib'}",
           f"-L{CUDA_LIB}", "-lcudart"]  # rawspectest.c itself calls the CUDA runtime
    subprocess.run(cmd, check=True, capture_output=True)
    assert exe.exists()
    undefined = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True, check=True).stdout
    for fn in ["rawspec_initialize", "rawspec_copy_blocks_to_gpu", "rawspec_start_processing",
               "rawspec_wait_for_completion", "rawspec_cleanup"]:
        assert fn in undefined
