"""Host-side checks of the job server's interface (no GPU): the ctypes
mirror's structures have the C header's layout, and the server refuses to
start without a usable GPU instead of failing later."""
import ctypes as C
import json
import subprocess
from pathlib import Path

import pytest

from rawspec_gb300 import serve

ROOT = Path(__file__).resolve().parent.parent

PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "rawspec_gb300_serve.h"
#define F(T, m) printf("\"%s.%s\": %zu,", #T, #m, offsetof(T, m))
int main(void) {
  printf("{");
  F(rawspec_gb300_job_stats, state); F(rawspec_gb300_job_stats, buffers); F(rawspec_gb300_job_stats, dumps);
  F(rawspec_gb300_job_stats, t_submit); F(rawspec_gb300_job_stats, dump_p99_ms);
  F(rawspec_gb300_job_stats, device_bytes);
  F(rawspec_gb300_server_stats, failed); F(rawspec_gb300_server_stats, budget);
  F(rawspec_gb300_server_stats, peak_used); F(rawspec_gb300_server_stats, peak_active);
  F(rawspec_gb300_server_stats, buffers); F(rawspec_gb300_server_stats, dump_p99_ms);
  printf("\"job\": %zu, \"server\": %zu}\n", sizeof(rawspec_gb300_job_stats), sizeof(rawspec_gb300_server_stats));
  return 0;
}
"""


def test_stats_structures_match_the_header(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", "-o", str(exe), str(src)], check=True)
    c = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for key, off in c.items():
        if "." not in key:
            continue
        t, m = key.split(".")
        py = serve.JobStats if t == "rawspec_gb300_job_stats" else serve.ServerStats
        assert getattr(py, m).offset == off, key
    assert C.sizeof(serve.JobStats) == c["job"]
    assert C.sizeof(serve.ServerStats) == c["server"]


def test_server_needs_a_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    assert not serve.lib().rawspec_gb300_server_create(0, 1 << 30, 2, 2)
