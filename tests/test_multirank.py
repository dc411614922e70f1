"""Multi-GPU decomposition, tested on the host with two gloo ranks.

The spectrometer shards by coarse channel with no exchange: every channel's
products depend on that channel's voltages only, and the incoherent sum on
the antennas of one channel, which a rank keeps together.  Two ranks launched
by torch.distributed.run each take their shard through the library's shard
API and process it (the FP32 CPU chain stands in for the GPU); their dumps,
put back with rawspec_gb300_shard_place_dump, must equal a single-process run
bit for bit.  The workers also run bench.py's rank coordination.
"""
from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))

import multirank_worker as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from rawspec_gb300 import api, synth  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_channel_shards_match_single_process(tmp_path):
    O.lib()  # build the oracle before the ranks load it
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
           str(Path(__file__).resolve().parent / "multirank_worker.py"), str(tmp_path)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]

    blocks = synth.gaussian_blocks(W.NB, W.NC, W.NTPB, W.NP, sigma=16.0, seed=7)
    cfg = O.make_cfg(W.NC, W.NP, W.NTPB, W.NB, 8, W.PRODUCTS, Nant=W.NANT, weights=W.WEIGHTS)
    outs, icss = O.run_cpu(cfg, blocks, nthreads=1)
    placed = [np.zeros_like(o) for o in outs]
    placed_ics = [np.zeros_like(s) for s in icss]
    covered = 0
    for rank in range(2):
        got = np.load(tmp_path / f"rank{rank}.npz")
        k0, nk = int(got["k0"]), int(got["nk"])
        covered += nk
        for i, (nt, _, npo) in enumerate(W.PRODUCTS):
            assert got[f"out{i}"].shape[0] == outs[i].shape[0]
            for d in range(outs[i].shape[0]):
                api.shard_place_dump(got[f"out{i}"][d], placed[i][d], W.NC, W.NANT, k0, nk, nt)
                api.shard_place_dump(got[f"ics{i}"][d], placed_ics[i][d], W.NC, W.NANT, k0, nk, nt, ics=True)
    assert covered == W.NC // W.NANT
    for i in range(len(W.PRODUCTS)):
        np.testing.assert_array_equal(placed[i], outs[i])
        np.testing.assert_array_equal(placed_ics[i], icss[i])
