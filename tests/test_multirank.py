"""Multi-GPU decomposition, tested on the host with two gloo ranks.

The spectrometer shards by coarse channel with no exchange: every channel's
products depend on that channel's voltages only, and the incoherent sum on
the antennas of one channel, which a rank keeps together.  Two ranks launched
by torch.distributed.run each process their share (the FP32 CPU chain stands
in for the GPU); their dumps, put side by side, must equal a single-process
run bit for bit.  The workers also run bench.py's rank coordination.
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
from rawspec_gb300 import synth  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _split(a: np.ndarray, np_out: int, nc: int, nt: int) -> np.ndarray:
    """[ndumps, Nd*|P|*Nc*Nt] -> [ndumps, Nd, |P|, Nc, Nt]."""
    nd = a.shape[1] // (np_out * nc * nt)
    return a.reshape(a.shape[0], nd, np_out, nc, nt)


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
    nca = W.NC // W.NANT
    covered = []
    for rank in range(2):
        got = np.load(tmp_path / f"rank{rank}.npz")
        chans = list(got["chans"])
        covered += chans
        for i, (nt, _, npo) in enumerate(W.PRODUCTS):
            full = _split(outs[i], abs(npo), W.NC, nt)[:, :, :, chans, :]
            part = _split(got[f"out{i}"], abs(npo), len(chans), nt)
            np.testing.assert_array_equal(part, full)
            cw = [c for c in chans if c < nca]  # channel-within-antenna indices of this rank
            full_ics = _split(icss[i], abs(npo), nca, nt)[:, :, :, cw, :]
            part_ics = _split(got[f"ics{i}"], abs(npo), len(cw), nt)
            np.testing.assert_array_equal(part_ics, full_ics)
    assert sorted(covered) == list(range(W.NC))


@pytest.mark.parametrize("world", [1, 2, 3])
def test_shards_cover_channels_once(world):
    seen = []
    for r in range(world):
        seen += W.shard_channels(r, world)
    assert sorted(seen) == list(range(W.NC))
