"""One rank of the multi-process CPU test of the multi-GPU decomposition
(launched by tests/test_multirank.py under torch.distributed.run, gloo).

Each rank takes its shard of the coarse channels through the library's shard
API (rawspec_gb300_shard_range and rawspec_gb300_shard_fill_block: host code,
no GPU needed), runs the FP32 CPU chain on them in place of the GPU and saves
its dumps; it also exercises the host-side coordination that bench.py uses
for N > 1 (barrier, max over ranks, whole-job throughput).
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from oracle import oracle as O  # noqa: E402
from rawspec_gb300 import api, synth  # noqa: E402

NC, NP, NTPB, NB, NANT = 8, 2, 4096, 2, 2
PRODUCTS = [(1024, 4, 1), (16, 64, 4)]
WEIGHTS = [0.75, 1.25]


def main() -> int:
    out_dir = Path(sys.argv[1])
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    group = bench.RankGroup(world)
    group.barrier()
    m = group.max_over_ranks(float(rank) + 1.5)
    assert m == world + 0.5, m
    gbs = bench.whole_job_gbs(world, 1 << 30, 4, group.max_over_ranks(2.0 + rank))
    assert abs(gbs - world * 4 * (1 << 30) / (2.0 + world - 1) / 1e9) < 1e-9

    blocks = synth.gaussian_blocks(NB, NC, NTPB, NP, sigma=16.0, seed=7)
    k0, nk = api.shard_range(NC, NANT, rank, world)
    mine = np.stack([api.shard_fill_block(b, NC, NANT, k0, nk) for b in blocks])
    cfg = O.make_cfg(NANT * nk, NP, NTPB, NB, 8, PRODUCTS, Nant=NANT, weights=WEIGHTS)
    outs, icss = O.run_cpu(cfg, mine, nthreads=1)
    np.savez(out_dir / f"rank{rank}.npz", k0=k0, nk=nk,
             **{f"out{i}": o for i, o in enumerate(outs)}, **{f"ics{i}": s for i, s in enumerate(icss)})
    group.barrier()
    group.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
