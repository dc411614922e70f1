"""Channel shards of one observation (include/rawspec_gb300.h, shard.c),
checked on the CPU: the ranges cover every channel once with all antennas of
a channel together, the block and dump helpers move exactly the shard's
channels, and shards processed separately by the FP32 CPU chain and put back
with the library's helpers equal the whole observation bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from rawspec_gb300 import api, synth


@pytest.mark.parametrize("nc,nant,world", [(64, 1, 1), (64, 1, 8), (64, 4, 3), (12, 3, 4), (7, 1, 7)])
def test_ranges_cover_every_channel_once(nc, nant, world):
    nca = nc // nant
    seen = []
    sizes = []
    for r in range(world):
        k0, nk = api.shard_range(nc, nant, r, world)
        sizes.append(nk)
        seen += [a * nca + k for a in range(nant) for k in range(k0, k0 + nk)]
    assert sorted(seen) == list(range(nc))
    assert max(sizes) - min(sizes) <= 1


def test_invalid_shards_are_refused():
    for args in [(8, 3, 0, 1), (8, 1, 2, 2), (8, 1, -1, 2), (4, 1, 0, 5), (0, 1, 0, 1)]:
        with pytest.raises(ValueError):
            api.shard_range(*args)


def test_fill_block_and_place_dump_move_the_shard_channels():
    nc, nant, cb, nt, rows = 12, 3, 40, 8, 5
    block = np.arange(nc * cb, dtype=np.uint32).astype(np.uint8)
    k0, nk = api.shard_range(nc, nant, 1, 2)
    got = api.shard_fill_block(block, nc, nant, k0, nk)
    want = block.reshape(nant, nc // nant, cb)[:, k0:k0 + nk].reshape(-1)
    np.testing.assert_array_equal(got, want)
    # dumps: [rows][Nc][Nt] and incoherent sums [rows][Nc/Nant][Nt]
    full = np.zeros(rows * nc * nt, np.float32)
    shard = np.random.default_rng(1).standard_normal(rows * nant * nk * nt).astype(np.float32)
    api.shard_place_dump(shard, full, nc, nant, k0, nk, nt)
    f = full.reshape(rows, nant, nc // nant, nt)
    np.testing.assert_array_equal(f[:, :, k0:k0 + nk], shard.reshape(rows, nant, nk, nt))
    assert not f[:, :, :k0].any() and not f[:, :, k0 + nk:].any()
    ics_full = np.zeros(rows * (nc // nant) * nt, np.float32)
    ics = shard[: rows * nk * nt]
    api.shard_place_dump(ics, ics_full, nc, nant, k0, nk, nt, ics=True)
    np.testing.assert_array_equal(ics_full.reshape(rows, nc // nant, nt)[:, k0:k0 + nk], ics.reshape(rows, nk, nt))


def test_shards_through_the_cpu_chain_equal_the_whole_observation():
    nc, nant, ntpb, nb, world = 12, 3, 2048, 2, 3
    prods = [(512, 4, -4), (16, 32, 1)]
    w = [0.5, 1.0, 1.5]
    blocks = synth.gaussian_blocks(nb, nc, ntpb, 2, sigma=16.0, seed=9)
    outs, icss = O.run_cpu(O.make_cfg(nc, 2, ntpb, nb, 8, prods, Nant=nant, weights=w), blocks, nthreads=1)
    placed = [np.zeros_like(o) for o in outs]
    placed_ics = [np.zeros_like(s) for s in icss]
    for r in range(world):
        k0, nk = api.shard_range(nc, nant, r, world)
        mine = np.stack([api.shard_fill_block(b, nc, nant, k0, nk) for b in blocks])
        so, si = O.run_cpu(O.make_cfg(nant * nk, 2, ntpb, nb, 8, prods, Nant=nant, weights=w), mine, nthreads=1)
        for i, (nt, _na, _p) in enumerate(prods):
            for d in range(so[i].shape[0]):
                api.shard_place_dump(so[i][d], placed[i][d], nc, nant, k0, nk, nt)
                api.shard_place_dump(si[i][d], placed_ics[i][d], nc, nant, k0, nk, nt, ics=True)
    for i in range(len(prods)):
        np.testing.assert_array_equal(placed[i], outs[i])
        np.testing.assert_array_equal(placed_ics[i], icss[i])
