"""Channel shards of one observation on the GPU: each shard runs as its own
context (rawspec_gb300_shard_context) on its channels (filled with
rawspec_gb300_shard_fill_block), one after another on one GPU as separate
GPUs would run them; their dumps and incoherent sums, put back with
rawspec_gb300_shard_place_dump, equal the whole observation's context within
the parity tolerance (the kernels' partial-sum splits depend on the channel
count, so the summation order may differ)."""
import numpy as np
import pytest

from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_shards_equal_the_whole_observation(cuda_device, world):
    nc, nant, ntpb, nblk = 12, 2, 65536, 4
    prods = [(1024, 8, 1), (65536, 1, -4), (16, 64, 4)]
    w = [0.75, 1.25]
    blocks = synth.gaussian_blocks(nblk, nc, ntpb, 2, sigma=18.0, seed=77)
    with api.Spectrometer(nc, 2, ntpb, 8, prods, Nant=nant, weights=w) as full:
        full.process(blocks)
        want = [np.array(d) for d in full.dumps]
        want_ics = [np.array(s) for s in full.ics]
    placed = [np.zeros_like(x) for x in want]
    placed_ics = [np.zeros_like(x) for x in want_ics]
    for r in range(world):
        with api.Spectrometer(nc, 2, ntpb, 8, prods, Nant=nant, weights=w, shard=(r, world)) as sh:
            assert sh.ctx.Nc == nant * sh.nk
            mine = np.stack([api.shard_fill_block(b, nc, nant, sh.k0, sh.nk) for b in blocks])
            sh.process(mine)
            for i, (nt, _na, _p) in enumerate(prods):
                assert len(sh.dumps[i]) == want[i].shape[0]
                for d, dump in enumerate(sh.dumps[i]):
                    api.shard_place_dump(dump, placed[i][d], nc, nant, sh.k0, sh.nk, nt)
                    api.shard_place_dump(sh.ics[i][d], placed_ics[i][d], nc, nant, sh.k0, sh.nk, nt, ics=True)
    for i, (nt, _na, npol) in enumerate(prods):
        assert normalized_error(placed[i], want[i], npol, nc, nt) < REL_TOL
        assert normalized_error(placed_ics[i], want_ics[i], npol, nc // nant, nt) < REL_TOL
