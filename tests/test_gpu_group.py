"""Buffers of several contexts started together
(rawspec_gb300_start_processing_group): the small-FFT kernel launches that
share a configuration run as one grid, and every context's dumps are
identical, bit for bit, to those of the same buffers processed alone; through
the job server, jobs started together in the mix give the dumps they give
alone."""
import threading

import numpy as np
import pytest

from rawspec_gb300 import api, serve, synth

pytestmark = pytest.mark.gpu

# (Nc, Ntpb, nbits, products, conj, fft_dir): the 8-point total-power product
# is common to all four; two more share a 256-point full-pol product
CTXS = [
    (8, 1 << 16, 8, [(8, 128, 1), (1024, 16, 4)], 0, 1),
    (32, 1 << 15, 8, [(256, 32, 4), (8, 64, 1)], 1, 1),
    (16, 1 << 16, 4, [(8, 256, 1)], 0, -1),
    (4, 1 << 16, 8, [(256, 8, 4), (8, 512, 1), (4096, 4, -4)], 0, 1),
]
NBUF = 3


def blocks_for(k):
    Nc, Ntpb, nbits, _p, _c, _d = CTXS[k]
    if nbits == 4:
        return synth.int4_blocks(NBUF, Nc, Ntpb, 2, seed=80 + k)[0]
    return synth.gaussian_blocks(NBUF, Nc, Ntpb, 2, sigma=18.0, seed=80 + k)


def make(k):
    Nc, Ntpb, nbits, prods, conj, _d = CTXS[k]
    return api.Spectrometer(Nc, 2, Ntpb, nbits, prods, conj=conj)


def test_group_of_contexts_equals_each_alone(cuda_device):
    data = [blocks_for(k) for k in range(len(CTXS))]
    alone = []
    for k in range(len(CTXS)):
        with make(k) as sp:
            for b in range(NBUF):
                sp.wait()
                sp.load_blocks(data[k][b:b + 1])
                sp.copy_to_gpu()
                sp.start(CTXS[k][5])
            sp.wait()
            alone.append([[np.array(d) for d in p] for p in sp.dumps])
    specs = [make(k) for k in range(len(CTXS))]
    try:
        for b in range(NBUF):
            for k, sp in enumerate(specs):
                sp.wait()
                sp.load_blocks(data[k][b:b + 1])
                sp.copy_to_gpu()
            api.start_group(specs, [c[5] for c in CTXS])
        for sp in specs:
            assert sp.wait() == 0
        # the 8-point launch of every context and the 256-point launch of two
        # of them were shared, once per buffer
        for k, sp in enumerate(specs):
            assert sp.shared_launches() == NBUF * (2 if k in (1, 3) else 1), (k, sp.shared_launches())
            got = [[np.array(d) for d in p] for p in sp.dumps]
            assert [len(p) for p in got] == [len(p) for p in alone[k]]
            for p in range(len(got)):
                assert len(got[p]) > 0
                for a, w in zip(got[p], alone[k][p]):
                    assert np.array_equal(a, w), (k, p)
    finally:
        for sp in specs:
            sp.close()


def test_server_starts_ready_jobs_together(cuda_device):
    # two jobs of each shape, every one sharing the 8-point product
    kinds = list(range(len(CTXS))) * 2
    data = [blocks_for(k) for k in range(len(CTXS))]
    alone = []
    for k in range(len(CTXS)):
        with make(k) as sp:
            sp.process(data[k], fft_dir=CTXS[k][5], combined=True)
            alone.append([[np.array(d) for d in p] for p in sp.dumps])
    with serve.Server(budget_bytes=8 << 30, max_active=len(kinds), max_queued=NBUF) as srv:
        jobs = [srv.submit(CTXS[k][0], 2, CTXS[k][1], CTXS[k][2], CTXS[k][3], conj=CTXS[k][4], fft_dir=CTXS[k][5])
                for k in kinds]
        feeders = [threading.Thread(target=lambda j=j, k=k: [srv.push(j, data[k][b:b + 1]) for b in range(NBUF)])
                   for j, k in zip(jobs, kinds)]
        for t in feeders:
            t.start()
        for t in feeders:
            t.join()
        for j in jobs:
            srv.close_job(j)
        for j in jobs:
            assert srv.wait_job(j, 120.0) == serve.JOB_DONE
        st = srv.stats()
        assert st.failed == 0
        print(f"group calls {st.group_calls}")
        assert st.group_calls > 0
        for j, k in zip(jobs, kinds):
            for p in range(len(alone[k])):
                assert len(srv.dumps[j][p]) == len(alone[k][p]) > 0, (k, p)
                for a, w in zip(srv.dumps[j][p], alone[k][p]):
                    assert np.array_equal(a, w), (k, p)
