"""The job server (include/rawspec_gb300_serve.h) on the GPU: admission under
the device-memory budget, jobs of different shapes processed concurrently,
and each job's dumps identical to those of the same buffers streamed through
a context alone."""
import ctypes as C
import threading

import numpy as np
import pytest

from rawspec_gb300 import api, serve, synth

pytestmark = pytest.mark.gpu

# (Nc, Np, Ntpb, nbits, products, Nant, weights, conj, fft_dir, buffers)
JOBS = [
    (8, 2, 1 << 16, 8, [(1024, 16, 1), (8, 64, 4)], 1, None, 0, 1, 4),
    (8, 2, 1 << 16, 4, [(4096, 4, -4)], 2, [0.75, 1.25], 1, 1, 3),
    (2, 2, 1 << 17, 8, [(1 << 16, 1, 1)], 1, None, 0, 1, 3),
    (16, 2, 1 << 15, 8, [(256, 32, -4), (1024, 64, 4)], 1, None, 1, -1, 4),
]


def job_blocks(k):
    Nc, Np, Ntpb, nbits, prods, Nant, w, conj, fft_dir, nbuf = JOBS[k]
    spec = api.Spectrometer(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w, conj=conj, collect=False)
    nb = spec.Nb
    spec.close()
    if nbits == 4:
        blocks, _ = synth.int4_blocks(nb * nbuf, Nc, Ntpb, Np, Nant=Nant, seed=60 + k)
    else:
        blocks = synth.gaussian_blocks(nb * nbuf, Nc, Ntpb, Np, sigma=18.0, seed=60 + k)
    return nb, blocks


def run_alone(k, blocks):
    Nc, Np, Ntpb, nbits, prods, Nant, w, conj, fft_dir, nbuf = JOBS[k]
    spec = api.Spectrometer(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w, conj=conj)
    try:
        spec.process(blocks, fft_dir=fft_dir, combined=True)
        return [[np.array(d) for d in p] for p in spec.dumps], [[np.array(s) for s in p] for p in spec.ics]
    finally:
        spec.close()


def submit(srv, k):
    Nc, Np, Ntpb, nbits, prods, Nant, w, conj, fft_dir, nbuf = JOBS[k]
    return srv.submit(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w, conj=conj, fft_dir=fft_dir)


def feed(srv, job, nb, blocks):
    for b0 in range(0, blocks.shape[0], nb):
        srv.push(job, blocks[b0:b0 + nb])
    srv.close_job(job)


def test_device_bytes_estimate_equals_the_allocation(cuda_device):
    cases = [(64, 2, 1 << 19, 8, [(1 << 20, 51, 1), (8, 128, 1), (1024, 3072, 1)], 1, None),
             (64, 2, 1 << 19, 8, [(1 << 20, 51, 4), (8, 128, 4), (1024, 3072, 4)], 1, None),
             (16, 2, 1 << 18, 4, [(4096, 64, -4), (64, 1024, -4)], 4, [1.0, 0.5, 1.5, 1.0]),
             (4, 1, 1 << 16, 16, [(1 << 17, 1, 1), (512, 8, 1)], 1, None),
             # integrations of >= 3072 spectra over many buffers: staging and compensation planes
             (2, 2, 1 << 16, 8, [(1 << 16, 4096, 1), (256, 3072, 4)], 1, None)]
    for Nc, Np, Ntpb, nbits, prods, Nant, w in cases:
        ctx = api.make_context(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w)
        est = serve.device_bytes_estimate(ctx)
        spec = api.Spectrometer(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w, collect=False)
        try:
            got = spec.lib.rawspec_gb300_device_bytes(C.byref(spec.ctx))
        finally:
            spec.close()
        assert est == got, (prods, est, got)


def test_jobs_alone_and_in_the_mix_give_identical_dumps(cuda_device):
    data = [job_blocks(k) for k in range(len(JOBS))]
    alone = [run_alone(k, data[k][1]) for k in range(len(JOBS))]
    with serve.Server(budget_bytes=8 << 30, max_active=8, max_queued=2) as srv:
        jobs = [submit(srv, k) for k in range(len(JOBS))]
        feeders = [threading.Thread(target=feed, args=(srv, jobs[k], *data[k])) for k in range(len(JOBS))]
        for t in feeders:
            t.start()
        for t in feeders:
            t.join()
        for j in jobs:
            assert srv.wait_job(j, 120.0) == serve.JOB_DONE
        st = srv.stats()
        assert st.done == len(JOBS) and st.failed == 0
        assert st.peak_active >= 2          # the jobs overlapped on the device
        for k, j in enumerate(jobs):
            want_d, want_s = alone[k]
            assert len(srv.dumps[j]) == len(want_d)
            for p in range(len(want_d)):
                assert len(srv.dumps[j][p]) == len(want_d[p]) > 0, (k, p)
                for a, b in zip(srv.dumps[j][p], want_d[p]):
                    assert np.array_equal(a, b), (k, p)
                for a, b in zip(srv.ics[j][p], want_s[p]):
                    assert np.array_equal(a, b), (k, p, "ics")
            js = srv.job_stats(j)
            assert js.buffers == JOBS[k][-1]
            assert js.dumps == sum(len(x) for x in want_d)
            assert 0 < js.buffer_p50_ms <= js.buffer_p99_ms
            assert 0 < js.dump_p50_ms <= js.dump_p99_ms


def test_admission_keeps_within_the_memory_budget(cuda_device):
    # a budget that holds one of these jobs at a time: the others wait as
    # pending and are admitted as memory is released; results unchanged
    data = [job_blocks(k) for k in (0, 3)]
    ests = []
    for k in (0, 3):
        Nc, Np, Ntpb, nbits, prods, Nant, w, conj, fft_dir, nbuf = JOBS[k]
        ests.append(serve.device_bytes_estimate(api.make_context(Nc, Np, Ntpb, nbits, prods, Nant=Nant, weights=w)))
    budget = sum(ests) - 1  # either job fits, both do not
    alone = [run_alone(k, data[i][1]) for i, k in enumerate((0, 3))]
    with serve.Server(budget_bytes=budget, max_active=4, max_queued=1) as srv:
        jobs = [submit(srv, k) for k in (0, 3, 0)]
        feeders = [threading.Thread(target=feed, args=(srv, jobs[i], *data[i % 2])) for i in range(3)]
        for t in feeders:
            t.start()
        for t in feeders:
            t.join()
        for j in jobs:
            assert srv.wait_job(j, 120.0) == serve.JOB_DONE
        st = srv.stats()
        assert st.peak_used <= budget and st.peak_active == 1 and st.used == 0
        for i, j in enumerate(jobs):
            for p, want in enumerate(alone[i % 2][0]):
                assert all(np.array_equal(a, b) for a, b in zip(srv.dumps[j][p], want))
        # admitted one after another, in submission order
        t = [srv.job_stats(j) for j in jobs]
        assert t[0].t_done <= t[1].t_admit and t[1].t_done <= t[2].t_admit


def test_job_larger_than_the_budget_is_rejected(cuda_device):
    with serve.Server(budget_bytes=1 << 20) as srv:
        with pytest.raises(ValueError):
            submit(srv, 0)


def test_server_refuses_bad_requests(cuda_device):
    import ctypes as Cc
    with serve.Server(budget_bytes=1 << 30, max_active=2, max_queued=1) as srv:
        job = submit(srv, 3)
        nb, blocks = job_blocks(3)
        with pytest.raises(RuntimeError):          # wrong buffer size
            srv.push(job, blocks[:nb, :-16])
        with pytest.raises(RuntimeError):          # unknown job
            srv.push(job + 100, blocks[:nb])
        assert srv.wait_job(job + 100, 0.1) == -1
        with pytest.raises(KeyError):
            srv.job_stats(job + 100)
        srv.push(job, blocks[:nb])
        srv.close_job(job)
        with pytest.raises(RuntimeError):          # closed job
            srv.push(job, blocks[:nb])
        assert srv.wait_job(job, 60.0) == serve.JOB_DONE
        st = srv.job_stats(job)
        assert st.buffers == 1 and st.state == serve.JOB_DONE and st.device_bytes > 0
        assert srv.stats().used == 0
        # an invalid configuration is refused at submission
        bad = api.make_context(16, 2, 1 << 15, 8, [(1000, 3, 1)])
        assert serve.lib().rawspec_gb300_server_submit(srv.h, Cc.byref(bad), 1, srv._cb, None) == -1
