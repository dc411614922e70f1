"""The production configuration compared bin by bin at its real shape.

64 channels x 2 polarisations of 8-bit complex Gaussian voltages (sigma 20),
Ntpb 524288 (128 MiB blocks, two-block 256 MiB buffers), three products
Nfft 2^20 / 8 / 1024 with Nint 51 / 128 / 3072, total power and full pol.
102 blocks (51 buffers) are streamed, so that the 2^20-point product, one
spectrum per buffer integrated over 51 buffers, dumps once; the 1024-point
product (Nint 3072 over three buffers) dumps 17 times, the 8-point one every
buffer.  The input is drawn on the GPU per buffer (synth.gaussian_buffer_cuda)
so that every process generates the same bytes without holding 13 GiB.

Checks:
  * every bin of every channel against the reference's own GPU library
    (rawspec_gpu.cu with cuFFT callbacks, run in a child process), when its
    sources are present;
  * channels 0 and 63 against the FP64 oracle (run on those two channels
    only; a channel's spectra depend on that channel alone).  The oracle is
    run in full-pol mode: total power is XX + YY."""
import concurrent.futures as cf

import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref_build, ref_gpu
from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error, rms_normalized_error

pytestmark = pytest.mark.gpu

NC, NP, NTPB, NB = 64, 2, 524288, 2
NBUF = 51
PRODUCTS = [(1 << 20, 51), (8, 128), (1024, 3072)]
SEED, SIGMA = 20, 20.0
KEEP8 = [0, 1, 25, 50]  # dumps of the 8-point product compared (it dumps every buffer)
CHANS = [0, 63]


def _products(npol):
    return [(nt, na, npol) for nt, na in PRODUCTS]


def _oracle_channel(chan_blocks, npol):
    cfg = O.make_cfg(1, NP, NTPB, NB, 8, _products(npol))
    return O.run_oracle(cfg, chan_blocks)[0]


@pytest.fixture(scope="module")
def production_runs(cuda_device):
    """Streams the 51 buffers through two native contexts (Npolout 1 and 4);
    meanwhile the FP64 oracle runs on channels 0 and 63 in two threads and the
    reference library (if present) in a child process."""
    ref_lib = ref_build.build_gpu()
    pool = cf.ThreadPoolExecutor(max_workers=3)
    ref_future = None
    if ref_lib is not None:
        jobs = []
        for npol in (1, 4):
            jobs.append((dict(Nc=NC, Np=NP, Ntpb=NTPB, nbits=8, products=[list(p) for p in _products(npol)],
                              fft_dir=1, generate=dict(nbuf=NBUF, sigma=SIGMA, seed=SEED), keep={1: KEEP8}), None))
        ref_future = pool.submit(ref_gpu.run_in_child, jobs, 1800)
    ours = {}
    chan = np.empty((len(CHANS), NBUF * NB, NTPB * NP * 2), dtype=np.uint8)
    specs = {npol: api.Spectrometer(NC, NP, NTPB, 8, _products(npol)) for npol in (1, 4)}
    try:
        for k in range(NBUF):
            buf = synth.gaussian_buffer_cuda(k, NB, NC, NTPB, NP, sigma=SIGMA, seed=SEED)
            for j, c in enumerate(CHANS):
                chan[j, k * NB:(k + 1) * NB] = buf.reshape(NB, NC, -1)[:, c]
            for spec in specs.values():
                spec.process(buf)
        for npol, spec in specs.items():
            d = [np.array(x) for x in spec.dumps]
            d[1] = d[1][KEEP8]
            ours[npol] = d
            assert [len(x) for x in spec.dumps] == [1, NBUF, NBUF // 3], [len(x) for x in spec.dumps]
    finally:
        for spec in specs.values():
            spec.close()
    oracle_futures = [pool.submit(_oracle_channel, chan[j], 4) for j in range(len(CHANS))]
    orc = [f.result() for f in oracle_futures]
    ref = ref_future.result() if ref_future is not None else None
    pool.shutdown()
    return ours, orc, ref


def _channels(arr, npol, nt, chans):
    """[ndumps, Nd*|P|*Nc*Nt] -> the given channels, same layout with Nc = len(chans)."""
    a = arr.reshape(arr.shape[0], -1, abs(npol), NC, nt)[:, :, :, chans]
    return a.reshape(arr.shape[0], -1)


@pytest.mark.parametrize("npol", [1, 4])
def test_production_shape_channels_match_fp64_oracle(production_runs, npol):
    ours, orc, _ = production_runs
    for i, (nt, _na) in enumerate(PRODUCTS):
        # oracle: [ndumps, Nd*4*1*Nt] per channel, full pol
        per_chan = [o[i].reshape(o[i].shape[0], -1, 4, 1, nt) for o in orc]
        full = np.concatenate(per_chan, axis=3)  # [ndumps, Nd, 4, 2, Nt]
        if i == 1:
            full = full[KEEP8]
        if npol == 1:
            full = full[:, :, 0:1] + full[:, :, 1:2]
        ref = full.reshape(full.shape[0], -1)
        got = _channels(ours[npol][i], npol, nt, CHANS)
        assert got.shape == ref.shape, (i, got.shape, ref.shape)
        err = normalized_error(got, ref, npol, len(CHANS), nt)
        rms = rms_normalized_error(got, ref, npol, len(CHANS), nt)
        print(f"Nfft {nt} Npolout {npol}, channels {CHANS} vs FP64 oracle: max {err:.2e} rms {rms:.2e}")
        assert err < REL_TOL, (nt, npol, err)


@pytest.mark.parametrize("npol", [1, 4])
def test_production_shape_every_channel_matches_reference(production_runs, npol):
    ours, _, ref = production_runs
    if ref is None:
        pytest.skip("the reference's GPU sources are not present")
    r = ref[0 if npol == 1 else 1]
    for i, (nt, _na) in enumerate(PRODUCTS):
        got, exp = ours[npol][i], r[f"out{i}"]
        assert got.shape == exp.shape, (i, got.shape, exp.shape)
        err = normalized_error(got, exp, npol, NC, nt)
        rms = rms_normalized_error(got, exp, npol, NC, nt)
        print(f"Nfft {nt} Npolout {npol}, all 64 channels vs reference cuFFT build: max {err:.2e} rms {rms:.2e}")
        assert err < REL_TOL, (nt, npol, err)
