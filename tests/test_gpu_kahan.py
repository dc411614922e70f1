"""Compensated (Kahan) integration across buffers, against the FP64 oracle.

Products that integrate at least 3072 spectra over several buffers fold each
buffer's FP32 sums into the running sum with a compensation plane
(k_kahan_merge).  The tests integrate thousands of buffers, where a plain FP32
running sum drifts, and compare the compensated and the plain result
(RAWSPEC_GB300_KAHAN=0) with the oracle; the forced cases run the staging
path of every kernel family on short integrations."""
import numpy as np
import pytest

from cases import derived_nb
from oracle import oracle as O
from rawspec_gb300 import api, synth
from util import REL_TOL, normalized_error, rms_normalized_error

pytestmark = pytest.mark.gpu
MERGE = api.KERNEL_CLASS_NAMES.index("merge")


def run(c, blocks, monkeypatch, kahan):
    if kahan is None:
        monkeypatch.delenv("RAWSPEC_GB300_KAHAN", raising=False)
    else:
        monkeypatch.setenv("RAWSPEC_GB300_KAHAN", kahan)
    spec = api.Spectrometer(c["Nc"], c["Np"], c["Ntpb"], 8, c["products"])
    try:
        spec.set_profiling(True)
        spec.process(blocks)
        return [np.array(d) for d in spec.dumps], spec.profile(MERGE)[1]
    finally:
        spec.close()


def oracle(c, blocks):
    cfg = O.make_cfg(c["Nc"], c["Np"], c["Ntpb"], derived_nb(c), 8, c["products"])
    return O.run_oracle(cfg, blocks)[0]


# (name, Nc, Np, Ntpb, Nt, Na): one dump after Na / (spectra per buffer) buffers
LONG = [("k_small 256", 2, 2, 256, 256, 4096),            # 4096 buffers of one spectrum
        ("k_tc 1024", 2, 2, 2048, 1024, 4096),            # 2048 buffers of two spectra
        ("k_large_a/b 8192", 1, 1, 8192, 8192, 3072)]     # 3072 buffers, one polarisation


@pytest.mark.parametrize("name,Nc,Np,Ntpb,nt,na", LONG, ids=[x[0] for x in LONG])
def test_long_integration_is_compensated(cuda_device, monkeypatch, name, Nc, Np, Ntpb, nt, na):
    c = dict(Nc=Nc, Np=Np, Ntpb=Ntpb, products=[(nt, na, 1)])
    nbuf = na * nt // Ntpb
    blocks = synth.gaussian_blocks(nbuf, Nc, Ntpb, Np, sigma=20.0, seed=700 + nt)
    ref = oracle(c, blocks)[0]
    got_k, merges = run(c, blocks, monkeypatch, None)
    got_p, merges_p = run(c, blocks, monkeypatch, "0")
    assert merges == nbuf - 1 and merges_p == 0
    assert got_k[0].shape == ref.shape == got_p[0].shape
    ek, ep = normalized_error(got_k[0], ref, 1, Nc, nt), normalized_error(got_p[0], ref, 1, Nc, nt)
    rk, rp = rms_normalized_error(got_k[0], ref, 1, Nc, nt), rms_normalized_error(got_p[0], ref, 1, Nc, nt)
    print(f"{name}: {nbuf} buffers, max / rms relative error compensated {ek:.2e} / {rk:.2e}, "
          f"plain {ep:.2e} / {rp:.2e}")
    # measured: compensated 1.8e-7 .. 5.8e-7 (the rest is the per-buffer FFT
    # error), plain 3.0e-6 .. 4.2e-6 over these 2048 .. 4096 buffers
    assert ek < 1e-6
    assert ek <= ep and rk <= rp


FORCED = [("fused TP", 1, 2, 1 << 16, 1 << 16, 8, 1),      # output tensor map of the staging plane
          ("fused full pol", 1, 2, 1 << 16, 1 << 16, 8, 4),
          ("k_small Stokes", 3, 2, 4096, 512, 64, -4),      # chunked units: finalize into the staging plane
          ("k_tc 4096", 2, 2, 8192, 4096, 12, 1)]


@pytest.mark.parametrize("name,Nc,Np,Ntpb,nt,na,npol", FORCED, ids=[x[0] for x in FORCED])
def test_forced_compensation_matches_the_oracle(cuda_device, monkeypatch, name, Nc, Np, Ntpb, nt, na, npol):
    c = dict(Nc=Nc, Np=Np, Ntpb=Ntpb, products=[(nt, na, npol)])
    nss = max(1, Ntpb // nt)
    nbuf = 2 * na // nss  # two integrations
    blocks = synth.gaussian_blocks(nbuf, Nc, Ntpb, Np, sigma=20.0, seed=800 + nt)
    ref = oracle(c, blocks)[0]
    got_k, merges = run(c, blocks, monkeypatch, "1")
    got_p, _ = run(c, blocks, monkeypatch, "0")
    assert merges == nbuf - 2            # every buffer but the first of each integration
    assert got_k[0].shape == ref.shape
    assert normalized_error(got_k[0], ref, npol, Nc, nt) < REL_TOL
    # a handful of buffers: the compensated and the plain sum differ by rounding only
    assert normalized_error(got_k[0], got_p[0].astype(np.float64), npol, Nc, nt) < 1e-6
